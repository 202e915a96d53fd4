// anl_capi.cu -- the extern "C" entry points declared in include/anneal_gb300.h, the
// context life cycle and the host-side element matrix.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "anl_ctx.cuh"

namespace anl {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

std::recursive_mutex& device_sync_mutex() {
    static std::recursive_mutex m;
    return m;
}

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

// ------------------------------------------------------------------ element matrix (host, FP64)

static const int LOCAL[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

// hex8_matrices (fem.py:71-84): Ke = sum over the 2x2x2 Gauss points of B^T D B |J|, with
// D the isotropic E = 1 constitutive matrix in Voigt order xx yy zz xy yz zx
// (fem.py:36-43) and B the strain-displacement matrix of the trilinear brick (fem.py:46-68).
void hex8_ke(double nu, double h, double* ke) {
    const double c = 1.0 / ((1 + nu) * (1 - 2 * nu));
    double D[6][6] = {};
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) D[a][b] = nu * c;
    for (int a = 0; a < 3; ++a) D[a][a] = (1 - nu) * c;
    for (int a = 3; a < 6; ++a) D[a][a] = 0.5 * (1 - 2 * nu) * c;
    std::memset(ke, 0, sizeof(double) * 576);
    const double g = 1.0 / std::sqrt(3.0), jac = 0.5 * h, w = jac * jac * jac;
    for (int q = 0; q < 8; ++q) {
        const double xi = (q & 4) ? g : -g, eta = (q & 2) ? g : -g, zeta = (q & 1) ? g : -g;
        double B[6][24] = {};
        for (int a = 0; a < 8; ++a) {
            const double s0 = 2 * LOCAL[a][0] - 1, s1 = 2 * LOCAL[a][1] - 1, s2 = 2 * LOCAL[a][2] - 1;
            const double dx = s0 * (1 + s1 * eta) * (1 + s2 * zeta) / 8 / jac;
            const double dy = s1 * (1 + s0 * xi) * (1 + s2 * zeta) / 8 / jac;
            const double dz = s2 * (1 + s0 * xi) * (1 + s1 * eta) / 8 / jac;
            B[0][3 * a] = dx;
            B[1][3 * a + 1] = dy;
            B[2][3 * a + 2] = dz;
            B[3][3 * a] = dy;
            B[3][3 * a + 1] = dx;
            B[4][3 * a + 1] = dz;
            B[4][3 * a + 2] = dy;
            B[5][3 * a] = dz;
            B[5][3 * a + 2] = dx;
        }
        double DB[6][24];
        for (int r = 0; r < 6; ++r)
            for (int col = 0; col < 24; ++col) {
                double s = 0;
                for (int k = 0; k < 6; ++k) s += D[r][k] * B[k][col];
                DB[r][col] = s;
            }
        for (int r = 0; r < 24; ++r)
            for (int col = 0; col < 24; ++col) {
                double s = 0;
                for (int k = 0; k < 6; ++k) s += B[k][r] * DB[k][col];
                ke[r * 24 + col] += s * w;
            }
    }
}

static int local_index(int x, int y, int z) {
    for (int a = 0; a < 8; ++a)
        if (LOCAL[a][0] == x && LOCAL[a][1] == y && LOCAL[a][2] == z) return a;
    return -1;
}

double ke_blocks(const double* ke, KeBlocks<double>* out) {
    for (int dl = 0; dl < 8; ++dl) {
        const int b = local_index(dl & 1, (dl >> 1) & 1, (dl >> 2) & 1);
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) out->blk[dl][3 * r + q] = ke[r * 24 + 3 * b + q];
    }
    double dev = 0.0;
    for (int a = 0; a < 8; ++a) {
        for (int b = 0; b < 8; ++b) {
            const int dx = std::abs(LOCAL[b][0] - LOCAL[a][0]), dy = std::abs(LOCAL[b][1] - LOCAL[a][1]),
                      dz = std::abs(LOCAL[b][2] - LOCAL[a][2]);
            const int dl = dx + 2 * dy + 4 * dz;
            for (int r = 0; r < 3; ++r)
                for (int q = 0; q < 3; ++q) {
                    const double sr = 1 - 2 * LOCAL[a][r], sq = 1 - 2 * LOCAL[a][q];
                    const double want = sr * sq * out->blk[dl][3 * r + q];
                    dev = std::max(dev, std::fabs(want - ke[(3 * a + r) * 24 + 3 * b + q]));
                }
        }
    }
    return dev;
}

double ke_modal(const double* ke, KeModal<double>* out) {
    // KA = T^T Ke T with T[3a+c][3m+c] = s_m(p_a), modes 1, sx, sy, sz, sx sy, sy sz, sz sx, sx sy sz
    double S[8][8];
    for (int a = 0; a < 8; ++a) {
        const double sx = 2 * LOCAL[a][0] - 1, sy = 2 * LOCAL[a][1] - 1, sz = 2 * LOCAL[a][2] - 1;
        const double m[8] = {1, sx, sy, sz, sx * sy, sy * sz, sz * sx, sx * sy * sz};
        for (int q = 0; q < 8; ++q) S[a][q] = m[q];
    }
    auto ka = [&](int m, int c, int n, int e) {  // KA[(m,c),(n,e)] / 64
        double s = 0;
        for (int a = 0; a < 8; ++a)
            for (int b = 0; b < 8; ++b) s += S[a][m] * ke[(3 * a + c) * 24 + 3 * b + e] * S[b][n];
        return s / 64.0;
    };
    const double A = ka(1, 0, 1, 0), B = ka(1, 0, 2, 1), C = ka(1, 1, 1, 1), D = ka(4, 0, 4, 0),
                 F = ka(4, 0, 5, 2), G = ka(4, 2, 4, 2), H = ka(4, 2, 5, 0), J = ka(7, 0, 7, 0);
    *out = KeModal<double>{A - B, B, C, D, F, G - H, H, J};
    // rebuild Ke column by column through modal_element and compare
    double kmax = 0.0, dev = 0.0;
    for (int t = 0; t < 576; ++t) kmax = std::max(kmax, std::fabs(ke[t]));
    for (int col = 0; col < 24; ++col) {
        double u[2][2][2][3] = {};
        const int bn = col / 3;
        u[LOCAL[bn][0]][LOCAL[bn][1]][LOCAL[bn][2]][col % 3] = 1.0;
        auto v3 = [&](int px, int py, int pz) {
            V3<double> v;
            v.xy.x = u[px][py][pz][0];
            v.xy.y = u[px][py][pz][1];
            v.z = u[px][py][pz][2];
            return v;
        };
        V3<double> dxb[2], dxt[2], dyb[2], dyt[2], dz[2][2], f[2][2][2];
        for (int q = 0; q < 2; ++q) {
            dxb[q] = v3(1, q, 0) - v3(0, q, 0);
            dxt[q] = v3(1, q, 1) - v3(0, q, 1);
            dyb[q] = v3(q, 1, 0) - v3(q, 0, 0);
            dyt[q] = v3(q, 1, 1) - v3(q, 0, 1);
            for (int r = 0; r < 2; ++r) dz[q][r] = v3(q, r, 1) - v3(q, r, 0);
        }
        modal_element<double>(*out, 1.0, dxb, dxt, dyb, dyt, dz, f);
        // the energy form on the unit vector gives the diagonal entry
        V3<double> bm[8];
        modal_amplitudes<double>(dxb, dxt, dyb, dyt, dz, bm);
        dev = std::max(dev, std::fabs(modal_energy<double>(*out, bm) - ke[col * 24 + col]));
        for (int a = 0; a < 8; ++a) {
            const V3<double>& fa = f[LOCAL[a][0]][LOCAL[a][1]][LOCAL[a][2]];
            const double fc[3] = {fa.xy.x, fa.xy.y, fa.z};
            for (int c = 0; c < 3; ++c) dev = std::max(dev, std::fabs(fc[c] - ke[(3 * a + c) * 24 + col]));
        }
    }
    return dev / kmax;
}

// ------------------------------------------------------------------ declarations from other units

void cheb_coefficients(double bound, double lo_frac, int degree, double* out);

int solver_setup_domain(anl_ctx* c, const uint8_t* active, const uint8_t* fixed, cudaStream_t s);
int solver_apply(anl_ctx* c, const float* escale, const void* u, void* y, cudaStream_t s);
int solver_solve(anl_ctx* c, const float* escale, const double* f, double* x, int nrhs, double rtol, int maxiter,
                 int rebuild, int* iters, double* relres, cudaStream_t s);
int solver_dot(anl_ctx* c, const double* a, const double* b, double* out, cudaStream_t s);
int filter_init(anl_ctx* c, double r, cudaStream_t s);
int element_stress(anl_ctx* c, const double* u, const double* Emat, double Escalar, double* sig, double* vm,
                   cudaStream_t s);
int filter_apply(anl_ctx* c, bool forward, const float* in, float* out, cudaStream_t s);
int physical(anl_ctx* c, const float* x, const uint8_t* frozen, double beta, double eta, float* xphys, float* dxp,
             cudaStream_t s);
int stiffness_scale(anl_ctx* c, const float* xphys, const float* phi, double E0, double emin, double p, float* escale,
                    cudaStream_t s);
int sensitivity(anl_ctx* c, const double* u, int nrhs, const double* coef, const float* xphys, const float* dxp,
                const float* phi, double p, double emin, double E0, float* out, float* dv, bool energy_only,
                cudaStream_t s);
int oc_update(anl_ctx* c, const float* x, const float* dcx, const float* dvx, const float* phi, const uint8_t* frozen,
              double move, double beta, double eta, double vtarget, float* xnew, int* steps_out, double* lam_out,
              cudaStream_t s);
int design_stats(anl_ctx* c, const float* xold, const float* xnew, const float* xphys, const float* phi,
                 const uint8_t* frozen, double* out, cudaStream_t s);
int ku_grid_blocks(const Dims& d);
void ku_prepare();
int solver_profile_apply(anl_ctx* c, const void* u, void* y, int reps, double* ms, cudaStream_t s);
int solver_profile_pass(anl_ctx* c, int pass, int reps, double* ms, cudaStream_t s);

// ------------------------------------------------------------------ context

// the smoother's coefficients for every level: kChebMax steps (the pair of step k does not
// depend on how many steps a sweep takes, so every level reads the prefix it needs: 2 steps on
// levels 0-1, mg_degree_coarse below, 16 on a last level that is not solved densely)
static cudaError_t upload_cheb(anl_ctx* c) {
    std::vector<double> h(c->lev.size() * kChebStride, 0.0);
    for (size_t l = 0; l < c->lev.size(); ++l) {
        cheb_coefficients(c->lmax_bound, l >= 2 ? c->cheb_lo_coarse : c->cheb_lo, kChebMax, h.data() + l * kChebStride);
        c->lev[l].lmax = c->lmax_bound;
    }
    return cudaMemcpy(c->cheb_d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
}

static void free_ctx(anl_ctx* c) {
    if (!c) return;
    if (c->sc_base) {  // the single-vector pointers may point at another slot: free the arrays
        c->sc = c->sc_base;
        c->xbuf = c->xbuf_base;
        c->bbuf = c->bbuf_base;
        c->bdf = c->bdf_base;
        if (!c->lev.empty()) c->lev[0].b = c->b0_base;
    }
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    auto f = [](void* p) {
        if (p) cudaFree(p);
    };
    for (auto& L : c->lev) {
        f(L.E);
        f(L.eact);
        f(L.nmask);
        f(L.diag);
        f(L.x);
        f(L.xt);
        f(L.b);
        f(L.r);
        f(L.dv);
    }
    f(c->ke_d);
    f(c->cheb_d);
    f(c->active);
    f(c->A);
    f(c->Ainv);
    f(c->ainv_hi);
    f(c->sens_df);
    f(c->oc_el);
    f(c->oc_gw);
    f(c->oc_state);
    f(c->ainv_lo);
    f(c->flag_d);
    f(c->restart_d);
    f(c->p);
    f(c->q);
    f(c->xhi);
    f(c->xdf);
    f(c->bdf);
    f(c->xlo);
    f(c->y1);
    f(c->y2);
    f(c->tmp);
    f(c->xbuf);
    f(c->bbuf);
    f(c->sc);
    f(c->partials);
    f(c->counter);
    f(c->red_out);
    f(c->filt.w);
    f(c->filt.Hs);
    f(c->ftmp);
    f(c->ftmp2);
    if (c->cg_exec) cudaGraphExecDestroy(c->cg_exec);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    if (c->sc_h) cudaFreeHost(c->sc_h);
    if (c->red_h) cudaFreeHost(c->red_h);
    delete c;
}

static int create(anl_ctx** out, int nx, int ny, int nz, double h, double nu, int flags) {
    if (!out || nx < 1 || ny < 1 || nz < 1 || !(h > 0) || !(nu > -1.0 && nu < 0.5)) {
        set_error("anl_ctx_create: bad arguments (grid %d x %d x %d, h %g, nu %g)", nx, ny, nz, h, nu);
        return ANL_ERR_BADARG;
    }
    anl_ctx* c = new (std::nothrow) anl_ctx();
    if (!c) return ANL_ERR_NOMEM;
    *out = nullptr;
    c->d = Dims{nx, ny, nz};
    c->h = h;
    c->nu = nu;
    c->flags = flags;
    c->fp64 = (flags & ANL_FLAG_FP64) != 0;
    c->rmax = std::max(1, (flags >> 8) & 0xFF);
    c->tsize = c->fp64 ? 8 : 4;
    hex8_ke(nu, 1.0, c->ke);
    const double dev = ke_blocks(c->ke, &c->kbd);
    if (dev > 1e-12) {
        set_error("element matrix lacks the reflection structure (deviation %g)", dev);
        free_ctx(c);
        return ANL_ERR_BADARG;
    }
    const double mdev = ke_modal(c->ke, &c->kmd);
    if (!(mdev < 1e-12)) {
        set_error("element matrix lacks the isotropic mode structure (deviation %g)", mdev);
        free_ctx(c);
        return ANL_ERR_BADARG;
    }
    c->kmf = KeModal<float>{(float)c->kmd.ab, (float)c->kmd.b, (float)c->kmd.c,  (float)c->kmd.d,
                            (float)c->kmd.f,  (float)c->kmd.gh, (float)c->kmd.h, (float)c->kmd.j};
    c->kmdf = KeModal<DF>{DF(c->kmd.ab), DF(c->kmd.b), DF(c->kmd.c),  DF(c->kmd.d),
                          DF(c->kmd.f),  DF(c->kmd.gh), DF(c->kmd.h), DF(c->kmd.j)};
    c->kdiag = c->ke[0];
    {  // largest eigenvalue of Ke by power iteration in FP64 (Ke is positive semidefinite)
        double v[24], w[24], lam = 0.0;
        for (int i = 0; i < 24; ++i) v[i] = 1.0 + 0.01 * i * (i % 3 + 1);
        for (int it = 0; it < 3000; ++it) {
            double nrm = 0.0;
            for (int i = 0; i < 24; ++i) {
                double sacc = 0.0;
                for (int j = 0; j < 24; ++j) sacc += c->ke[i * 24 + j] * v[j];
                w[i] = sacc;
                nrm += sacc * sacc;
            }
            nrm = std::sqrt(nrm);
            double vw = 0.0, vv = 0.0;
            for (int i = 0; i < 24; ++i) {
                vw += v[i] * w[i];
                vv += v[i] * v[i];
            }
            lam = vw / vv;
            for (int i = 0; i < 24; ++i) v[i] = w[i] / nrm;
        }
        c->lmax_bound = 1.001 * lam / c->kdiag;
    }

#define ALLOC(ptr, bytes)                                                  \
    do {                                                                   \
        if (cudaMalloc((void**)&(ptr), (bytes)) != cudaSuccess) {          \
            set_error("cudaMalloc of %zu bytes failed", (size_t)(bytes));  \
            cudaGetLastError();                                            \
            free_ctx(c);                                                   \
            return ANL_ERR_NOMEM;                                          \
        }                                                                  \
    } while (0)

    // hierarchy
    Dims dd = c->d;
    while (true) {
        Level L;
        L.d = dd;
        c->lev.push_back(L);
        const int64_t ndof = 3 * dd.nn();
        if (ndof <= 400 || dd.nx < 2 || dd.ny < 2 || dd.nz < 2 || c->lev.size() >= 16) break;
        dd = Dims{(dd.nx + 1) / 2, (dd.ny + 1) / 2, (dd.nz + 1) / 2};
    }
    const size_t ts = c->tsize;
    const size_t R = (size_t)c->rmax;
    for (auto& L : c->lev) {
        const int64_t ne = L.d.ne(), nn = L.d.nn();
        L.vs = (3 * nn + 63) / 64 * 64;
        ALLOC(L.E, ne * sizeof(float));
        ALLOC(L.eact, ne);
        ALLOC(L.nmask, nn);
        ALLOC(L.diag, nn * sizeof(float));
        ALLOC(L.x, R * L.vs * ts);
        ALLOC(L.xt, R * L.vs * ts);
        ALLOC(L.b, R * L.vs * ts);
        ALLOC(L.r, R * L.vs * ts);
        ALLOC(L.dv, R * L.vs * ts);
    }
    const int64_t vs0 = c->lev[0].vs;
    const Level& C = c->lev.back();
    c->nc = (int)(3 * C.d.nn());
    c->dense_coarse = c->nc <= 700;
    if (c->dense_coarse) {
        ALLOC(c->A, (size_t)c->nc * c->nc * sizeof(double));
        ALLOC(c->Ainv, (size_t)c->nc * c->nc * sizeof(double));
        if (!c->fp64) {
            ALLOC(c->ainv_hi, (size_t)c->nc * c->nc * sizeof(float));
            ALLOC(c->ainv_lo, (size_t)c->nc * c->nc * sizeof(float));
        }
    }
    ALLOC(c->flag_d, 4 * sizeof(int));
    ALLOC(c->restart_d, R * sizeof(int));
    ALLOC(c->cheb_d, c->lev.size() * kChebStride * sizeof(double));
    ALLOC(c->ke_d, 576 * sizeof(double));
    if (cudaMemcpy(c->ke_d, c->ke, 576 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("copy of the element matrix failed");
        free_ctx(c);
        return ANL_ERR_CUDA;
    }
    const int64_t ne = c->d.ne(), nn = c->d.nn();
    ALLOC(c->active, ne);
    ALLOC(c->p, R * vs0 * ts);
    ALLOC(c->q, R * vs0 * ts);
    ALLOC(c->xhi, 3 * nn * ts);
    ALLOC(c->xlo, 3 * nn * ts);
    if (!c->fp64) {
        ALLOC(c->xdf, 3 * nn * sizeof(DF));
        ALLOC(c->bdf, R * vs0 * sizeof(DF));
    }
    ALLOC(c->y1, 3 * nn * ts);
    ALLOC(c->y2, 3 * nn * ts);
    ALLOC(c->tmp, 3 * nn * ts);
    ALLOC(c->xbuf, R * vs0 * sizeof(double));
    ALLOC(c->bbuf, R * vs0 * sizeof(double));
    ALLOC(c->sc, R * sizeof(PcgScalars));
    c->part_cap = std::max(ku_grid_blocks(c->d), kRedBlocks);
    {
        // the filter reduction grid (32 x 8 columns of 16 layers) can exceed both
        const int fb = ceil_div(c->d.nx, 32) * ceil_div(c->d.ny, 8) * ceil_div(c->d.nz, 16);
        c->part_cap = std::max(c->part_cap, fb);
    }
    c->part_stride = (int64_t)c->part_cap * kMaxRedVals;
    ALLOC(c->partials, R * c->part_stride * sizeof(double));
    ALLOC(c->counter, (16 + R) * sizeof(unsigned));
    ALLOC(c->red_out, 16 * sizeof(double));
    ALLOC(c->filt.Hs, ne * sizeof(float));
    ALLOC(c->ftmp, ne * sizeof(float));
    ALLOC(c->ftmp2, ne * sizeof(float));
#undef ALLOC
    if (cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("stream creation failed");
        free_ctx(c);
        return ANL_ERR_CUDA;
    }
    c->use_graph = std::getenv("ANL_NO_GRAPH") == nullptr;
    if (const char* e = std::getenv("ANL_BOX_FROM")) c->box_from = std::atoi(e);
    if (const char* e = std::getenv("ANL_TC")) c->use_tc = !c->fp64 && std::atoi(e) != 0;
    ku_prepare();
    kbox_prepare();
    if (c->use_tc && kutc_prepare(c->ke) != ANL_OK) {
        free_ctx(c);
        return ANL_ERR_CUDA;
    }
    // the V-cycle tail: the first level (level 2 or below, on the box levels) from which every
    // level to the coarsest fits one CTA (at most 1024 elements, the vectors in shared memory)
    {
        // on by default (ANL_TAIL=0 turns it off): on the 256x128x128 L-bracket the tail takes
        // levels 4-6 in 104 us per V-cycle against about 180 us for their 35 launches, 34.7
        // against 33.9 SIMP iterations/s at the same CG iterations
        const char* e = std::getenv("ANL_TAIL");
        const bool tail_on = !(e && std::atoi(e) == 0);
        const int nl = (int)c->lev.size();
        if (tail_on && !c->fp64 && c->dense_coarse && nl >= 2) {
            for (int l = std::max(c->box_from, 2); l <= nl - 2 && c->tail_from < 0; ++l) {
                if (nl - l > kTailMaxLevels || c->lev[l].d.ne() > 1024) continue;
                TailLevel tl[kTailMaxLevels];
                for (int q = l; q < nl; ++q) tl[q - l].d = c->lev[q].d;
                if (tail_smem_bytes(tl, nl - l) <= (size_t)kTailMaxSmem) c->tail_from = l;
            }
        }
        if (c->tail_from >= 0 && vtail_prepare() != ANL_OK) {
            free_ctx(c);
            return ANL_ERR_CUDA;
        }
    }
    c->b0_base = c->lev[0].b;
    c->xbuf_base = c->xbuf;
    c->bbuf_base = c->bbuf;
    c->bdf_base = c->bdf;
    c->sc_base = c->sc;
    if (cudaMallocHost((void**)&c->sc_h, R * sizeof(PcgScalars)) != cudaSuccess ||
        cudaMallocHost((void**)&c->red_h, 16 * sizeof(double)) != cudaSuccess) {
        set_error("pinned host allocation failed");
        free_ctx(c);
        return ANL_ERR_NOMEM;
    }
    if (cudaMemset(c->counter, 0, (16 + R) * sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(c->restart_d, 0, R * sizeof(int)) != cudaSuccess ||
        upload_cheb(c) != cudaSuccess ||
        cudaMemset(c->flag_d, 0, 4 * sizeof(int)) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
        set_error("context initialisation failed: %s", cudaGetErrorString(cudaGetLastError()));
        free_ctx(c);
        return ANL_ERR_CUDA;
    }
    *out = c;
    return ANL_OK;
}

}  // namespace anl

using namespace anl;

static inline cudaStream_t S(anl_stream_t s) { return (cudaStream_t)s; }

#define NEED(cond, msg)            \
    do {                           \
        if (!(cond)) {             \
            anl::set_error(msg);   \
            return ANL_ERR_BADARG; \
        }                          \
    } while (0)

extern "C" {

int anl_version(void) { return 100; }

const char* anl_last_error(void) { return anl::g_err; }

int64_t anl_launch_count(void) { return (int64_t)anl::g_launches.load(); }

int anl_debug_oob(long long* count_h, long long* first_h) {
    NEED(count_h && first_h, "anl_debug_oob: null argument");
    first_h[0] = first_h[1] = first_h[2] = 0;
#if ANL_DEBUG
    unsigned long long n = 0;
    ANL_TRY(anl::debug_take_ku(&n, first_h));
    ANL_TRY(anl::debug_take_kbox(&n, first_h));
    ANL_TRY(anl::debug_take_solver(&n, first_h));
    ANL_TRY(anl::debug_take_design(&n, first_h));
    ANL_TRY(anl::debug_take_vtail(&n, first_h));
    *count_h = (long long)n;
#else
    *count_h = -1;
#endif
    return ANL_OK;
}

int anl_ctx_create(anl_ctx** out, int nx, int ny, int nz, double h, double nu, int flags) {
    anl::g_err[0] = 0;
    std::lock_guard<std::recursive_mutex> lock(anl::device_sync_mutex());
    return create(out, nx, ny, nz, h, nu, flags);
}

void anl_ctx_destroy(anl_ctx* ctx) { free_ctx(ctx); }

int anl_set_domain(anl_ctx* ctx, const uint8_t* active, const uint8_t* fixed, int64_t* nfree_h, anl_stream_t stream) {
    NEED(ctx && active && fixed, "anl_set_domain: null argument");
    int st = solver_setup_domain(ctx, active, fixed, S(stream));
    if (st == ANL_OK && nfree_h) *nfree_h = ctx->nfree;
    return st;
}

int anl_free_mask(anl_ctx* ctx, uint8_t* mask, anl_stream_t stream);

int anl_apply_K(anl_ctx* ctx, const float* escale, const void* u, void* y, anl_stream_t stream) {
    NEED(ctx && escale && u && y, "anl_apply_K: null argument");
    if (!ctx->domain_set) {
        set_error("anl_apply_K: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    return solver_apply(ctx, escale, u, y, S(stream));
}

int anl_solve(anl_ctx* ctx, const float* escale, const double* f, double* x, int nrhs, double rtol, int maxiter,
              int rebuild, int* iters, double* relres, anl_stream_t stream) {
    NEED(ctx && escale && f && x && iters && relres, "anl_solve: null argument");
    NEED(nrhs >= 1 && rtol > 0 && maxiter >= 1, "anl_solve: need nrhs >= 1, rtol > 0, maxiter >= 1");
    if (!ctx->domain_set) {
        set_error("anl_solve: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    return solver_solve(ctx, escale, f, x, nrhs, rtol, maxiter, rebuild, iters, relres, S(stream));
}

int anl_solve_status(const anl_ctx* ctx, int k) {
    NEED(ctx, "anl_solve_status: null context");
    NEED(k >= 0 && k < (int)ctx->last_status.size(), "anl_solve_status: k outside the last solve's cases");
    return ctx->last_status[k];
}

int anl_dot(anl_ctx* ctx, const double* a, const double* b, double* out_h, anl_stream_t stream) {
    NEED(ctx && a && b && out_h, "anl_dot: null argument");
    return solver_dot(ctx, a, b, out_h, S(stream));
}

int anl_element_energy(anl_ctx* ctx, const double* u, float* ce, anl_stream_t stream) {
    NEED(ctx && u && ce, "anl_element_energy: null argument");
    if (!ctx->domain_set) {
        set_error("anl_element_energy: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    return sensitivity(ctx, u, 1, nullptr, nullptr, nullptr, nullptr, 1.0, 0.0, 1.0, ce, nullptr, true, S(stream));
}

int anl_element_stress(anl_ctx* ctx, const double* u, const double* E_material, double E_scalar, double* sig,
                       double* vm, anl_stream_t stream) {
    NEED(ctx && u && (sig || vm), "anl_element_stress: null argument");
    if (!ctx->domain_set) {
        set_error("anl_element_stress: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    return element_stress(ctx, u, E_material, E_scalar, sig, vm, S(stream));
}

int anl_sensitivity(anl_ctx* ctx, const double* u, int nrhs, const double* coef, const float* xphys, const float* dxp,
                    const float* phi, double p, double emin, double E0, float* out, float* dv, anl_stream_t stream) {
    NEED(ctx && u && coef && xphys && phi && out, "anl_sensitivity: null argument");
    if (!ctx->domain_set) {
        set_error("anl_sensitivity: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    return sensitivity(ctx, u, nrhs, coef, xphys, dxp, phi, p, emin, E0, out, dv, false, S(stream));
}

int anl_stiffness_scale(anl_ctx* ctx, const float* xphys, const float* phi, double E0, double emin, double p,
                        float* escale, anl_stream_t stream) {
    NEED(ctx && xphys && phi && escale, "anl_stiffness_scale: null argument");
    if (!ctx->domain_set) {
        set_error("anl_stiffness_scale: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    return stiffness_scale(ctx, xphys, phi, E0, emin, p, escale, S(stream));
}

int anl_filter_init(anl_ctx* ctx, double r_vox, anl_stream_t stream) {
    NEED(ctx, "anl_filter_init: null context");
    if (!ctx->domain_set) {
        set_error("anl_filter_init: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    return filter_init(ctx, r_vox, S(stream));
}

#define NEED_FILTER(name)                                         \
    do {                                                          \
        if (!ctx->filt.ready) {                                   \
            set_error(name ": call anl_filter_init first");       \
            return ANL_ERR_STATE;                                 \
        }                                                         \
    } while (0)

int anl_filter_fwd(anl_ctx* ctx, const float* in, float* out, anl_stream_t stream) {
    NEED(ctx && in && out, "anl_filter_fwd: null argument");
    NEED_FILTER("anl_filter_fwd");
    return filter_apply(ctx, true, in, out, S(stream));
}

int anl_filter_bwd(anl_ctx* ctx, const float* in, float* out, anl_stream_t stream) {
    NEED(ctx && in && out, "anl_filter_bwd: null argument");
    NEED_FILTER("anl_filter_bwd");
    return filter_apply(ctx, false, in, out, S(stream));
}

int anl_physical(anl_ctx* ctx, const float* x, const uint8_t* frozen, double beta, double eta, float* xphys, float* dxp,
                 anl_stream_t stream) {
    NEED(ctx && x && frozen && xphys, "anl_physical: null argument");
    NEED_FILTER("anl_physical");
    return physical(ctx, x, frozen, beta, eta, xphys, dxp, S(stream));
}

int anl_oc_update(anl_ctx* ctx, const float* x, const float* dcx, const float* dvx, const float* phi,
                  const uint8_t* frozen, double move, double beta, double eta, double vtarget, float* xnew,
                  int* steps_h, double* lambda_h, anl_stream_t stream) {
    NEED(ctx && x && dcx && dvx && phi && frozen && xnew, "anl_oc_update: null argument");
    NEED_FILTER("anl_oc_update");
    return oc_update(ctx, x, dcx, dvx, phi, frozen, move, beta, eta, vtarget, xnew, steps_h, lambda_h, S(stream));
}

int anl_profile_apply(anl_ctx* ctx, const void* u, void* y, int reps, double* ms_h, anl_stream_t stream) {
    NEED(ctx && u && y && ms_h && reps >= 1, "anl_profile_apply: bad argument");
    if (!ctx->domain_set) {
        set_error("anl_profile_apply: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    return solver_profile_apply(ctx, u, y, reps, ms_h, S(stream));
}

int anl_profile_pass(anl_ctx* ctx, int pass, int reps, double* ms_h, anl_stream_t stream) {
    NEED(ctx && ms_h && reps >= 1, "anl_profile_pass: bad argument");
    if (!ctx->domain_set || !ctx->coarse_ready) {
        set_error("anl_profile_pass: run a solve on this context first");
        return ANL_ERR_STATE;
    }
    return solver_profile_pass(ctx, pass, reps, ms_h, S(stream));
}

int anl_mg_info(anl_ctx* ctx, int* nlev_h, int* dims_h, double* lmax_h) {
    NEED(ctx && nlev_h && dims_h && lmax_h, "anl_mg_info: null argument");
    *nlev_h = (int)ctx->lev.size();
    for (size_t l = 0; l < ctx->lev.size() && l < 16; ++l) {
        dims_h[3 * l] = ctx->lev[l].d.nx;
        dims_h[3 * l + 1] = ctx->lev[l].d.ny;
        dims_h[3 * l + 2] = ctx->lev[l].d.nz;
        lmax_h[l] = ctx->lev[l].lmax;
    }
    return ANL_OK;
}

int anl_design_stats(anl_ctx* ctx, const float* xold, const float* xnew, const float* xphys, const float* phi,
                     const uint8_t* frozen, double* out_h, anl_stream_t stream) {
    NEED(ctx && xold && xnew && xphys && phi && frozen && out_h, "anl_design_stats: null argument");
    if (!ctx->domain_set) {
        set_error("anl_design_stats: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    return design_stats(ctx, xold, xnew, xphys, phi, frozen, out_h, S(stream));
}

}  // extern "C"

// ------------------------------------------------------------------ free-DOF mask export

namespace anl {
__global__ void k_export_mask(int64_t nn, const uint8_t* nmask, uint8_t* out) {
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t m = nmask[n];
        out[3 * n] = m & 1;
        out[3 * n + 1] = (m >> 1) & 1;
        out[3 * n + 2] = (m >> 2) & 1;
    }
}
}  // namespace anl

extern "C" int anl_free_mask(anl_ctx* ctx, uint8_t* mask, anl_stream_t stream) {
    NEED(ctx && mask, "anl_free_mask: null argument");
    if (!ctx->domain_set) {
        set_error("anl_free_mask: call anl_set_domain first");
        return ANL_ERR_STATE;
    }
    const int64_t nn = ctx->d.nn();
    const int g = (int)std::min<int64_t>(4096, (nn + 255) / 256);
    k_export_mask<<<g, 256, 0, S(stream)>>>(nn, ctx->lev[0].nmask, mask);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}
