// anl_design.cu -- design-variable kernels of one SIMP iteration: density filter,
// projection, stiffness scale, sensitivity, OC bisection and the history statistics.
//
// Element fields are FP32 on the full grid (x fastest, zero on inactive elements); sums
// that decide the OC bisection and the history values accumulate in FP64.
#include <algorithm>
#include <cstddef>
#include <cmath>
#include <vector>

#include "anl_ctx.cuh"

namespace anl {

constexpr int DT = 256;
static inline int dgrid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(kRedBlocks, (n + DT - 1) / DT)); }

// ------------------------------------------------------------------ density filter

// Filter (optimize.py:24-47). One CTA of 32x8 threads owns a 32x8 column of elements over
// FT_ZC layers and marches up z: a ring of 2R + 2 element planes (each with an R-element halo
// in x and y) in shared memory, one new plane staged per layer, one barrier per layer (the ring
// has one slot more than the stencil reads, so the next plane never lands in a slot in use).
// The taps are summed in (dz, dy, dx) order.
enum { F_HS = 0, F_FWD = 1, F_BWD = 2, F_PHYS = 3, F_OCVOL = 4 };

constexpr int FT_X = 32, FT_Y = 8, FT_ZC = 16, FT_N = FT_X * FT_Y;

struct FilterArgs {
    Dims d;
    int R;
    const float* w;        // (2R+1)^3 cone weights
    const uint8_t* active;
    const float* Hs;
    const float* in;       // FWD/BWD/PHYS input field
    float* out;
    // PHYS
    const uint8_t* frozen;
    float* dxp;
    float beta, eta, t0, t1;
    // OCVOL: the filtered field is xn(lambda) built on the fly
    const float* x;
    const float* dcx;
    const float* dvx;
    const float* phi;
    float lam, move;
    double* partials;
    unsigned* counter;
    double* red_out;
};

// optimize.py:150-152: ratio = sqrt(max(-dcx,0) / max(dvx*lam, 1e-300)),
// xn = clip(x*ratio, max(0, x-mv), min(1, x+mv)). Split into the part of an element that does
// not depend on lambda (x sqrt(max(-dcx,0)/dvx)) and one multiply by 1/sqrt(lambda), so a bank
// of lambdas costs a multiply and a clamp each.
struct OcElem {
    float s;       // x sqrt(max(-dcx, 0) / dvx)
    float dvx;
    float lo, hi;  // the move limits
    bool grows;    // max(-dcx, 0) > 0 and x > 0: the ratio is huge where dvx lambda underflows
};
__device__ __forceinline__ OcElem oc_elem(float x, float dcx, float dvx, float move) {
    OcElem o;
    const float num = fmaxf(-dcx, 0.f);
    o.s = dvx > 0.f ? x * sqrtf(num / dvx) : 0.f;
    o.dvx = dvx;
    o.lo = fmaxf(0.f, x - move);
    o.hi = fminf(1.f, x + move);
    o.grows = num > 0.f && x > 0.f;
    return o;
}
__device__ __forceinline__ float oc_rl(float lam) { return 1.f / sqrtf(lam); }
__device__ __forceinline__ float oc_xn(const OcElem& o, float lam, float rl) {
    const float v = o.dvx * lam > 1e-30f ? o.s * rl : (o.grows ? INFINITY : 0.f);
    return fminf(fmaxf(v, o.lo), o.hi);
}
__device__ __forceinline__ float oc_xn(float x, float dcx, float dvx, float lam, float move) {
    return oc_xn(oc_elem(x, dcx, dvx, move), lam, oc_rl(lam));
}

// the filter's input value of element (gi, gj, gk) (zero outside the grid and on inactive
// elements): the active flag and the field are loaded independently of each other
template <int MODE>
__device__ __forceinline__ float filter_input(const FilterArgs& a, int gi, int gj, int gk) {
    const Dims& d = a.d;
    if (gi < 0 || gj < 0 || gk < 0 || gi >= d.nx || gj >= d.ny || gk >= d.nz) return 0.f;
    const int64_t e = d.elem(gi, gj, gk);
    if (!ANL_IN_RANGE(e, d.ne())) return 0.f;
    const bool act = a.active[e] != 0;
    float v = 1.f;
    if (MODE == F_FWD || MODE == F_PHYS) v = a.in[e];
    else if (MODE == F_BWD) v = a.in[e] / a.Hs[e];
    else if (MODE == F_OCVOL) v = a.frozen[e] ? 1.f : oc_xn(a.x[e], a.dcx[e], a.dvx[e], a.lam, a.move);
    return act ? v : 0.f;
}

// RT: the halo at compile time (1: the 27-tap cone of radii up to 2, weights in registers),
// or 0 for any R up to kMaxFilterR
template <int MODE, int RT>
__global__ void __launch_bounds__(FT_N) k_filter(FilterArgs a) {
    extern __shared__ float sm[];
    const Dims d = a.d;
    const int R = RT > 0 ? RT : a.R, W = 2 * R + 1;
    const int TX = FT_X + 2 * R, TY = FT_Y + 2 * R, PL = TX * TY, NS = W + 1;  // ring of NS planes
    float* ring = sm;
    float* wts = sm + NS * PL;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + FT_X * ty;
    const int i0 = blockIdx.x * FT_X, j0 = blockIdx.y * FT_Y, kb = blockIdx.z * FT_ZC;
    const int kend = min(kb + FT_ZC, d.nz);
    for (int t = tid; t < W * W * W; t += FT_N) wts[t] = a.w[t];
    // stage element plane gk into its ring slot
    auto stage = [&](int gk) {
        float* pl = ring + ((gk + NS * (kMaxFilterR + 1)) % NS) * PL;
        for (int y = ty; y < TY; y += FT_Y)
            for (int x = tx; x < TX; x += FT_X) pl[y * TX + x] = filter_input<MODE>(a, i0 - R + x, j0 - R + y, gk);
    };
    // the next plane's values of this thread, loaded a layer ahead (registers; the plane of a
    // 27-tap filter is 34 x 10 values, at most 2 per thread)
    constexpr int PF = RT == 1 ? (34 * 10 + FT_N - 1) / FT_N : 1;
    float pf[PF];
    auto prefetch = [&](int gk) {
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            const int t = tid + q * FT_N, y = t / (FT_X + 2), x = t - y * (FT_X + 2);
            pf[q] = t < PL ? filter_input<MODE>(a, i0 - 1 + x, j0 - 1 + y, gk) : 0.f;
        }
    };
    auto commit = [&](int gk) {
        float* pl = ring + ((gk + NS * (kMaxFilterR + 1)) % NS) * PL;
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            const int t = tid + q * FT_N;
            if (t < PL) pl[t] = pf[q];
        }
    };
    for (int gk = kb - R; gk < kb + R; ++gk) stage(gk);
    if (RT == 1) prefetch(kb + R);
    __syncthreads();
    float wr[RT > 0 ? 27 : 1];
    if (RT == 1) {
#pragma unroll
        for (int q = 0; q < (RT > 0 ? 27 : 1); ++q) wr[q] = wts[q];
    }
    const int i = i0 + tx, j = j0 + ty;
    const bool in_xy = i < d.nx && j < d.ny;
    double vol = 0.0;
    for (int k = kb; k < kend; ++k) {
        // this layer's epilogue inputs, loaded before the barrier so their latency overlaps it
        const int64_t e = in_xy ? d.elem(i, j, k) : 0;
        const bool in_e = in_xy && ANL_IN_RANGE(e, d.ne());
        bool act = false, fzn = false;
        float hs = 1.f, ph = 0.f;
        if (in_e) {
            act = a.active[e] != 0;
            if (MODE == F_FWD || MODE == F_PHYS || MODE == F_OCVOL) hs = a.Hs[e];
            if (MODE == F_PHYS || MODE == F_OCVOL) fzn = a.frozen[e] != 0;
            if (MODE == F_OCVOL) ph = a.phi[e];
        }
        if (RT == 1) {  // plane k + 1 was loaded during the previous layer; load plane k + 2
            commit(k + 1);
            if (k + 1 < kend) prefetch(k + 2);
        } else {
            stage(k + R);
        }
        __syncthreads();
        if (in_e) {
            float s = 0.f;
            if (RT == 1) {
#pragma unroll
                for (int dz = 0; dz < 3; ++dz) {
                    const float* pl = ring + ((k - 1 + dz + NS * (kMaxFilterR + 1)) % NS) * PL;
#pragma unroll
                    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                        for (int dx = 0; dx < 3; ++dx) s = fmaf(wr[(dz * 3 + dy) * 3 + dx], pl[(ty + dy) * TX + tx + dx], s);
                }
            } else {
                for (int dz = 0; dz < W; ++dz) {
                    const float* pl = ring + ((k - R + dz + NS * (kMaxFilterR + 1)) % NS) * PL;
                    for (int dy = 0; dy < W; ++dy) {
                        const float* row = pl + (ty + dy) * TX + tx;
                        const float* w = wts + (dz * W + dy) * W;
                        for (int dx = 0; dx < W; ++dx) s = fmaf(w[dx], row[dx], s);
                    }
                }
            }
            if (MODE == F_HS) {
                a.out[e] = s == 0.f ? 1.f : s;
            } else if (MODE == F_FWD) {
                a.out[e] = act ? s / hs : 0.f;
            } else if (MODE == F_BWD) {
                a.out[e] = act ? s : 0.f;
            } else {
                // physical(): projection (optimize.py:81-87), frozen -> 1 (optimize.py:92)
                float xt = act ? s / hs : 0.f;
                float xp = xt, g = 1.f;
                if (a.beta > 0.f) {
                    const float th = tanhf(a.beta * (xt - a.eta));
                    xp = (a.t0 + th) / (a.t0 + a.t1);
                    g = a.beta * (1.f - th * th) / (a.t0 + a.t1);
                }
                if (fzn) xp = 1.f;
                if (!act) {
                    xp = 0.f;
                    g = 0.f;
                }
                if (MODE == F_PHYS) {
                    a.out[e] = xp;
                    if (a.dxp) a.dxp[e] = g;
                } else {
                    vol += act ? (double)ph * (double)xp : 0.0;
                }
            }
        }
    }
    if (MODE == F_OCVOL) {
        __shared__ double red[FT_N / 32];
        double v[1] = {vol};
        block_sum<1, FT_N>(v, red, tid);
        const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        finish_reduction<1, FT_N>(v, bid, gridDim.x * gridDim.y * gridDim.z, a.partials, a.counter, a.red_out, tid, red);
    }
}

static int launch_filter(anl_ctx* c, int mode, FilterArgs a, cudaStream_t s) {
    const Dims& d = c->d;
    a.d = d;
    a.R = c->filt.R;
    a.w = c->filt.w;
    a.active = c->active;
    a.Hs = c->filt.Hs;
    const int W = 2 * a.R + 1;
    const size_t smem = sizeof(float) * ((W + 1) * (FT_X + 2 * a.R) * (FT_Y + 2 * a.R) + W * W * W);
    dim3 grid(ceil_div(d.nx, FT_X), ceil_div(d.ny, FT_Y), ceil_div(d.nz, FT_ZC)), block(FT_X, FT_Y);
    if (mode == F_OCVOL && (int64_t)grid.x * grid.y * grid.z > c->part_cap) {
        set_error("filter reduction needs %d blocks, scratch holds %d", grid.x * grid.y * grid.z, c->part_cap);
        return ANL_ERR_BADARG;
    }
#define F_LAUNCH(M)                                                              \
    (a.R == 1 ? k_filter<M, 1><<<grid, block, smem, s>>>(a) : k_filter<M, 0><<<grid, block, smem, s>>>(a))
    switch (mode) {
        case F_HS: F_LAUNCH(F_HS); break;
        case F_FWD: F_LAUNCH(F_FWD); break;
        case F_BWD: F_LAUNCH(F_BWD); break;
        case F_PHYS: F_LAUNCH(F_PHYS); break;
        case F_OCVOL: F_LAUNCH(F_OCVOL); break;
        default: return ANL_ERR_BADARG;
    }
#undef F_LAUNCH
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int filter_init(anl_ctx* c, double r, cudaStream_t s) {
    int R = (int)std::ceil(r) - 1;
    if (R < 1) R = 1;
    if (R > kMaxFilterR || !(r > 0)) {
        set_error("filter radius %.3f voxels needs a %d-element halo; at most %d is supported", r, R, kMaxFilterR);
        return ANL_ERR_BADARG;
    }
    const int W = 2 * R + 1;
    std::vector<float> w(W * W * W);
    for (int dz = -R; dz <= R; ++dz)
        for (int dy = -R; dy <= R; ++dy)
            for (int dx = -R; dx <= R; ++dx) {
                const double v = r - std::sqrt((double)(dx * dx + dy * dy + dz * dz));
                w[(dx + R) + W * ((dy + R) + W * (dz + R))] = v > 0 ? (float)v : 0.f;
            }
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    if (c->filt.w) cudaFree(c->filt.w);
    c->filt.w = nullptr;
    ANL_CUDA(cudaMalloc(&c->filt.w, sizeof(float) * w.size()));
    ANL_CUDA(cudaMemcpyAsync(c->filt.w, w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice, s));
    c->filt.R = R;
    c->filt.r = r;
    FilterArgs a{};
    a.out = c->filt.Hs;
    ANL_TRY(launch_filter(c, F_HS, a, s));
    ANL_CUDA(cudaStreamSynchronize(s));  // the host weights vector goes out of scope
    c->filt.ready = true;
    return ANL_OK;
}

int filter_apply(anl_ctx* c, bool forward, const float* in, float* out, cudaStream_t s) {
    FilterArgs a{};
    a.in = in;
    a.out = out;
    return launch_filter(c, forward ? F_FWD : F_BWD, a, s);
}

int physical(anl_ctx* c, const float* x, const uint8_t* frozen, double beta, double eta, float* xphys, float* dxp,
             cudaStream_t s) {
    FilterArgs a{};
    a.in = x;
    a.out = xphys;
    a.frozen = frozen;
    a.dxp = dxp;
    a.beta = (float)beta;
    a.eta = (float)eta;
    if (beta > 0) {
        a.t0 = (float)std::tanh(beta * eta);
        a.t1 = (float)std::tanh(beta * (1 - eta));
    }
    return launch_filter(c, F_PHYS, a, s);
}

// ------------------------------------------------------------------ stiffness scale

__global__ void k_escale(int64_t ne, const uint8_t* active, const float* xphys, const float* phi, float E0, float emin,
                         float p, float* escale) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        float v = 0.f;
        if (active[e]) {
            const float xp = xphys[e];
            const float xpp = p == 1.f ? xp : (p == 3.f ? xp * xp * xp : powf(xp, p));
            v = E0 * phi[e] * (emin + xpp * (1.f - emin));
        }
        escale[e] = v;
    }
}

int stiffness_scale(anl_ctx* c, const float* xphys, const float* phi, double E0, double emin, double p, float* escale,
                    cudaStream_t s) {
    const int64_t ne = c->d.ne();
    k_escale<<<dgrid(ne), DT, 0, s>>>(ne, c->active, xphys, phi, (float)E0, (float)emin, (float)p, escale);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

// ------------------------------------------------------------------ sensitivity

constexpr int kMaxCases = 16;
struct SensArgs {
    Dims d;
    const uint8_t* active;
    const DF* u;      // nrhs nodal vectors as float pairs (k_split_pairs)
    int nrhs;
    int64_t stride;   // 3 * nn
    float coef[kMaxCases];
    const float* xphys;
    const float* dxp;
    const float* phi;
    float p, emin, E0, h;
    float* out;       // dc (combined, clipped, times dxp) or ce (energy only)
    float* dv;        // phi * dxp (optional)
    int energy_only;
};

// The FP64 displacements as float pairs, once per node (split_double: no FP64 arithmetic);
// the element kernel then reads each corner as one 8-byte pair instead of splitting it again
// for each of its up to 8 elements.
__global__ void k_split_pairs(int64_t n, const double* x, DF* xdf) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float h, l;
        split_double(x[i], h, l);
        xdf[i] = DF(h, l);
    }
}

// u_e^T Ke u_e from the modal energy form (modal_energy): edge differences are formed in
// double-float arithmetic from the FP64 displacements and rounded once to FP32, and rigid
// rotations cancel inside squares, so the result keeps its accuracy relative to the element's
// own strain energy.
__device__ __forceinline__ float element_energy(const KeModal<float>& K, const DF* u, const Dims& d, int i, int j,
                                                int k) {
    const int64_t sx = 1, sy = d.nx + 1, sz = (int64_t)(d.nx + 1) * (d.ny + 1);
    const int64_t n0 = d.node(i, j, k);
    if (!ANL_IN_RANGE(n0, d.nn()) || !ANL_IN_RANGE(n0 + sx + sy + sz, d.nn())) return 0.f;
    float ch[2][2][2][3], cl[2][2][2][3];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int px = q & 1, py = (q >> 1) & 1, pz = (q >> 2) & 1;
        const int64_t n = n0 + px * sx + py * sy + pz * sz;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 t = __ldg(reinterpret_cast<const float2*>(u + 3 * n + c));
            ch[px][py][pz][c] = t.x;
            cl[px][py][pz][c] = t.y;
        }
    }
    auto diff = [&](int ax, int bx, int ay, int by, int az, int bz) {
        V3<float> v;
        v.xy.x = df_diff(ch[ax][ay][az][0], cl[ax][ay][az][0], ch[bx][by][bz][0], cl[bx][by][bz][0]);
        v.xy.y = df_diff(ch[ax][ay][az][1], cl[ax][ay][az][1], ch[bx][by][bz][1], cl[bx][by][bz][1]);
        v.z = df_diff(ch[ax][ay][az][2], cl[ax][ay][az][2], ch[bx][by][bz][2], cl[bx][by][bz][2]);
        return v;
    };
    V3<float> dxb[2], dxt[2], dyb[2], dyt[2], dz[2][2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        dxb[q] = diff(1, 0, q, q, 0, 0);
        dxt[q] = diff(1, 0, q, q, 1, 1);
        dyb[q] = diff(q, q, 1, 0, 0, 0);
        dyt[q] = diff(q, q, 1, 0, 1, 1);
#pragma unroll
        for (int r = 0; r < 2; ++r) dz[q][r] = diff(q, q, r, r, 1, 0);
    }
    V3<float> bm[8];
    modal_amplitudes<float>(dxb, dxt, dyb, dyt, dz, bm);
    return modal_energy<float>(K, bm);
}

__global__ void k_sens(SensArgs a, KeModal<float> K) {
    const Dims d = a.d;
    const int64_t ne = d.ne();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        float v = 0.f;
        if (a.active[e]) {
            const int i = (int)(e % d.nx), j = (int)((e / d.nx) % d.ny), k = (int)(e / ((int64_t)d.nx * d.ny));
            if (a.energy_only) {
                v = a.h * element_energy(K, a.u, d, i, j, k);
            } else {
                const float xp = a.xphys[e];
                const float dpow = a.p == 1.f ? 1.f : (a.p == 3.f ? xp * xp : powf(xp, a.p - 1.f));
                const float pre = -a.p * dpow * (1.f - a.emin) * a.E0 * a.phi[e] * a.h;
                float dc = 0.f;
                for (int c = 0; c < a.nrhs; ++c) dc += a.coef[c] * pre * element_energy(K, a.u + c * a.stride, d, i, j, k);
                dc = fminf(dc, 0.f);
                v = a.dxp ? dc * a.dxp[e] : dc;
            }
        }
        a.out[e] = v;
        if (a.dv) a.dv[e] = a.active[e] ? (a.dxp ? a.phi[e] * a.dxp[e] : a.phi[e]) : 0.f;
    }
}

// Element-centre stress (fem.py:244-263): at the centre only the linear modes have slopes,
// du_c/dx_d = b_dc / (4 h) with b_dc = sum of the 4 edge differences of component c along d,
// so the strain is eps = (b1x, b2y, b3z, b2x + b1y, b3y + b2z, b1z + b3x) / (4 h) (Voigt,
// engineering shear) and sigma = E D eps with the isotropic D of unit modulus. FP64.
__global__ void k_stress(Dims d, const uint8_t* active, const double* u, const double* Emat, double Escalar, double h,
                         double lam, double mu, double* sig, double* vm) {
    const int64_t ne = d.ne();
    const int64_t sx = 1, sy = d.nx + 1, sz = (int64_t)(d.nx + 1) * (d.ny + 1);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        if (!active[e]) {
            if (sig)
                for (int q = 0; q < 6; ++q) sig[6 * e + q] = 0.0;
            if (vm) vm[e] = 0.0;
            continue;
        }
        const int i = (int)(e % d.nx), j = (int)((e / d.nx) % d.ny), k = (int)(e / ((int64_t)d.nx * d.ny));
        const int64_t n0 = d.node(i, j, k);
        double g[3][3] = {};  // g[c][dir]: sum of edge differences of component c along dir
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int a = q & 1, b = q >> 1;
            const int64_t ex = n0 + a * sy + b * sz, ey = n0 + a * sx + b * sz, ez = n0 + a * sx + b * sy;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                g[c][0] += u[3 * (ex + sx) + c] - u[3 * ex + c];
                g[c][1] += u[3 * (ey + sy) + c] - u[3 * ey + c];
                g[c][2] += u[3 * (ez + sz) + c] - u[3 * ez + c];
            }
        }
        const double s = 1.0 / (4.0 * h);
        const double exx = g[0][0] * s, eyy = g[1][1] * s, ezz = g[2][2] * s;
        const double gxy = (g[0][1] + g[1][0]) * s, gyz = (g[1][2] + g[2][1]) * s, gzx = (g[2][0] + g[0][2]) * s;
        const double E = Emat ? Emat[e] : Escalar;
        const double tr = exx + eyy + ezz;
        const double S[6] = {E * (lam * tr + 2 * mu * exx), E * (lam * tr + 2 * mu * eyy), E * (lam * tr + 2 * mu * ezz),
                             E * mu * gxy, E * mu * gyz, E * mu * gzx};
        if (sig)
            for (int q = 0; q < 6; ++q) sig[6 * e + q] = S[q];
        if (vm)
            vm[e] = sqrt(0.5 * ((S[0] - S[1]) * (S[0] - S[1]) + (S[1] - S[2]) * (S[1] - S[2]) + (S[2] - S[0]) * (S[2] - S[0])) +
                         3.0 * (S[3] * S[3] + S[4] * S[4] + S[5] * S[5]));
    }
}

int element_stress(anl_ctx* c, const double* u, const double* Emat, double Escalar, double* sig, double* vm,
                   cudaStream_t s) {
    const double nu = c->nu;
    const double lam = nu / ((1 + nu) * (1 - 2 * nu)), mu = 1.0 / (2 * (1 + nu));
    k_stress<<<dgrid(c->d.ne()), DT, 0, s>>>(c->d, c->active, u, Emat, Escalar, c->h, lam, mu, sig, vm);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int sensitivity(anl_ctx* c, const double* u, int nrhs, const double* coef, const float* xphys, const float* dxp,
                const float* phi, double p, double emin, double E0, float* out, float* dv, bool energy_only,
                cudaStream_t s) {
    if (nrhs < 1 || nrhs > kMaxCases) {
        set_error("sensitivity supports 1..%d load cases, got %d", kMaxCases, nrhs);
        return ANL_ERR_BADARG;
    }
    const int64_t ndof = 3 * c->d.nn();
    ANL_TRY(grow(c->sens_df, c->sens_df_cap, (size_t)nrhs * ndof, sizeof(DF)));
    k_split_pairs<<<dgrid(nrhs * ndof), DT, 0, s>>>(nrhs * ndof, u, c->sens_df);
    ANL_LAUNCH_CHECK();
    SensArgs a{};
    a.d = c->d;
    a.active = c->active;
    a.u = c->sens_df;
    a.nrhs = nrhs;
    a.stride = ndof;
    for (int k = 0; k < nrhs; ++k) a.coef[k] = coef ? (float)coef[k] : 1.f;
    a.xphys = xphys;
    a.dxp = dxp;
    a.phi = phi;
    a.p = (float)p;
    a.emin = (float)emin;
    a.E0 = (float)E0;
    a.h = (float)c->h;
    a.out = out;
    a.dv = energy_only ? nullptr : dv;
    a.energy_only = energy_only ? 1 : 0;
    const int64_t ne = c->d.ne();
    k_sens<<<dgrid(ne), DT, 0, s>>>(a, c->kmf);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

// ------------------------------------------------------------------ OC update

// sums over design (active, non-frozen) elements: -dcx, dvx, count
// a float-pair running sum (TwoSum per term): FP32 instructions only
struct PairSum {
    float h = 0.f, l = 0.f;
    __device__ __forceinline__ void add(float x) {
        float t, e;
        two_sum_f(h, x, t, e);
        h = t;
        l += e;
    }
};
template <int NV>
__device__ __forceinline__ bool finish_pair_sums(const PairSum (&v)[NV], double* partials, unsigned* counter,
                                                 double* out, float2* smem) {
    float h[NV], l[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        h[q] = v[q].h;
        l[q] = v[q].l;
    }
    block_pair_sum<NV, DT>(h, l, smem, threadIdx.x);
    return finish_pair_reduction<NV, DT>(h, l, blockIdx.x, gridDim.x, partials, counter, out, threadIdx.x, smem);
}

__global__ void k_oc_scale(int64_t ne, const uint8_t* active, const uint8_t* frozen, const float* dcx, const float* dvx,
                           double* partials, unsigned* counter, double* out) {
    __shared__ float2 sm[3 * DT / 32];
    PairSum v[3];
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x)
        if (active[e] && !frozen[e]) {
            v[0].add(-dcx[e]);
            v[1].add(dvx[e]);
            v[2].add(1.f);
        }
    finish_pair_sums<3>(v, partials, counter, out, sm);
}

// With no projection the volume is linear in xn: vol = sum_j wv_j xn_j + sum_frozen phi,
// wv = Filter.backward(phi on non-frozen elements). One pass evaluates a bank of up to OC_BANK
// lambdas, the nodes of OC_BANK_DEPTH consecutive bisection steps; each volume is its own
// deterministic two-stage sum, so the bisection takes the decisions a pass per step would.
// The part of each element's update that does not depend on lambda is formed once per OC
// update (k_oc_prep): (s, dvx, lo, hi) and (g, w), with g the value where dvx lambda underflows
// (hi if the element grows, else lo), frozen elements as lo = hi = 1 and inactive ones with w = 0.
// A pass then costs a multiply, a compare, a clamp and a multiply-add per lambda and element.
constexpr int OC_BANK_DEPTH = 4;
constexpr int OC_BANK = (1 << OC_BANK_DEPTH) - 1;
static_assert(OC_BANK <= kMaxRedVals, "one partial per lambda and block");
static_assert(OC_BANK <= 16, "the bank's volumes fit red_out");
struct OcBank {
    float lam[OC_BANK];
    int n;
};

__global__ void k_oc_prep(int64_t ne, const uint8_t* __restrict__ active, const uint8_t* __restrict__ frozen,
                          const float* __restrict__ x, const float* __restrict__ dcx, const float* __restrict__ dvx,
                          const float* __restrict__ wv, float move, float4* __restrict__ el, float2* __restrict__ gw) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        if (!active[e]) {
            el[e] = make_float4(0.f, 1.f, 0.f, 0.f);
            gw[e] = make_float2(0.f, 0.f);
        } else if (frozen[e]) {
            el[e] = make_float4(0.f, 1.f, 1.f, 1.f);
            gw[e] = make_float2(1.f, wv[e]);
        } else {
            const OcElem o = oc_elem(x[e], dcx[e], dvx[e], move);
            el[e] = make_float4(o.s, o.dvx, o.lo, o.hi);
            gw[e] = make_float2(o.grows ? o.hi : o.lo, wv[e]);
        }
    }
}

// One element of the bank pass: adds w * xn(lambda_j) to acc[j] for every lambda of the bank.
// Each thread takes its elements in grid-stride order and adds them per lambda in FP32 in a
// fixed order; blocks and the grid add in float pairs.
// The bisection's state in device memory: the passes, the decisions between them and the final
// update run back to back on the stream with no host round trip (optimize.py:147-160).
struct OcState {
    double lo, hi, lam;
    double vfrozen, vtarget;
    int steps, stop;
    OcBank bank;            // the lambdas of the next pass (FP32, as the passes use them)
    double lamd[OC_BANK];   // the same lambdas in FP64: the decisions' sqrt(lo hi)
};

// The bank of the next OC_BANK_DEPTH (at most 100 - steps) bisection steps from [lo, hi], by one
// warp: level by level of the bisection tree (node j of the in-order numbering), the nodes of a
// level in parallel lanes, so the FP64 square roots (slow on this part) form a chain of `depth`.
// Each node's value is sqrt(l h) of its interval, as the bisection forms it.
__device__ void oc_make_bank(OcState* st, int lane) {
    __shared__ double L[OC_BANK], H[OC_BANK];
    const int depth = min(OC_BANK_DEPTH, 100 - st->steps);
    const int nodes = (1 << depth) - 1, root = (1 << (depth - 1)) - 1;
    if (lane == 0) {
        L[root] = st->lo;
        H[root] = st->hi;
        st->bank.n = nodes;
    }
    __syncwarp();
    for (int level = 0; level < depth; ++level) {
        const int half = 1 << (depth - 1 - level);
        const int j = half - 1 + lane * 2 * half;
        if (lane < (1 << level)) {
            const double t = sqrt(L[j] * H[j]);
            st->lamd[j] = t;
            st->bank.lam[j] = (float)t;
            if (level + 1 < depth) {
                L[j - half / 2] = L[j];
                H[j - half / 2] = t;
                L[j + half / 2] = t;
                H[j + half / 2] = H[j];
            }
        }
        __syncwarp();
    }
}

// one warp
__global__ void k_oc_begin(OcState* st, const double* sums, const double* vfrozen, double vtarget) {
    if (threadIdx.x == 0) {
        // optimize.py:145: the bracket from the mean sensitivities of the design elements
        double scale = 1.0;
        const double nd = sums[2];
        if (nd > 0) {
            const double mdc = sums[0] / nd, mdv = sums[1] / nd;
            scale = fmax(mdc / fmax(mdv, 1e-30), 1e-300);
        }
        st->lo = scale * 1e-8;
        st->hi = scale * 1e8;
        st->lam = sqrt(st->lo * st->hi);
        st->vfrozen = vfrozen ? *vfrozen : 0.0;
        st->vtarget = vtarget;
        st->steps = 0;
        st->stop = 0;
    }
    __syncwarp();
    oc_make_bank(st, threadIdx.x);
}

// one warp: the bank's steps, one per level of the tree (optimize.py:147-160), then the next bank
__global__ void k_oc_decide(OcState* st, const double* vols) {
    if (st->stop) return;  // the same for every lane
    if (threadIdx.x == 0) {
        const int depth = min(OC_BANK_DEPTH, 100 - st->steps);
        int idx = (1 << (depth - 1)) - 1, step = depth >= 2 ? 1 << (depth - 2) : 0;
        double lo = st->lo, hi = st->hi, lam = st->lam;
        for (int d = 0; d < depth; ++d) {
            lam = st->lamd[idx];  // sqrt(lo hi) of the current bracket
            const double vol = vols[idx] + st->vfrozen;
            if (vol > st->vtarget) {
                lo = lam;
                idx += step;
            } else {
                hi = lam;
                idx -= step;
            }
            step >>= 1;
            ++st->steps;
            if (hi / lo < 1 + 1e-9) {
                st->stop = 1;
                break;
            }
        }
        st->lo = lo;
        st->hi = hi;
        st->lam = lam;
        if (st->steps >= 100) st->stop = 1;
    }
    __syncwarp();
    if (!st->stop) oc_make_bank(st, threadIdx.x);
}

constexpr int OCB_T = 512;  // threads of a bank pass: one CTA per SM, each thread ~54 elements at 12.8M DOF
__global__ void __launch_bounds__(OCB_T, 1) k_oc_vol_bank(int64_t ne, const float4* __restrict__ el,
                                                    const float2* __restrict__ gw, const OcState* st,
                                                    double* partials, unsigned* counter, double* out) {
    if (st->stop) return;  // the same for every block
    const OcBank bank = st->bank;
    __shared__ float2 sm[OC_BANK * OCB_T / 32];
    float acc[OC_BANK], rl[OC_BANK];
#pragma unroll
    for (int j = 0; j < OC_BANK; ++j) {
        acc[j] = 0.f;
        rl[j] = oc_rl(bank.lam[j]);
    }
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    constexpr int U = 4;  // elements per trip, their loads issued before any is used
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += U * stride) {
        float4 q[U];
        float2 t[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool in = e + u * stride < ne;
            q[u] = in ? el[e + u * stride] : make_float4(0.f, 1.f, 0.f, 0.f);
            t[u] = in ? gw[e + u * stride] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int j = 0; j < OC_BANK; ++j) {
            if (j < bank.n) {  // oc_xn with the elements' lambda-free parts
                float a = acc[j];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const float v = q[u].y * bank.lam[j] > 1e-30f ? fminf(fmaxf(q[u].x * rl[j], q[u].z), q[u].w)
                                                                   : t[u].x;
                    a = fmaf(t[u].y, v, a);
                }
                acc[j] = a;
            }
        }
    }
    float lo[OC_BANK];
#pragma unroll
    for (int j = 0; j < OC_BANK; ++j) lo[j] = 0.f;
    block_pair_sum<OC_BANK, OCB_T>(acc, lo, sm, threadIdx.x);
    finish_pair_reduction<OC_BANK, OCB_T>(acc, lo, blockIdx.x, gridDim.x, partials, counter, out, threadIdx.x, sm);
}

__global__ void k_oc_weights(int64_t ne, const uint8_t* active, const uint8_t* frozen, const float* phi, float* v,
                             double* partials, unsigned* counter, double* out) {
    __shared__ float2 sm[DT / 32];
    PairSum f[1];
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        const bool a = active[e] != 0, fz = frozen[e] != 0;
        v[e] = a && !fz ? phi[e] : 0.f;
        if (a && fz) f[0].add(phi[e]);
    }
    finish_pair_sums<1>(f, partials, counter, out, sm);
}

__global__ void k_oc_final(int64_t ne, const uint8_t* active, const uint8_t* frozen, const float* x, const float* dcx,
                           const float* dvx, const OcState* st, float move, float* xnew) {
    const float lam = (float)st->lam;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x)
        xnew[e] = active[e] ? (frozen[e] ? 1.f : oc_xn(x[e], dcx[e], dvx[e], lam, move)) : 0.f;
}

static int read_red(anl_ctx* c, int nv, cudaStream_t s) {
    ANL_CUDA(cudaMemcpyAsync(c->red_h, c->red_out, nv * sizeof(double), cudaMemcpyDeviceToHost, s));
    ANL_CUDA(cudaStreamSynchronize(s));
    return ANL_OK;
}

int oc_update(anl_ctx* c, const float* x, const float* dcx, const float* dvx, const float* phi, const uint8_t* frozen,
              double move, double beta, double eta, double vtarget, float* xnew, int* steps_out, double* lam_out,
              cudaStream_t s) {
    const int64_t ne = c->d.ne();
    ANL_TRY(grow(c->oc_state, c->oc_state_cap, 1, sizeof(OcState)));
    OcState* st = reinterpret_cast<OcState*>(c->oc_state);
    k_oc_scale<<<dgrid(ne), DT, 0, s>>>(ne, c->active, frozen, dcx, dvx, c->partials, c->counter, c->red_out);
    ANL_LAUNCH_CHECK();
    const double mv = beta <= 1 ? move : move / 2;  // optimize.py:151
    const bool linear = !(beta > 0);
    if (linear) {
        // With no projection the volume is linear in xn (see k_oc_vol_bank): frozen volume and
        // the filtered weights, the lambda-free element data, then the passes, each followed by
        // its decisions, on the device; one synchronisation at the end
        k_oc_weights<<<dgrid(ne), DT, 0, s>>>(ne, c->active, frozen, phi, c->ftmp2, c->partials, c->counter,
                                              c->red_out + 8);
        ANL_LAUNCH_CHECK();
        k_oc_begin<<<1, 32, 0, s>>>(st, c->red_out, c->red_out + 8, vtarget);
        ANL_LAUNCH_CHECK();
        ANL_TRY(filter_apply(c, false, c->ftmp2, c->ftmp, s));
        ANL_TRY(grow(c->oc_el, c->oc_el_cap, (size_t)ne, sizeof(float4)));
        ANL_TRY(grow(c->oc_gw, c->oc_gw_cap, (size_t)ne, sizeof(float2)));
        k_oc_prep<<<dgrid(ne), DT, 0, s>>>(ne, c->active, frozen, x, dcx, dvx, c->ftmp, (float)mv, c->oc_el,
                                           c->oc_gw);
        ANL_LAUNCH_CHECK();
        // the bracket ratio starts at 1e16 and is square-rooted by every step: 36 steps reach
        // 1 + 1e-9; passes for 40, then more only if the state has not stopped (never seen)
        int passes = (40 + OC_BANK_DEPTH - 1) / OC_BANK_DEPTH;
        static int sms = 0;
        if (sms == 0) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        }
        const int bank_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(sms, (ne + OCB_T - 1) / OCB_T));
        for (int round = 0; round < 100 / OC_BANK_DEPTH + 1; ++round) {
            for (int q = 0; q < passes; ++q) {
                k_oc_vol_bank<<<bank_blocks, OCB_T, 0, s>>>(ne, c->oc_el, c->oc_gw, st, c->partials, c->counter,
                                                            c->red_out);
                ANL_LAUNCH_CHECK();
                k_oc_decide<<<1, 32, 0, s>>>(st, c->red_out);
                ANL_LAUNCH_CHECK();
            }
            ANL_CUDA(cudaMemcpyAsync(c->red_h, st, offsetof(OcState, bank), cudaMemcpyDeviceToHost, s));
            ANL_CUDA(cudaStreamSynchronize(s));
            if (reinterpret_cast<const OcState*>(c->red_h)->stop) break;
            passes = 1;
        }
    } else {
        ANL_TRY(read_red(c, 3, s));
        double scale = 1.0;  // optimize.py:145
        const double nd = c->red_h[2];
        if (nd > 0) {
            const double mdc = c->red_h[0] / nd, mdv = c->red_h[1] / nd;
            scale = std::max(mdc / std::max(mdv, 1e-30), 1e-300);
        }
        double lo = scale * 1e-8, hi = scale * 1e8, lam = std::sqrt(lo * hi);
        int steps = 0;
        for (int k = 0; k < 100; ++k) {  // projected volume: one filter pass per step
            lam = std::sqrt(lo * hi);
            FilterArgs a{};
            a.frozen = frozen;
            a.beta = (float)beta;
            a.eta = (float)eta;
            a.t0 = (float)std::tanh(beta * eta);
            a.t1 = (float)std::tanh(beta * (1 - eta));
            a.x = x;
            a.dcx = dcx;
            a.dvx = dvx;
            a.phi = phi;
            a.lam = (float)lam;
            a.move = (float)mv;
            a.partials = c->partials;
            a.counter = c->counter;
            a.red_out = c->red_out;
            ANL_TRY(launch_filter(c, F_OCVOL, a, s));
            ANL_TRY(read_red(c, 1, s));
            const double vol = c->red_h[0];
            if (vol > vtarget) lo = lam;
            else hi = lam;
            ++steps;
            if (hi / lo < 1 + 1e-9) break;
        }
        OcState* h = reinterpret_cast<OcState*>(c->red_h);  // pinned; its head fields only
        h->lo = lo;
        h->hi = hi;
        h->lam = lam;
        h->vfrozen = 0.0;
        h->vtarget = vtarget;
        h->steps = steps;
        h->stop = 1;
        ANL_CUDA(cudaMemcpyAsync(st, h, offsetof(OcState, bank), cudaMemcpyHostToDevice, s));
        ANL_CUDA(cudaStreamSynchronize(s));
    }
    k_oc_final<<<dgrid(ne), DT, 0, s>>>(ne, c->active, frozen, x, dcx, dvx, st, (float)mv, xnew);
    ANL_LAUNCH_CHECK();
    const OcState& r = *reinterpret_cast<const OcState*>(c->red_h);
    if (steps_out) *steps_out = r.steps;
    if (lam_out) *lam_out = r.lam;
    return ANL_OK;
}

// ------------------------------------------------------------------ history statistics

__global__ void k_stats(int64_t ne, const uint8_t* active, const uint8_t* frozen, const float* xold, const float* xnew,
                        const float* xphys, const float* phi, double* partials, unsigned* counter, double* out) {
    // grey count, design count, volume as float-pair sums; the largest change as a fifth
    // partial (a maximum is exact in any order), carried as the pair (max, 0)
    __shared__ float2 sm[4 * DT / 32];
    __shared__ float smax[DT / 32];
    __shared__ bool last;
    PairSum v[3];
    float mx = 0.f;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        if (!active[e]) continue;
        const float xp = xphys[e];
        float pv, pe;
        two_prod(phi[e], xp, pv, pe);  // the exact product as a pair
        v[2].add(pv);
        v[2].add(pe);
        if (!frozen[e]) {
            mx = fmaxf(mx, fabsf(xnew[e] - xold[e]));
            if (xp > 0.1f && xp < 0.9f) v[0].add(1.f);
            v[1].add(1.f);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if (lane == 0) smax[warp] = mx;
    float h[3], l[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        h[q] = v[q].h;
        l[q] = v[q].l;
    }
    block_pair_sum<3, DT>(h, l, sm, threadIdx.x);  // its barrier also publishes smax
    float2* p = reinterpret_cast<float2*>(partials);
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int w = 0; w < DT / 32; ++w) m = fmaxf(m, smax[w]);
        for (int q = 0; q < 3; ++q) p[(int64_t)blockIdx.x * 4 + q] = make_float2(h[q], l[q]);
        p[(int64_t)blockIdx.x * 4 + 3] = make_float2(m, 0.f);
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    float m = 0.f;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        h[q] = 0.f;
        l[q] = 0.f;
    }
    for (unsigned b = threadIdx.x; b < gridDim.x; b += DT) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float2 x = __ldcg(p + (int64_t)b * 4 + q);
            float t, e;
            two_sum_f(h[q], x.x, t, e);
            h[q] = t;
            l[q] += x.y + e;
        }
        m = fmaxf(m, __ldcg(p + (int64_t)b * 4 + 3).x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    __syncthreads();
    if (lane == 0) smax[warp] = m;
    block_pair_sum<3, DT>(h, l, sm, threadIdx.x);
    if (threadIdx.x == 0) {
        float mm = 0.f;
        for (int w = 0; w < DT / 32; ++w) mm = fmaxf(mm, smax[w]);
        double r[3];
        for (int q = 0; q < 3; ++q) r[q] = (double)h[q] + (double)l[q];
        // change, grey fraction of the design elements, volume, design element count
        out[0] = mm;
        out[1] = r[1] > 0 ? r[0] / r[1] : 0.0;
        out[2] = r[2];
        out[3] = r[1];
        *counter = 0u;
    }
}

int design_stats(anl_ctx* c, const float* xold, const float* xnew, const float* xphys, const float* phi,
                 const uint8_t* frozen, double* out, cudaStream_t s) {
    const int64_t ne = c->d.ne();
    k_stats<<<dgrid(ne), DT, 0, s>>>(ne, c->active, frozen, xold, xnew, xphys, phi, c->partials, c->counter, c->red_out);
    ANL_LAUNCH_CHECK();
    ANL_TRY(read_red(c, 4, s));
    for (int q = 0; q < 4; ++q) out[q] = c->red_h[q];
    return ANL_OK;
}

ANL_DEBUG_UNIT(design)

}  // namespace anl
