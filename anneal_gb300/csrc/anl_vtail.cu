// anl_vtail.cu -- the smallest levels of the V-cycle in one CTA, entirely in shared memory.
//
// Below about a thousand elements a multigrid level is pure latency: each of its ~17 passes per
// V-cycle (8 + 8 Chebyshev steps, the residual, the grid transfers) is a launch that moves a few
// kilobytes. Here one CTA takes the right-hand side of the first such level and returns its
// V-cycle correction: it smooths, restricts, solves the coarsest grid with the dense inverse
// (kept as float pairs), prolongs and smooths back up, with only __syncthreads between the
// steps. The arithmetic is that of the per-level kernels: the modal element product
// (modal_element), Chebyshev on D^-1 K with the level's coefficients, trilinear transfers,
// masks on fixed DOFs.
//
// K x on a level is two phases with one barrier after each: every element writes its 8 corner
// forces to shared memory (structure of arrays, corner-component major), then every node sums
// the corners of its up to 8 elements in a fixed order and applies its Chebyshev update (or
// forms its residual) in the same pass. Node coordinates and element corner nodes come from
// per-level tables built once per launch, so the steps do no integer division.
#include "anl_common.cuh"
#include "anl_kernels.cuh"

namespace anl {

namespace {

constexpr int TT = 1024;  // threads: one element each on a 1,024-element level

// shared-memory carve-up of the tail, in 4-byte words (floats; int tables; node masks as bytes
// padded to 4): per level x, b (and on the smoothed levels the direction / residual dv, the
// inverse diagonal g, E, the packed node coordinates and the elements' first nodes), then one
// element-force array for the largest smoothed level
struct TailLayout {
    int off_x[kTailMaxLevels], off_b[kTailMaxLevels], off_d[kTailMaxLevels], off_g[kTailMaxLevels];
    int off_e[kTailMaxLevels], off_n[kTailMaxLevels], off_e0[kTailMaxLevels], off_m[kTailMaxLevels];
    int off_f;
    int words;
};

__host__ __device__ inline TailLayout tail_layout(const TailLevel* lev, int nlev) {
    TailLayout t{};
    int o = 0, max_ne = 0;
    for (int l = 0; l < nlev; ++l) {
        const int nn = (int)lev[l].d.nn(), ne = (int)lev[l].d.ne();
        const bool coarsest = l == nlev - 1;
        t.off_x[l] = o;
        o += 3 * nn;
        t.off_b[l] = o;
        o += 3 * nn;
        t.off_d[l] = t.off_g[l] = t.off_e[l] = t.off_n[l] = t.off_e0[l] = -1;
        if (!coarsest) {
            t.off_d[l] = o;
            o += 3 * nn;
            t.off_g[l] = o;
            o += nn;
            t.off_e[l] = o;
            o += ne;
            t.off_n[l] = o;
            o += nn;
            t.off_e0[l] = o;
            o += ne;
            max_ne = max_ne > ne ? max_ne : ne;
        }
        t.off_m[l] = o;
        o += (nn + 3) / 4;
    }
    t.off_f = o;
    o += 24 * max_ne;
    t.words = o;
    return t;
}

// packed node coordinates (i, j, k < 2048, 2048, 1024)
__device__ __forceinline__ int pack_ijk(int i, int j, int k) { return i | (j << 11) | (k << 22); }

// Everything a step indexes by level at run time (the levels, the carve-up) lives in shared
// memory; a reference to the kernel's parameter would copy it to local memory.
constexpr int kTailMaxDegree = 16;  // Chebyshev steps per sweep the tail holds coefficients for

struct TailCtx {
    const TailLevel* lev;  // shared-memory copy of the levels
    const TailLayout& L;   // in shared memory
    const float (*cheb)[2 * kTailMaxDegree];  // per level (c1, c2) of each step, in shared memory
    float* sm;
    int tid;
    KeModal<float> km;
    const float* ainv_hi;
    const float* ainv_lo;
    int nc;
    __device__ float* X(int l) const { return sm + L.off_x[l]; }
    __device__ float* B(int l) const { return sm + L.off_b[l]; }
    __device__ float* Dv(int l) const { return sm + L.off_d[l]; }
    __device__ float* G(int l) const { return sm + L.off_g[l]; }
    __device__ float* E(int l) const { return sm + L.off_e[l]; }
    __device__ int* Nijk(int l) const { return reinterpret_cast<int*>(sm + L.off_n[l]); }
    __device__ int* E0(int l) const { return reinterpret_cast<int*>(sm + L.off_e0[l]); }
    __device__ uint8_t* M(int l) const { return reinterpret_cast<uint8_t*>(sm + L.off_m[l]); }
    __device__ float* F() const { return sm + L.off_f; }

    // phase 1 of K x on level l: the corner forces of every element into F (corner q = px +
    // 2 py + 4 pz, component c at F[(3 q + c) ne + e]); ends with a barrier
    __device__ void element_forces(int l) const {
        const Dims d = lev[l].d;
        const int ne = (int)d.ne();
        const int sy = d.nx + 1, sz = (d.nx + 1) * (d.ny + 1);
        const float* x = X(l);
        const float* Ev = E(l);
        const int* e0 = E0(l);
        float* F_ = F();
        for (int e = tid; e < ne; e += TT) {
            const float Ee = Ev[e];
            V3<float> f[2][2][2];
            if (Ee != 0.f) {
                const int n0 = e0[e];
                V3<float> u[2][2][2];
#pragma unroll
                for (int pz = 0; pz < 2; ++pz)
#pragma unroll
                    for (int py = 0; py < 2; ++py)
#pragma unroll
                        for (int px = 0; px < 2; ++px) {
                            const float* p = x + 3 * (n0 + px + py * sy + pz * sz);
                            u[px][py][pz].xy = make_float2(p[0], p[1]);
                            u[px][py][pz].z = p[2];
                        }
                V3<float> dxb[2], dxt[2], dyb[2], dyt[2], dz[2][2];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    dxb[q] = u[1][q][0] - u[0][q][0];
                    dxt[q] = u[1][q][1] - u[0][q][1];
                    dyb[q] = u[q][1][0] - u[q][0][0];
                    dyt[q] = u[q][1][1] - u[q][0][1];
                }
#pragma unroll
                for (int px = 0; px < 2; ++px)
#pragma unroll
                    for (int py = 0; py < 2; ++py) dz[px][py] = u[px][py][1] - u[px][py][0];
                modal_element<float>(km, Ee, dxb, dxt, dyb, dyt, dz, f);
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) (&f[0][0][0])[q] = v3zero<float>();
            }
#pragma unroll
            for (int pz = 0; pz < 2; ++pz)
#pragma unroll
                for (int py = 0; py < 2; ++py)
#pragma unroll
                    for (int px = 0; px < 2; ++px) {
                        const int q = px + 2 * py + 4 * pz;
                        F_[(3 * q) * ne + e] = f[px][py][pz].xy.x;
                        F_[(3 * q + 1) * ne + e] = f[px][py][pz].xy.y;
                        F_[(3 * q + 2) * ne + e] = f[px][py][pz].z;
                    }
        }
        __syncthreads();
    }

    // phase 2: (K x)(n), the corners of node n's elements summed in a fixed order
    __device__ __forceinline__ void node_force(int l, int n, float (&y)[3]) const {
        const Dims d = lev[l].d;
        const int ne = (int)d.ne();
        const int pk = Nijk(l)[n];
        const int i = pk & 2047, j = (pk >> 11) & 2047, k = pk >> 22;
        const float* F_ = F();
        y[0] = y[1] = y[2] = 0.f;
#pragma unroll
        for (int pz = 0; pz < 2; ++pz) {
            const int ke = k - pz;
            if (ke < 0 || ke >= d.nz) continue;
#pragma unroll
            for (int py = 0; py < 2; ++py) {
                const int je = j - py;
                if (je < 0 || je >= d.ny) continue;
#pragma unroll
                for (int px = 0; px < 2; ++px) {
                    const int ie = i - px;
                    if (ie < 0 || ie >= d.nx) continue;
                    const int e = ie + d.nx * (je + d.ny * ke);
                    const int q = px + 2 * py + 4 * pz;
                    y[0] += F_[(3 * q) * ne + e];
                    y[1] += F_[(3 * q + 1) * ne + e];
                    y[2] += F_[(3 * q + 2) * ne + e];
                }
            }
        }
    }

    // `deg` Chebyshev steps on level l (from x = 0 when `from_zero`)
    __device__ void smooth(int l, int deg, bool from_zero) const {
        const int nn = (int)lev[l].d.nn();
        const float* cf = cheb[l];
        float* x = X(l);
        float* dv = Dv(l);
        const float* b = B(l);
        const float* g = G(l);
        const uint8_t* m = M(l);
        int k0 = 0;
        if (from_zero) {  // step 0: x = d = c2_0 D^-1 b
            const float c2 = cf[1];
            for (int n = tid; n < nn; n += TT) {
                const uint8_t mn = m[n];
                const float gn = c2 * g[n];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float v = (mn >> c) & 1 ? gn * b[3 * n + c] : 0.f;
                    x[3 * n + c] = v;
                    dv[3 * n + c] = v;
                }
            }
            __syncthreads();
            k0 = 1;
        }
        for (int k = k0; k < deg; ++k) {
            element_forces(l);
            const float c1 = (k == 0) ? 0.f : cf[2 * k], c2 = cf[2 * k + 1];
            for (int n = tid; n < nn; n += TT) {
                const uint8_t mn = m[n];
                if (!(mn & 7)) continue;
                float y[3];
                node_force(l, n, y);
                const float gn = c2 * g[n];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    if ((mn >> c) & 1) {
                        const int q = 3 * n + c;
                        const float dn = c1 * dv[q] + (b[q] - y[c]) * gn;
                        dv[q] = dn;
                        x[q] += dn;
                    }
                }
            }
            __syncthreads();
        }
    }

    // Dv(l) = b - K x (masked): the residual restricted to level l + 1 (the post-smoothing's
    // first step does not read the direction)
    __device__ void residual(int l) const {
        element_forces(l);
        const int nn = (int)lev[l].d.nn();
        float* r = Dv(l);
        const float* b = B(l);
        const uint8_t* m = M(l);
        for (int n = tid; n < nn; n += TT) {
            const uint8_t mn = m[n];
            float y[3] = {0.f, 0.f, 0.f};
            if (mn & 7) node_force(l, n, y);
#pragma unroll
            for (int c = 0; c < 3; ++c) r[3 * n + c] = (mn >> c) & 1 ? b[3 * n + c] - y[c] : 0.f;
        }
        __syncthreads();
    }

    // B(l + 1) = P^T Dv(l): trilinear weights 1, 1/2, 1/4, 1/8, zero on fixed coarse DOFs
    __device__ void restrict_to(int l) const {
        const Dims f = lev[l].d, c = lev[l + 1].d;
        const float* r = Dv(l);
        float* bc = B(l + 1);
        const uint8_t* mc = M(l + 1);
        const int cnn = (int)c.nn();
        const int fsy = f.nx + 1, fsz = (f.nx + 1) * (f.ny + 1);
        const int cx = c.nx + 1, cxy = (c.nx + 1) * (c.ny + 1);
        for (int N = tid; N < cnn; N += TT) {
            const uint8_t m = mc[N];
            if (!(m & 7)) {
                bc[3 * N] = bc[3 * N + 1] = bc[3 * N + 2] = 0.f;
                continue;
            }
            const int K = N / cxy, J = (N - K * cxy) / cx, I = N - K * cxy - J * cx;
            float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int dk = -1; dk <= 1; ++dk) {
                const int k = 2 * K + dk;
                if (k < 0 || k > f.nz) continue;
                const float wk = dk == 0 ? 1.f : 0.5f;
#pragma unroll
                for (int dj = -1; dj <= 1; ++dj) {
                    const int j = 2 * J + dj;
                    if (j < 0 || j > f.ny) continue;
                    const float wj = dj == 0 ? wk : 0.5f * wk;
#pragma unroll
                    for (int di = -1; di <= 1; ++di) {
                        const int i = 2 * I + di;
                        if (i < 0 || i > f.nx) continue;
                        const float w = di == 0 ? wj : 0.5f * wj;
                        const float* p = r + 3 * (i + fsy * j + fsz * k);
                        acc[0] += w * p[0];
                        acc[1] += w * p[1];
                        acc[2] += w * p[2];
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 3; ++q) bc[3 * N + q] = (m >> q) & 1 ? acc[q] : 0.f;
        }
        __syncthreads();
    }

    // X(l) += P X(l + 1) on free fine DOFs
    __device__ void prolong_add(int l) const {
        const Dims f = lev[l].d, c = lev[l + 1].d;
        const float* xc = X(l + 1);
        float* xf = X(l);
        const uint8_t* mf = M(l);
        const int* nijk = Nijk(l);
        const int fnn = (int)f.nn();
        const int csy = c.nx + 1, csz = (c.nx + 1) * (c.ny + 1);
        for (int n = tid; n < fnn; n += TT) {
            const uint8_t m = mf[n];
            if (!(m & 7)) continue;
            const int pk = nijk[n];
            const int i = pk & 2047, j = (pk >> 11) & 2047, k = pk >> 22;
            const int I = i >> 1, J = j >> 1, K = k >> 1, di = i & 1, dj = j & 1, dk = k & 1;
            const float w = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f) * (dk ? 0.5f : 1.f);
            float acc[3] = {0.f, 0.f, 0.f};
            for (int g = 0; g <= dk; ++g)
                for (int bb = 0; bb <= dj; ++bb)
                    for (int aa = 0; aa <= di; ++aa) {
                        const float* p = xc + 3 * ((I + aa) + csy * (J + bb) + csz * (K + g));
                        acc[0] += p[0];
                        acc[1] += p[1];
                        acc[2] += p[2];
                    }
#pragma unroll
            for (int q = 0; q < 3; ++q)
                if ((m >> q) & 1) xf[3 * n + q] += w * acc[q];
        }
        __syncthreads();
    }

    // X(L) = A^-1 B(L) on the coarsest grid: the inverse as float pairs, one warp per row (the
    // inverse is symmetric: lane t reads entries t, t + 32, ... of column `row`), compensated
    // FP32 accumulation, the lanes' pairs added in a fixed tree
    __device__ void coarse_solve(int l) const {
        const int n = nc;
        const float* b = B(l);
        float* x = X(l);
        const uint8_t* m = M(l);
        const int lane = tid & 31, warp = tid >> 5;
        for (int row = warp; row < n; row += TT / 32) {
            Acc2 acc;
            const float* hi = ainv_hi + (int64_t)row * n;
            const float* lo = ainv_lo + (int64_t)row * n;
            for (int c = lane; c < n; c += 32) {
                if (!ANL_IN_RANGE((int64_t)row * n + c, (int64_t)n * n)) break;
                const float bc = b[c];
                acc.add_prod(__ldg(hi + c), bc);
                acc.add_prod(__ldg(lo + c), bc);
            }
            float s = acc.s, e = acc.c;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float s2 = __shfl_down_sync(0xffffffffu, s, o), e2 = __shfl_down_sync(0xffffffffu, e, o);
                float t, f;
                two_sum(s, s2, t, f);
                s = t;
                e += e2 + f;
            }
            if (lane == 0) x[row] = (m[row / 3] >> (row % 3)) & 1 ? s + e : 0.f;
        }
        __syncthreads();
    }
};

__global__ void __launch_bounds__(TT, 1) k_vtail(TailArgs a) {
    const int slot = blockIdx.x;
    const int* done = slot_bytes(a.done, slot, a.sc_bytes);
    if (done != nullptr && *done) return;
    const float* b0 = slot_ptr(a.b0, slot, a.vstride);
    float* x0 = slot_ptr(a.x0, slot, a.vstride);
    extern __shared__ __align__(16) float tail_smem[];
    __shared__ TailLevel slev[kTailMaxLevels];
    const int tid = threadIdx.x;
#pragma unroll
    for (int q = 0; q < kTailMaxLevels; ++q)  // static indices: the parameter stays in its bank
        if (tid == q) slev[q] = a.lev[q];
    __shared__ TailLayout sL;
    __shared__ float scheb[kTailMaxLevels][2 * kTailMaxDegree];
    __syncthreads();
    if (tid == 0) sL = tail_layout(slev, a.nlev);
    {  // the sweeps' coefficients: a dependent global load per step otherwise
        const int l = tid / (2 * kTailMaxDegree), q = tid % (2 * kTailMaxDegree);
        if (l < a.nlev - 1 && q < 2 * a.degree) scheb[l][q] = (float)slev[l].cheb[q];
    }
    __syncthreads();
    const TailCtx t{slev, sL, scheb, tail_smem, tid, a.km, a.ainv_hi, a.ainv_lo, a.nc};
    // the levels' element scales, inverse diagonals, masks and index tables, and the first
    // level's b
    for (int l = 0; l < a.nlev; ++l) {
        const TailLevel& lv = slev[l];
        const Dims d = lv.d;
        const int nn = (int)d.nn(), ne = (int)d.ne();
        for (int q = tid; q < nn; q += TT) t.M(l)[q] = lv.nmask[q];
        if (l < a.nlev - 1) {
            for (int q = tid; q < ne; q += TT) {
                t.E(l)[q] = lv.E[q];
                const int i = q % d.nx, j = (q / d.nx) % d.ny, k = q / (d.nx * d.ny);
                t.E0(l)[q] = (int)d.node(i, j, k);
            }
            for (int q = tid; q < nn; q += TT) {
                t.G(l)[q] = lv.diag[q];
                const int i = q % (d.nx + 1), j = (q / (d.nx + 1)) % (d.ny + 1), k = q / ((d.nx + 1) * (d.ny + 1));
                t.Nijk(l)[q] = pack_ijk(i, j, k);
            }
        }
    }
    {
        const int nn = (int)slev[0].d.nn();
        for (int q = tid; q < 3 * nn; q += TT) t.B(0)[q] = b0[q];
    }
    __syncthreads();
    const int last = a.nlev - 1;
    for (int l = 0; l < last; ++l) {
        t.smooth(l, a.degree, true);
        t.residual(l);
        t.restrict_to(l);
    }
    t.coarse_solve(last);
    for (int l = last - 1; l >= 0; --l) {
        t.prolong_add(l);
        t.smooth(l, a.degree, false);
    }
    const int nn = (int)slev[0].d.nn();
    for (int q = tid; q < 3 * nn; q += TT) x0[q] = t.X(0)[q];
}

__global__ void k_ainv_split(const double* ainv, int64_t n2, float* hi, float* lo) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n2; q += (int64_t)gridDim.x * blockDim.x) {
        float h, l;
        split_double(ainv[q], h, l);
        hi[q] = h;
        lo[q] = l;
    }
}

}  // namespace

size_t tail_smem_bytes(const TailLevel* lev, int nlev) { return sizeof(float) * (size_t)tail_layout(lev, nlev).words; }

int vtail_prepare() {
    static bool done = false;
    if (!done) {
        ANL_CUDA(cudaFuncSetAttribute(k_vtail, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailMaxSmem));
        done = true;
    }
    return ANL_OK;
}

int launch_vtail(const TailArgs& a, cudaStream_t s) {
    const size_t bytes = tail_smem_bytes(a.lev, a.nlev);
    if (a.degree > kTailMaxDegree || a.nlev > kTailMaxLevels || bytes > (size_t)kTailMaxSmem || a.lev[0].d.ne() > 1024 || a.lev[0].d.nx > 2047 || a.lev[0].d.ny > 2047 ||
        a.lev[0].d.nz > 1023) {
        set_error("V-cycle tail: %zu bytes of shared memory or %lld elements exceed one CTA", bytes,
                  (long long)a.lev[0].d.ne());
        return ANL_ERR_BADARG;
    }
    k_vtail<<<std::max(1, a.nrhs), TT, bytes, s>>>(a);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int launch_ainv_split(const double* ainv, int n, float* hi, float* lo, cudaStream_t s) {
    const int64_t n2 = (int64_t)n * n;
    k_ainv_split<<<(int)std::min<int64_t>(1024, (n2 + 255) / 256), 256, 0, s>>>(ainv, n2, hi, lo);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

ANL_DEBUG_UNIT(vtail)

}  // namespace anl
