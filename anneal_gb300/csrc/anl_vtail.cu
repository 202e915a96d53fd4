// anl_vtail.cu -- the smallest levels of the V-cycle in one CTA, entirely in shared memory.
//
// Below about a thousand elements a multigrid level is pure latency: each of its ~17 passes per
// V-cycle (8 + 8 Chebyshev steps, the residual, the grid transfers) is a launch that moves a few
// kilobytes. Here one CTA of 1024 threads takes the right-hand side of the first such level and
// returns its V-cycle correction: it smooths, restricts, solves the coarsest grid with the dense
// inverse (kept as float pairs), prolongs and smooths back up, with only __syncthreads between
// the steps. The arithmetic is that of the per-level kernels: the modal element product
// (modal_element), Chebyshev on D^-1 K with the level's coefficients, trilinear transfers,
// masks on fixed DOFs.
//
// K x on a level: one thread per element (at most 1024 elements) forms its 8 corner forces,
// then 8 passes (one per corner octant, a barrier each) add them onto the nodes: within a pass
// no two elements share a node, so the sum needs no atomics and has a fixed order.
#include "anl_common.cuh"
#include "anl_kernels.cuh"

namespace anl {

namespace {

constexpr int TT = 1024;  // threads

// shared-memory carve-up of the tail (floats; node masks as bytes, padded to 4)
struct TailLayout {
    int off_x[kTailMaxLevels], off_b[kTailMaxLevels], off_d[kTailMaxLevels], off_y[kTailMaxLevels];
    int off_e[kTailMaxLevels], off_g[kTailMaxLevels], off_m[kTailMaxLevels];
    int floats;
};

__host__ __device__ inline TailLayout tail_layout(const TailLevel* lev, int nlev) {
    TailLayout t{};
    int o = 0;
    for (int l = 0; l < nlev; ++l) {
        const int nn = (int)lev[l].d.nn(), ne = (int)lev[l].d.ne();
        const bool coarsest = l == nlev - 1;
        t.off_x[l] = o;
        o += 3 * nn;
        t.off_b[l] = o;
        o += 3 * nn;
        t.off_d[l] = t.off_y[l] = t.off_e[l] = t.off_g[l] = -1;
        if (!coarsest) {
            t.off_d[l] = o;
            o += 3 * nn;
            t.off_y[l] = o;
            o += 3 * nn;
            t.off_e[l] = o;
            o += ne;
            t.off_g[l] = o;
            o += nn;
        }
        t.off_m[l] = o;
        o += (nn + 3) / 4;
    }
    t.floats = o;
    return t;
}

struct TailCtx {
    const TailArgs& a;
    const TailLayout& L;
    float* sm;
    int tid;
    __device__ float* X(int l) const { return sm + L.off_x[l]; }
    __device__ float* B(int l) const { return sm + L.off_b[l]; }
    __device__ float* Dv(int l) const { return sm + L.off_d[l]; }
    __device__ float* Y(int l) const { return sm + L.off_y[l]; }
    __device__ float* E(int l) const { return sm + L.off_e[l]; }
    __device__ float* G(int l) const { return sm + L.off_g[l]; }
    __device__ uint8_t* M(int l) const { return reinterpret_cast<uint8_t*>(sm + L.off_m[l]); }

    // Y = K X on level l
    __device__ void apply(int l) const {
        const Dims d = a.lev[l].d;
        const int nn = (int)d.nn(), ne = (int)d.ne();
        float* y = Y(l);
        const float* x = X(l);
        for (int q = tid; q < 3 * nn; q += TT) y[q] = 0.f;
        V3<float> f[2][2][2];
        int n0 = 0;
        const int e = tid;
        if (e < ne) {
            const int i = e % d.nx, j = (e / d.nx) % d.ny, k = e / (d.nx * d.ny);
            n0 = (int)d.node(i, j, k);
            const float Ee = E(l)[e];
            if (Ee != 0.f) {
                const int sy = d.nx + 1, sz = (d.nx + 1) * (d.ny + 1);
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
                modal_element<float>(a.km, Ee, dxb, dxt, dyb, dyt, dz, f);
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) (&f[0][0][0])[q] = v3zero<float>();
            }
        }
        __syncthreads();  // y is zero
        const int sy = d.nx + 1, sz = (d.nx + 1) * (d.ny + 1);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int px = q & 1, py = (q >> 1) & 1, pz = q >> 2;
            if (e < ne) {
                float* p = y + 3 * (n0 + px + py * sy + pz * sz);
                const V3<float>& v = f[px][py][pz];
                p[0] += v.xy.x;
                p[1] += v.xy.y;
                p[2] += v.z;
            }
            __syncthreads();
        }
    }

    // `deg` Chebyshev steps on level l (from x = 0 when `from_zero`)
    __device__ void smooth(int l, int deg, bool from_zero) const {
        const Dims d = a.lev[l].d;
        const int nn = (int)d.nn();
        const double* cf = a.lev[l].cheb;
        float* x = X(l);
        float* dv = Dv(l);
        const float* b = B(l);
        const float* g = G(l);
        const uint8_t* m = M(l);
        int k0 = 0;
        if (from_zero) {  // step 0: x = d = c2_0 D^-1 b
            const float c2 = (float)cf[1];
            for (int q = tid; q < 3 * nn; q += TT) {
                const int n = q / 3, c = q - 3 * n;
                const float v = (m[n] >> c) & 1 ? c2 * g[n] * b[q] : 0.f;
                x[q] = v;
                dv[q] = v;
            }
            __syncthreads();
            k0 = 1;
        }
        for (int k = k0; k < deg; ++k) {
            apply(l);
            const float c1 = (k == 0) ? 0.f : (float)cf[2 * k], c2 = (float)cf[2 * k + 1];
            const float* y = Y(l);
            for (int q = tid; q < 3 * nn; q += TT) {
                const int n = q / 3, c = q - 3 * n;
                if ((m[n] >> c) & 1) {
                    const float dn = c1 * dv[q] + c2 * (b[q] - y[q]) * g[n];
                    dv[q] = dn;
                    x[q] += dn;
                }
            }
            __syncthreads();
        }
    }

    // Y(l) = b - K x (masked): the residual restricted to level l + 1
    __device__ void residual(int l) const {
        apply(l);
        const int nn = (int)a.lev[l].d.nn();
        float* y = Y(l);
        const float* b = B(l);
        const uint8_t* m = M(l);
        for (int q = tid; q < 3 * nn; q += TT) {
            const int n = q / 3, c = q - 3 * n;
            y[q] = (m[n] >> c) & 1 ? b[q] - y[q] : 0.f;
        }
        __syncthreads();
    }

    // B(l + 1) = P^T Y(l): trilinear weights 1, 1/2, 1/4, 1/8, zero on fixed coarse DOFs
    __device__ void restrict_to(int l) const {
        const Dims f = a.lev[l].d, c = a.lev[l + 1].d;
        const float* r = Y(l);
        float* bc = B(l + 1);
        const uint8_t* mc = M(l + 1);
        const int cnn = (int)c.nn();
        for (int N = tid; N < cnn; N += TT) {
            const int I = N % (c.nx + 1), J = (N / (c.nx + 1)) % (c.ny + 1), K = N / ((c.nx + 1) * (c.ny + 1));
            float acc[3] = {0.f, 0.f, 0.f};
            for (int dk = -1; dk <= 1; ++dk) {
                const int k = 2 * K + dk;
                if (k < 0 || k > f.nz) continue;
                const float wk = dk == 0 ? 1.f : 0.5f;
                for (int dj = -1; dj <= 1; ++dj) {
                    const int j = 2 * J + dj;
                    if (j < 0 || j > f.ny) continue;
                    const float wj = dj == 0 ? wk : 0.5f * wk;
                    for (int di = -1; di <= 1; ++di) {
                        const int i = 2 * I + di;
                        if (i < 0 || i > f.nx) continue;
                        const float w = di == 0 ? wj : 0.5f * wj;
                        const float* p = r + 3 * f.node(i, j, k);
                        acc[0] += w * p[0];
                        acc[1] += w * p[1];
                        acc[2] += w * p[2];
                    }
                }
            }
            const uint8_t m = mc[N];
#pragma unroll
            for (int q = 0; q < 3; ++q) bc[3 * N + q] = (m >> q) & 1 ? acc[q] : 0.f;
        }
        __syncthreads();
    }

    // X(l) += P X(l + 1) on free fine DOFs
    __device__ void prolong_add(int l) const {
        const Dims f = a.lev[l].d, c = a.lev[l + 1].d;
        const float* xc = X(l + 1);
        float* xf = X(l);
        const uint8_t* mf = M(l);
        const int fnn = (int)f.nn();
        for (int n = tid; n < fnn; n += TT) {
            const uint8_t m = mf[n];
            if (!(m & 7)) continue;
            const int i = n % (f.nx + 1), j = (n / (f.nx + 1)) % (f.ny + 1), k = n / ((f.nx + 1) * (f.ny + 1));
            const int I = i >> 1, J = j >> 1, K = k >> 1, di = i & 1, dj = j & 1, dk = k & 1;
            const float w = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f) * (dk ? 0.5f : 1.f);
            float acc[3] = {0.f, 0.f, 0.f};
            for (int g = 0; g <= dk; ++g)
                for (int bb = 0; bb <= dj; ++bb)
                    for (int aa = 0; aa <= di; ++aa) {
                        const float* p = xc + 3 * c.node(I + aa, J + bb, K + g);
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

    // X(L) = A^-1 B(L) on the coarsest grid: the inverse as float pairs (symmetric, so thread
    // `row` reads column `row` for coalesced loads), compensated FP32 accumulation
    __device__ void coarse_solve(int l) const {
        const int n = a.nc;
        const float* b = B(l);
        float* x = X(l);
        const uint8_t* m = M(l);
        for (int row = tid; row < n; row += TT) {
            Acc2 acc;
            for (int c = 0; c < n; ++c) {
                const float bc = b[c];
                acc.add_prod(__ldg(a.ainv_hi + (int64_t)c * n + row), bc);
                acc.add_prod(__ldg(a.ainv_lo + (int64_t)c * n + row), bc);
            }
            x[row] = (m[row / 3] >> (row % 3)) & 1 ? acc.s + acc.c : 0.f;
        }
        __syncthreads();
    }
};

__global__ void __launch_bounds__(TT, 1) k_vtail(TailArgs a) {
    if (a.done != nullptr && *a.done) return;
    extern __shared__ __align__(16) float tail_smem[];
    const TailLayout L = tail_layout(a.lev, a.nlev);
    const TailCtx t{a, L, tail_smem, (int)threadIdx.x};
    const int tid = threadIdx.x;
    // the levels' element scales, inverse diagonals and masks, and the first level's b
    for (int l = 0; l < a.nlev; ++l) {
        const TailLevel& lv = a.lev[l];
        const int nn = (int)lv.d.nn(), ne = (int)lv.d.ne();
        for (int q = tid; q < nn; q += TT) t.M(l)[q] = lv.nmask[q];
        if (l < a.nlev - 1) {
            for (int q = tid; q < ne; q += TT) t.E(l)[q] = lv.E[q];
            for (int q = tid; q < nn; q += TT) t.G(l)[q] = lv.diag[q];
        }
    }
    {
        const int nn = (int)a.lev[0].d.nn();
        for (int q = tid; q < 3 * nn; q += TT) t.B(0)[q] = a.b0[q];
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
    const int nn = (int)a.lev[0].d.nn();
    for (int q = tid; q < 3 * nn; q += TT) a.x0[q] = t.X(0)[q];
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

size_t tail_smem_bytes(const TailLevel* lev, int nlev) { return sizeof(float) * (size_t)tail_layout(lev, nlev).floats; }

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
    if (bytes > (size_t)kTailMaxSmem || a.lev[0].d.ne() > TT) {
        set_error("V-cycle tail: %zu bytes of shared memory or %lld elements exceed one CTA", bytes,
                  (long long)a.lev[0].d.ne());
        return ANL_ERR_BADARG;
    }
    k_vtail<<<1, TT, bytes, s>>>(a);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int launch_ainv_split(const double* ainv, int n, float* hi, float* lo, cudaStream_t s) {
    const int64_t n2 = (int64_t)n * n;
    k_ainv_split<<<(int)std::min<int64_t>(1024, (n2 + 255) / 256), 256, 0, s>>>(ainv, n2, hi, lo);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

}  // namespace anl
