// anl_solver.cu -- geometric-multigrid preconditioned CG on the voxel grid.
//
// Replaces FEM.solve (fem.py:206-232): scipy CG with a pyamg smoothed-aggregation V-cycle
// on the assembled matrix. Here:
//  * the operator is the matrix-free K u of anl_ku.cu (FP32, or FP64 with ANL_FLAG_FP64);
//  * the preconditioner is a V-cycle on the voxel hierarchy (element dims halved per level):
//    coarse element scale = (sum of the 8 children)/4 (their mean at Ke(2h) = 2 Ke(h)),
//    trilinear prolongation P and restriction P^T, Chebyshev smoothing on D^-1 K below the
//    element bound lambda_max(Ke) / Ke_00 (an upper bound of the spectrum for every design):
//    2 steps over [0.03, 1] x bound on levels 0-1, 8 steps over [0.002, 1] x bound on the
//    latency-bound levels below; a dense FP64 Cholesky solve on the coarsest grid, refactored
//    every solve (a high-degree Chebyshev sweep if that grid is too large for a dense factor);
//  * the CG iterate x and right-hand side stay in FP64; the CG scalars come from FP64
//    reductions (compensated FP32 partials); the residual is replaced by the true residual
//    b - K x of the FP64 operator (in double-float arithmetic) periodically and before
//    convergence is accepted, so the stopping test ||b - K x|| <= rtol ||b|| holds for it;
//  * beta is the flexible (Polak-Ribiere) form, robust to the FP32 preconditioner;
//  * every loop kernel checks a device "done" flag, so the host enqueues a few iterations
//    at a time and synchronises once per chunk.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <utility>

#include "anl_ctx.cuh"

namespace anl {

constexpr int VT = 256;  // threads of the 1D vector kernels

static inline int vgrid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(kRedBlocks, (n + VT - 1) / VT)); }

// ------------------------------------------------------------------ accumulators

template <class T>
struct Sum;
template <>
struct Sum<float> {
    Acc2 a;
    __device__ void prod(float x, float y) { a.add_prod(x, y); }
    __device__ double get() const { return a.value(); }
};
template <>
struct Sum<double> {
    double s = 0;
    __device__ void prod(double x, double y) { s = fma(x, y, s); }
    __device__ double get() const { return s; }
};

// Grid sums of NV accumulators into out[0..NV) (finish_reduction's contract; true in the block
// that wrote them): float-pair trees for the FP32 sums, FP64 trees for FP64 ones. smem holds
// NV*NT/32 doubles.
template <int NV, int NT>
__device__ __forceinline__ bool finish_sums(const Sum<float> (&acc)[NV], int bid, int nblocks, double* partials,
                                            unsigned* counter, double* out, double* smem, int tid) {
    float h[NV], l[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        h[i] = acc[i].a.s;
        l[i] = acc[i].a.c;
    }
    float2* sp = reinterpret_cast<float2*>(smem);
    block_pair_sum<NV, NT>(h, l, sp, tid);
    return finish_pair_reduction<NV, NT>(h, l, bid, nblocks, partials, counter, out, tid, sp);
}
template <int NV, int NT>
__device__ __forceinline__ bool finish_sums(const Sum<double> (&acc)[NV], int bid, int nblocks, double* partials,
                                            unsigned* counter, double* out, double* smem, int tid) {
    double v[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = acc[i].get();
    block_sum<NV, NT>(v, smem, tid);
    return finish_reduction<NV, NT>(v, bid, nblocks, partials, counter, out, tid, smem);
}

// ------------------------------------------------------------------ masks and levels

__global__ void k_mask_level0(Dims d, const uint8_t* active, const uint8_t* fixed, uint8_t* nmask) {
    const int64_t nn = d.nn();
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(n % (d.nx + 1));
        const int j = (int)((n / (d.nx + 1)) % (d.ny + 1));
        const int k = (int)(n / ((int64_t)(d.nx + 1) * (d.ny + 1)));
        bool used = false;
        for (int o = 0; o < 8 && !used; ++o) {
            const int ei = i - 1 + (o & 1), ej = j - 1 + ((o >> 1) & 1), ek = k - 1 + ((o >> 2) & 1);
            if (ei >= 0 && ej >= 0 && ek >= 0 && ei < d.nx && ej < d.ny && ek < d.nz) used = active[d.elem(ei, ej, ek)] != 0;
        }
        uint8_t m = 0;
        if (used) {
            m = NODE_USED;
            for (int c = 0; c < 3; ++c)
                if (!fixed[3 * n + c]) m |= (uint8_t)(1 << c);
        }
        nmask[n] = m;
    }
}

__global__ void k_eact_coarse(Dims f, Dims c, const uint8_t* ef, uint8_t* ec) {
    const int64_t ne = c.ne();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        const int I = (int)(e % c.nx), J = (int)((e / c.nx) % c.ny), K = (int)(e / ((int64_t)c.nx * c.ny));
        uint8_t a = 0;
        for (int o = 0; o < 8; ++o) {
            const int i = 2 * I + (o & 1), j = 2 * J + ((o >> 1) & 1), k = 2 * K + ((o >> 2) & 1);
            if (i < f.nx && j < f.ny && k < f.nz) a |= ef[f.elem(i, j, k)];
        }
        ec[e] = a ? 1 : 0;
    }
}

// A coarse DOF is fixed when a used fine node within one fine spacing has that DOF fixed.
__global__ void k_mask_coarse(Dims f, Dims c, const uint8_t* nmf, const uint8_t* eac, uint8_t* nmc) {
    const int64_t nn = c.nn();
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        const int I = (int)(n % (c.nx + 1));
        const int J = (int)((n / (c.nx + 1)) % (c.ny + 1));
        const int K = (int)(n / ((int64_t)(c.nx + 1) * (c.ny + 1)));
        bool used = false;
        for (int o = 0; o < 8 && !used; ++o) {
            const int ei = I - 1 + (o & 1), ej = J - 1 + ((o >> 1) & 1), ek = K - 1 + ((o >> 2) & 1);
            if (ei >= 0 && ej >= 0 && ek >= 0 && ei < c.nx && ej < c.ny && ek < c.nz) used = eac[c.elem(ei, ej, ek)] != 0;
        }
        uint8_t m = 0;
        if (used) {
            uint8_t fixed = 0;
            for (int dk = -1; dk <= 1; ++dk)
                for (int dj = -1; dj <= 1; ++dj)
                    for (int di = -1; di <= 1; ++di) {
                        const int i = 2 * I + di, j = 2 * J + dj, k = 2 * K + dk;
                        if (i < 0 || j < 0 || k < 0 || i > f.nx || j > f.ny || k > f.nz) continue;
                        const uint8_t fm = nmf[f.node(i, j, k)];
                        if (fm & NODE_USED) fixed |= (uint8_t)(~fm & 7);
                    }
            m = (uint8_t)(NODE_USED | (~fixed & 7));
        }
        nmc[n] = m;
    }
}

__global__ void k_count_free(int64_t nn, const uint8_t* nmask, double* partials, unsigned* counter, double* out) {
    __shared__ double sm[VT / 32];
    double v[1] = {0.0};
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x)
        v[0] += (double)__popc(nmask[n] & 7);
    block_sum<1, VT>(v, sm, threadIdx.x);
    finish_reduction<1, VT>(v, blockIdx.x, gridDim.x, partials, counter, out, threadIdx.x, sm);
}

__global__ void k_level0_E(int64_t ne, const float* escale, const uint8_t* active, float h, float* E) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x)
        E[e] = active[e] ? h * escale[e] : 0.f;
}

__global__ void k_coarsen_E(Dims f, Dims c, const float* Ef, float* Ec) {
    const int64_t ne = c.ne();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        const int I = (int)(e % c.nx), J = (int)((e / c.nx) % c.ny), K = (int)(e / ((int64_t)c.nx * c.ny));
        float s = 0.f;
        for (int o = 0; o < 8; ++o) {
            const int i = 2 * I + (o & 1), j = 2 * J + ((o >> 1) & 1), k = 2 * K + ((o >> 2) & 1);
            if (i < f.nx && j < f.ny && k < f.nz) s += Ef[f.elem(i, j, k)];
        }
        Ec[e] = 0.25f * s;
    }
}

__global__ void k_diag(Dims d, const float* E, float kdiag, float* diag /* 1 / diag(K) */) {
    const int64_t nn = d.nn();
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(n % (d.nx + 1));
        const int j = (int)((n / (d.nx + 1)) % (d.ny + 1));
        const int k = (int)(n / ((int64_t)(d.nx + 1) * (d.ny + 1)));
        float s = 0.f;
        for (int o = 0; o < 8; ++o) {
            const int ei = i - 1 + (o & 1), ej = j - 1 + ((o >> 1) & 1), ek = k - 1 + ((o >> 2) & 1);
            if (ei >= 0 && ej >= 0 && ek >= 0 && ei < d.nx && ej < d.ny && ek < d.nz) s += E[d.elem(ei, ej, ek)];
        }
        diag[n] = s > 0.f ? 1.f / (kdiag * s) : 0.f;  // the inverse diagonal, 0 where no element
    }
}

// ------------------------------------------------------------------ transfers

// Grid transfers run one thread per output node on a 3-D launch (32 x 4 threads over x and y,
// one z plane per block row), so no thread divides a flat index: at the finest level the
// transfers are bound by their reads and writes.
// A batch of right-hand sides in one launch: slot r's vectors sit r * fs (this level, or the
// fine level of a transfer) or r * cs (the coarse level of a transfer) values after slot 0's,
// its PCG scalars (done flag) r * sc_bytes bytes after, its reduction scratch r * ps doubles
// after (and its ticket counter r after). nrhs = 1 is the plain single-vector launch.
struct Bt {
    int nrhs = 1;
    int64_t fs = 0, cs = 0;
    int sc_bytes = 0;
    int64_t ps = 0;
};

constexpr int TR_X = 32, TR_Y = 4;
static inline dim3 transfer_grid(const Dims& d, int nrhs = 1) {
    return dim3((unsigned)((d.nx + 1 + TR_X - 1) / TR_X), (unsigned)((d.ny + 1 + TR_Y - 1) / TR_Y),
                (unsigned)((d.nz + 1) * nrhs));
}

// The restriction stages the fine nodes around a coarse tile (TR_X x TR_Y coarse nodes of one
// plane) in shared memory with coalesced loads of consecutive floats, every load of a thread
// issued before any is stored: read straight from the interleaved layout, the stride-2 node
// pattern of a warp touched six times the sectors it used (3.9-6.6 us on the coarse levels
// against 6.0-7.2 us before, the same 20-21 us on the finest). The same staging for the
// prolongation's read-modify-write of the fine nodes was slower (66 against 38 us at 12.8M
// DOF, 25 us now that the prolongation issues all its loads first) and is not used.
constexpr int TRF_X = 2 * TR_X + 1, TRF_Y = 2 * TR_Y + 1;  // fine nodes around a coarse tile

// b_c = R r_f = P^T r_f (trilinear weights 1, 1/2, 1/4, 1/8), zero on fixed coarse DOFs. The
// fine nodes outside the grid are staged as zeros, which add nothing: the sums are those of a
// loop over the in-grid neighbours in the same order.
template <class T>
__global__ void __launch_bounds__(TR_X * TR_Y) k_restrict(Dims f, Dims c, const T* __restrict__ rf,
                                                          const uint8_t* __restrict__ nmc, T* __restrict__ bc,
                                                          const int* done, Bt bt) {
    __shared__ T S[3][TRF_Y][3 * TRF_X];  // fine planes 2K-1..2K+1, rows 2J0-1.., nodes 2I0-1..
    const int slot = blockIdx.z / (c.nz + 1), K = blockIdx.z - slot * (c.nz + 1);
    rf = slot_ptr(rf, slot, bt.fs);
    bc = slot_ptr(bc, slot, bt.cs);
    done = slot_bytes(done, slot, bt.sc_bytes);
    if (done && *done) return;
    const int I0 = blockIdx.x * TR_X, J0 = blockIdx.y * TR_Y;
    const int64_t fx = f.nx + 1, fxy = fx * (f.ny + 1);
    const int fi0 = 2 * I0 - 1;
    // every load of a thread issued before any is stored (a dependent store per load would
    // expose the memory latency once per value)
    constexpr int RPT = (3 * TRF_Y + TR_Y - 1) / TR_Y, QPT = (3 * TRF_X + TR_X - 1) / TR_X;
    T v[RPT][QPT];
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
        const int row = threadIdx.y + rr * TR_Y;
        const int kk = row / TRF_Y, jj = row - kk * TRF_Y;
        const int k = 2 * K - 1 + kk, j = 2 * J0 - 1 + jj;
        const bool rin = row < 3 * TRF_Y && k >= 0 && k <= f.nz && j >= 0 && j <= f.ny;
        const T* src = rf + 3 * ((int64_t)k * fxy + (int64_t)j * fx + fi0);
#pragma unroll
        for (int qq = 0; qq < QPT; ++qq) {
            const int q = threadIdx.x + qq * TR_X;
            const int i = fi0 + q / 3;
            v[rr][qq] = rin && q < 3 * TRF_X && i >= 0 && i <= f.nx &&
                                ANL_IN_RANGE((int64_t)k * fxy + (int64_t)j * fx + i, fxy * (f.nz + 1))
                            ? __ldg(src + q)
                            : T(0);
        }
    }
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
        const int row = threadIdx.y + rr * TR_Y;
        if (row >= 3 * TRF_Y) continue;
        const int kk = row / TRF_Y, jj = row - kk * TRF_Y;
#pragma unroll
        for (int qq = 0; qq < QPT; ++qq) {
            const int q = threadIdx.x + qq * TR_X;
            if (q < 3 * TRF_X) S[kk][jj][q] = v[rr][qq];
        }
    }
    __syncthreads();
    const int I = I0 + threadIdx.x, J = J0 + threadIdx.y;
    if (I > c.nx || J > c.ny) return;
    T acc0 = T(0), acc1 = T(0), acc2 = T(0);
#pragma unroll
    for (int dk = -1; dk <= 1; ++dk) {
        const T wk = dk == 0 ? T(1) : T(0.5);
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj) {
            const T wj = dj == 0 ? wk : wk * T(0.5);
            const T* row = &S[1 + dk][2 * threadIdx.y + 1 + dj][0];
#pragma unroll
            for (int di = -1; di <= 1; ++di) {
                const T w = di == 0 ? wj : wj * T(0.5);
                const T* q = row + 3 * (2 * threadIdx.x + 1 + di);
                acc0 += w * q[0];
                acc1 += w * q[1];
                acc2 += w * q[2];
            }
        }
    }
    const int64_t n = (int64_t)I + (int64_t)(c.nx + 1) * ((int64_t)J + (int64_t)(c.ny + 1) * K);
    if (!ANL_IN_RANGE(n, c.nn())) return;
    const uint8_t m = nmc[n];
    T* o = bc + 3 * n;
    o[0] = (m & 1) ? acc0 : T(0);
    o[1] = (m & 2) ? acc1 : T(0);
    o[2] = (m & 4) ? acc2 : T(0);
}

// x_f += P x_c on free fine DOFs (trilinear interpolation of the coarse correction). One
// thread per coarse node (I, J, K) updates the up to 8 fine nodes (2I + a, 2J + b, 2K + g),
// a, b, g in {0, 1}, from the up to 8 coarse nodes (I + a', J + b', K + g'). Every load of a
// thread (coarse values, fine masks and fine values) is issued before the first store and
// none depends on another, so one memory latency covers all of them (with the fine loads
// behind a test of their mask, each fine node cost two latencies in turn: 38 us at 12.8M DOF
// against 25 us).
template <class T>
__global__ void __launch_bounds__(TR_X * TR_Y, 4) k_prolong_add(Dims f, Dims c, const T* __restrict__ xc,
                                                                const uint8_t* __restrict__ nmf, T* __restrict__ xf,
                                                                const int* done, Bt bt) {
    const int slot = blockIdx.z / (c.nz + 1), K = blockIdx.z - slot * (c.nz + 1);
    xc = slot_ptr(xc, slot, bt.cs);
    xf = slot_ptr(xf, slot, bt.fs);
    done = slot_bytes(done, slot, bt.sc_bytes);
    if (done && *done) return;
    const int I = blockIdx.x * TR_X + threadIdx.x, J = blockIdx.y * TR_Y + threadIdx.y;
    if (I > c.nx || J > c.ny) return;
    const int64_t cx = c.nx + 1, cxy = cx * (c.ny + 1);
    const int64_t fx = f.nx + 1, fxy = fx * (f.ny + 1);
    // coarse corner values v[g][b][a] (zero beyond the coarse grid: never used with weight)
    T v[2][2][2][3];
#pragma unroll
    for (int g = 0; g < 2; ++g)
#pragma unroll
        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                const int64_t cn = (int64_t)(K + g) * cxy + (int64_t)(J + bb) * cx + (I + a);
                const bool in = I + a <= c.nx && J + bb <= c.ny && K + g <= c.nz && ANL_IN_RANGE(cn, cxy * (c.nz + 1));
                const T* q = xc + 3 * cn;
#pragma unroll
                for (int e = 0; e < 3; ++e) v[g][bb][a][e] = in ? __ldg(q + e) : T(0);
            }
    // fine node values and masks (mask 0 beyond the fine grid: nothing stored there)
    T xv[2][2][2][3];
    uint8_t mv[2][2][2];
#pragma unroll
    for (int g = 0; g < 2; ++g)
#pragma unroll
        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                const int i = 2 * I + a, j = 2 * J + bb, k = 2 * K + g;
                const int64_t nf = (int64_t)k * fxy + (int64_t)j * fx + i;
                const bool in = i <= f.nx && j <= f.ny && k <= f.nz && ANL_IN_RANGE(nf, fxy * (f.nz + 1));
                const int64_t n = in ? nf : 0;
                mv[g][bb][a] = in ? __ldg(nmf + n) : uint8_t(0);
#pragma unroll
                for (int e = 0; e < 3; ++e) xv[g][bb][a][e] = in ? xf[3 * n + e] : T(0);
            }
#pragma unroll
    for (int g = 0; g < 2; ++g)
#pragma unroll
        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                const uint8_t m = mv[g][bb][a];
                if (!(m & 7)) continue;
                const int64_t n = (int64_t)(2 * K + g) * fxy + (int64_t)(2 * J + bb) * fx + (2 * I + a);
                // fine node (i, j, k): the mean of the coarse nodes it lies between
                const T w = (a ? T(0.5) : T(1)) * (bb ? T(0.5) : T(1)) * (g ? T(0.5) : T(1));
                T* o = xf + 3 * n;
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    T t = v[0][0][0][e];
                    if (a) t += v[0][0][1][e];
                    if (bb) t += v[0][1][0][e] + (a ? v[0][1][1][e] : T(0));
                    if (g) {
                        T u = v[1][0][0][e];
                        if (a) u += v[1][0][1][e];
                        if (bb) u += v[1][1][0][e] + (a ? v[1][1][1][e] : T(0));
                        t += u;
                    }
                    if ((m >> e) & 1) o[e] = xv[g][bb][a][e] + w * t;
                }
            }
}

// x = d = c2 D^-1 b  (first Chebyshev step from x = 0)
template <class T>
__global__ void k_cheb_first(int64_t nn, const T* b, const float* dinv, const uint8_t* nmask, const double* c2p, T* x,
                             T* dv, const int* done, Bt bt) {
    b = slot_ptr(b, blockIdx.y, bt.fs);
    x = slot_ptr(x, blockIdx.y, bt.fs);
    dv = slot_ptr(dv, blockIdx.y, bt.fs);
    done = slot_bytes(done, blockIdx.y, bt.sc_bytes);
    if (done && *done) return;
    const T c2 = T(*c2p);
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t m = nmask[n];
        const T inv = T(dinv[n]);
        for (int c = 0; c < 3; ++c) {
            const T v = (m >> c) & 1 ? c2 * b[3 * n + c] * inv : T(0);
            x[3 * n + c] = v;
            dv[3 * n + c] = v;
        }
    }
}

// ------------------------------------------------------------------ coarsest grid (FP64)

// Dense K of the coarsest level, one thread per entry (deterministic: each entry sums
// the elements shared by its two nodes in a fixed order). Non-free rows/cols -> identity.
__global__ void k_assemble_dense(Dims d, const float* E, const uint8_t* nmask, const double* ke, int n, double* A) {
    const int64_t total = (int64_t)n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int row = (int)(t / n), col = (int)(t % n);
        const int64_t N = row / 3, M = col / 3;
        const int ci = row % 3, cj = col % 3;
        const bool fr = (nmask[N] >> ci) & 1, fc = (nmask[M] >> cj) & 1;
        if (!fr || !fc) {
            A[t] = row == col ? 1.0 : 0.0;
            continue;
        }
        const int Ni = (int)(N % (d.nx + 1)), Nj = (int)((N / (d.nx + 1)) % (d.ny + 1)),
                  Nk = (int)(N / ((int64_t)(d.nx + 1) * (d.ny + 1)));
        const int Mi = (int)(M % (d.nx + 1)), Mj = (int)((M / (d.nx + 1)) % (d.ny + 1)),
                  Mk = (int)(M / ((int64_t)(d.nx + 1) * (d.ny + 1)));
        double s = 0.0;
        if (abs(Ni - Mi) <= 1 && abs(Nj - Mj) <= 1 && abs(Nk - Mk) <= 1) {
            for (int o = 0; o < 8; ++o) {
                const int ei = Ni - 1 + (o & 1), ej = Nj - 1 + ((o >> 1) & 1), ek = Nk - 1 + ((o >> 2) & 1);
                if (ei < 0 || ej < 0 || ek < 0 || ei >= d.nx || ej >= d.ny || ek >= d.nz) continue;
                const int bi = Mi - ei, bj = Mj - ej, bk = Mk - ek;
                if (bi < 0 || bi > 1 || bj < 0 || bj > 1 || bk < 0 || bk > 1) continue;
                const int ai = Ni - ei, aj = Nj - ej, ak = Nk - ek;
                // local node numbering LOCAL (fem.py:20-21): bottom face counter-clockwise
                const int la = (ak << 2) | (aj ? (ai ? 2 : 3) : (ai ? 1 : 0));
                const int lb = (bk << 2) | (bj ? (bi ? 2 : 3) : (bi ? 1 : 0));
                s += (double)E[d.elem(ei, ej, ek)] * ke[(3 * la + ci) * 24 + 3 * lb + cj];
            }
        }
        A[t] = s;
    }
}

// In-place lower Cholesky factor of the n x n SPD matrix A (one CTA, right-looking).
__global__ void __launch_bounds__(1024) k_cholesky(double* A, int n, int* flag) {
    __shared__ double piv, dmax;
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int j = 0; j < n; ++j) m = fmax(m, A[(int64_t)j * n + j]);
        dmax = m;
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        if (threadIdx.x == 0) {
            const double a = A[(int64_t)j * n + j];
            // A pivot this small relative to the largest diagonal comes from near-void coarse
            // elements (E_min 1e-9 of a design) or from a floating piece. The factor only
            // preconditions, so it is regularised to stay positive definite; a part that
            // cannot carry its load shows up as a CG that does not converge.
            if (!(a > 1e-12 * dmax)) {
                *flag += 1;
                piv = sqrt(1e-12 * dmax);
            } else {
                piv = sqrt(a);
            }
            A[(int64_t)j * n + j] = piv;
        }
        __syncthreads();
        const double p = piv;
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) A[(int64_t)i * n + j] /= p;
        __syncthreads();
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
        for (int gi = j + 1 + warp; gi < n; gi += nw) {
            const double lij = A[(int64_t)gi * n + j];
            for (int gk = j + 1 + lane; gk <= gi; gk += 32) A[(int64_t)gi * n + gk] -= lij * A[(int64_t)gk * n + j];
        }
        __syncthreads();
    }
}

// Column c of A^-1 from the Cholesky factor L (lower triangle of A): one CTA per column.
__global__ void __launch_bounds__(128) k_chol_inverse(const double* L, double* Ainv, int n) {
    extern __shared__ double xs[];
    const int c = blockIdx.x;
    for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = i == c ? 1.0 : 0.0;
    __syncthreads();
    for (int j = 0; j < n; ++j) {  // L y = e_c
        const double yj = xs[j] / L[(int64_t)j * n + j];
        __syncthreads();
        if (threadIdx.x == 0) xs[j] = yj;
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) xs[i] -= L[(int64_t)i * n + j] * yj;
        __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {  // L^T x = y
        const double xj = xs[j] / L[(int64_t)j * n + j];
        __syncthreads();
        if (threadIdx.x == 0) xs[j] = xj;
        for (int i = threadIdx.x; i < j; i += blockDim.x) xs[i] -= L[(int64_t)j * n + i] * xj;
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) Ainv[(int64_t)i * n + c] = xs[i];
}

// The same factorisation and inverse with the matrix in shared memory, for n <= kCholSmemN
// (n^2 doubles within the 227 KB a CTA may hold): no global round trip per column step, and
// the inverse multiplies by precomputed reciprocal pivots.
constexpr int kCholSmemN = 160;

__global__ void __launch_bounds__(1024) k_cholesky_smem(double* A, int n, int* flag) {
    extern __shared__ double S[];
    __shared__ double piv, dmax;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) S[t] = A[t];
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int j = 0; j < n; ++j) m = fmax(m, S[j * n + j]);
        dmax = m;
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        if (threadIdx.x == 0) {
            const double a = S[j * n + j];
            // tiny pivots are regularised as in k_cholesky
            if (!(a > 1e-12 * dmax)) {
                *flag += 1;
                piv = sqrt(1e-12 * dmax);
            } else {
                piv = sqrt(a);
            }
            S[j * n + j] = piv;
        }
        __syncthreads();
        const double rp = 1.0 / piv;
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) S[i * n + j] *= rp;
        __syncthreads();
        // trailing update of the lower triangle: one thread per (i, k), k <= i
        const int m = n - j - 1;
        for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
            const int i = j + 1 + t / m, k = j + 1 + t % m;
            if (k <= i) S[i * n + k] -= S[i * n + j] * S[k * n + j];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) A[t] = S[t];
}

__global__ void __launch_bounds__(256) k_chol_inverse_smem(const double* L, double* Ainv, int n) {
    extern __shared__ double S[];  // L (n * n), reciprocal pivots (n), the column (n)
    double* rd = S + n * n;
    double* xs = rd + n;
    const int c = blockIdx.x;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) S[t] = L[t];
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        rd[i] = 1.0 / S[i * n + i];
        xs[i] = i == c ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int j = c; j < n; ++j) {  // L y = e_c (y_j = 0 for j < c)
        const double yj = xs[j] * rd[j];
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) xs[i] -= S[i * n + j] * yj;
        __syncthreads();
        if (threadIdx.x == 0) xs[j] = yj;
        __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {  // L^T x = y
        const double xj = xs[j] * rd[j];
        for (int i = threadIdx.x; i < j; i += blockDim.x) xs[i] -= S[j * n + i] * xj;
        __syncthreads();
        if (threadIdx.x == 0) xs[j] = xj;
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) Ainv[(int64_t)i * n + c] = xs[i];
}

// The FP32 solver's coarsest grid in double-float arithmetic (about 48 bits, on the FP32 pipes:
// FP64 arithmetic on this part runs at a small fraction of FP32, and the factor's trailing
// updates are ~n^3/6 multiply-adds on one SM): A = L D L^T, no square roots. The matrix comes in
// as FP64 and is split into float pairs without FP64 arithmetic (split_double). Each column
// step is two phases with a barrier after each: the column of L (and an unscaled copy), then
// the trailing update of the lower triangle, one warp per row. Every thread forms the pivot's
// reciprocal itself, so the pivot needs no phase of its own. Tiny pivots are regularised as in
// k_cholesky (to 1e-12 of the largest diagonal entry). On exit A holds L strictly below the
// diagonal (unit diagonal implied) and D on it.
__global__ void __launch_bounds__(1024) k_ldlt_df(double* A, int n, int* flag) {
    extern __shared__ DF SD[];  // the matrix (n * n), then the unscaled column (n)
    DF* ucol = SD + n * n;
    __shared__ float dmax;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        float h, l;
        split_double(A[t], h, l);
        SD[t] = DF(h, l);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        float m = 0.f;
        for (int j = threadIdx.x; j < n; j += 32) m = fmaxf(m, SD[j * n + j].hi);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) dmax = m;
    }
    __syncthreads();
    const float floor_ = 1e-12f * dmax;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < n; ++j) {
        DF a = SD[j * n + j];
        if (!(a.hi > floor_)) {  // every thread takes the same branch (the value is idempotent)
            a = DF(floor_);
            if (threadIdx.x == 0) {
                SD[j * n + j] = a;
                *flag += 1;
            }
        }
        const DF ia = df_recip(a);
        for (int k = j + 1 + threadIdx.x; k < n; k += blockDim.x) {
            const DF u = SD[k * n + j];
            ucol[k] = u;
            SD[k * n + j] = u * ia;
        }
        __syncthreads();
        for (int i = j + 1 + warp; i < n; i += nw) {
            const DF lij = SD[i * n + j];
            for (int k = j + 1 + lane; k <= i; k += 32) SD[i * n + k] = SD[i * n + k] - lij * ucol[k];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) A[t] = SD[t].value();
}

// Column c of A^-1 from L D L^T (k_ldlt_df), one CTA per column: L y = e_c, z = D^-1 y,
// L^T x = z, one barrier per step (each thread reads the settled entry of the step and
// updates the others).
__global__ void __launch_bounds__(256) k_ldlt_inverse_df(const double* LD, double* Ainv, int n) {
    extern __shared__ DF SD[];  // L (n * n), 1 / D (n), the column (n)
    DF* rd = SD + n * n;
    DF* xs = rd + n;
    const int c = blockIdx.x;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        float h, l;
        split_double(LD[t], h, l);
        SD[t] = DF(h, l);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        rd[i] = df_recip(SD[i * n + i]);
        xs[i] = DF(i == c ? 1.f : 0.f);
    }
    __syncthreads();
    for (int j = c; j < n - 1; ++j) {  // L y = e_c (y_j = 0 for j < c)
        const DF yj = xs[j];
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) xs[i] = xs[i] - SD[i * n + j] * yj;
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = xs[i] * rd[i];
    __syncthreads();
    for (int j = n - 1; j > 0; --j) {  // L^T x = z
        const DF xj = xs[j];
        for (int i = threadIdx.x; i < j; i += blockDim.x) xs[i] = xs[i] - SD[j * n + i] * xj;
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) Ainv[(int64_t)i * n + c] = xs[i].value();
}

// x = A^-1 b on the coarsest grid (FP64), one warp per row.
template <class T>
__global__ void k_coarse_apply(const double* Ainv, int n, const T* b, const uint8_t* nmask, T* x, const int* done,
                               Bt bt) {
    b = slot_ptr(b, blockIdx.y, bt.fs);
    x = slot_ptr(x, blockIdx.y, bt.fs);
    done = slot_bytes(done, blockIdx.y, bt.sc_bytes);
    if (done && *done) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int row = warp; row < n; row += nw) {
        double s = 0.0;
        for (int c = lane; c < n; c += 32) s += Ainv[(int64_t)row * n + c] * (double)b[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) x[row] = (nmask[row / 3] >> (row % 3)) & 1 ? T(s) : T(0);
    }
}

// ------------------------------------------------------------------ CG vector kernels

__global__ void k_mask_copy_d(int64_t nn, const double* in, const uint8_t* nmask, double* out) {
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t m = nmask[n];
        for (int c = 0; c < 3; ++c) out[3 * n + c] = (m >> c) & 1 ? in[3 * n + c] : 0.0;
    }
}

template <class T>
__global__ void k_mask_copy_t(int64_t nn, const T* in, const uint8_t* nmask, T* out) {
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t m = nmask[n];
        for (int c = 0; c < 3; ++c) out[3 * n + c] = (m >> c) & 1 ? in[3 * n + c] : T(0);
    }
}

__global__ void k_dot_d(int64_t n, const double* a, const double* b, double* partials, unsigned* counter, double* out) {
    __shared__ double sm[VT / 32];
    double v[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[0] = fma(a[i], b[i], v[0]);
    block_sum<1, VT>(v, sm, threadIdx.x);
    finish_reduction<1, VT>(v, blockIdx.x, gridDim.x, partials, counter, out, threadIdx.x, sm);
}

// x (FP64) -> hi + lo in two float vectors, without FP64 arithmetic (split_double)
__global__ void k_split_hl(int64_t n, const double* x, float* hi, float* lo) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        split_double(x[i], hi[i], lo[i]);
}

// r = b - y1 - y2 for the FP32 solver, b as float pairs (k_split_df), the differences and
// ||r||^2 in float-pair arithmetic; sets the CG state as k_true_resid does.
__global__ void k_true_resid_pair(int64_t n, const DF* b, const float* y1, const float* y2, float* r, PcgScalars* sc,
                                  int set_state, double* partials, unsigned* counter) {
    __shared__ double sm[VT / 32];
    Sum<float> acc[1];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const DF ri = b[i] - DF(y1[i]) - DF(y2[i]);
        const float rf = ri.hi + ri.lo;
        r[i] = rf;
        acc[0].prod(rf, rf);
    }
    __shared__ double res[1];
    if (finish_sums<1, VT>(acc, blockIdx.x, gridDim.x, partials, counter, res, sm, threadIdx.x)) {
        if (threadIdx.x == 0) {
            sc->rr_true = res[0];
            if (set_state) {
                sc->rr = res[0];
                if (!isfinite(res[0])) {
                    sc->done = 3;
                    sc->nonfinite = 1;
                } else {
                    sc->done = res[0] <= sc->tol2 ? 1 : 0;
                }
            }
        }
    }
}

// x (FP64) -> (hi, lo) float pairs, without FP64 arithmetic (split_double)
__global__ void k_split_df(int64_t n, const double* x, DF* xdf) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float h, l;
        split_double(x[i], h, l);
        xdf[i] = DF(h, l);
    }
}

// r = b - y1 - y2 (y2 may be null), ||r||^2; sets the CG state from the true residual.
template <class T>
__global__ void k_true_resid(int64_t n, const double* b, const T* y1, const T* y2, T* r, PcgScalars* sc,
                             int set_state, double* partials, unsigned* counter) {
    __shared__ double sm[VT / 32];
    double v[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double ri = b[i] - (double)y1[i];
        if (y2) ri -= (double)y2[i];
        r[i] = T(ri);
        v[0] = fma(ri, ri, v[0]);
    }
    block_sum<1, VT>(v, sm, threadIdx.x);
    __shared__ double res[1];
    if (finish_reduction<1, VT>(v, blockIdx.x, gridDim.x, partials, counter, res, threadIdx.x, sm)) {
        if (threadIdx.x == 0) {
            sc->rr_true = res[0];
            if (set_state) {
                sc->rr = res[0];
                if (!isfinite(res[0])) {
                    sc->done = 3;
                    sc->nonfinite = 1;
                } else {
                    sc->done = res[0] <= sc->tol2 ? 1 : 0;
                }
            }
        }
    }
}

__global__ void k_init_scalars(PcgScalars* sc, double rtol, int maxiter, const double* bb) {
    sc->bb = *bb;
    sc->tol2 = rtol * rtol * (*bb);
    sc->iters = 0;
    sc->done = 0;
    sc->nonfinite = 0;
    sc->maxiter = maxiter;
    sc->rz[0] = sc->rz[1] = 0.0;
    sc->alpha = 0.0;
    sc->zq = 0.0;
    sc->pq = 0.0;
}

// Four consecutive entries per access (16-byte loads and stores; every vector of the CG and
// the hierarchy starts on a 256-byte cudaMalloc boundary). The CG kernels walk the vectors in
// groups of four; the last n % 4 entries go to a scalar tail.
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
    const double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&v)[4]) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}
// calls f(i) for every index of [0, n) this thread owns: groups of four, then the tail
template <class F4, class F1>
__device__ __forceinline__ void for_each4(int64_t n, F4 f4, F1 f1) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x, t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t n4 = n >> 2;
    for (int64_t g = t; g < n4; g += stride) f4(4 * g);
    for (int64_t i = 4 * n4 + t; i < n; i += stride) f1(i);
}

template <class T>
__global__ void k_dots_rz_zq(int64_t n, const T* r, const T* z, const T* q, PcgScalars* sc, const int* restart,
                             double* partials, unsigned* counter, Bt bt) {
    __shared__ double sm[2 * VT / 32];
    {  // batch slot (grid.y)
        const int sl = blockIdx.y;
        r = slot_ptr(r, sl, bt.fs);
        z = slot_ptr(z, sl, bt.fs);
        q = slot_ptr(q, sl, bt.fs);
        sc += sl;
        restart += sl;
        partials = slot_ptr(partials, sl, bt.ps);
        counter += sl;
    }
    if (sc->done) return;
    const bool rs = *restart != 0;
    Sum<T> ab[2];
    Sum<T>& a = ab[0];
    Sum<T>& b = ab[1];
    for_each4(
        n,
        [&](int64_t i) {
            T zv[4], rv[4], qv[4];
            ld4(z + i, zv);
            ld4(r + i, rv);
#pragma unroll
            for (int e = 0; e < 4; ++e) a.prod(rv[e], zv[e]);
            if (!rs) {
                ld4(q + i, qv);
#pragma unroll
                for (int e = 0; e < 4; ++e) b.prod(zv[e], qv[e]);
            }
        },
        [&](int64_t i) {
            const T zi = z[i];
            a.prod(r[i], zi);
            if (!rs) b.prod(zi, q[i]);
        });
    __shared__ double res[2];
    if (finish_sums<2, VT>(ab, blockIdx.x, gridDim.x, partials, counter, res, sm, threadIdx.x)) {
        if (threadIdx.x == 0) {
            const int it = sc->iters;
            sc->rz[it & 1] = res[0];
            sc->zq = res[1];
            if (!isfinite(res[0]) || !isfinite(res[1])) {
                sc->done = 3;
                sc->nonfinite = 1;
            } else if (!(res[0] > 0.0)) {
                sc->done = 4;
            }
        }
    }
}

template <class T>
__global__ void k_pupdate(int64_t n, const T* z, T* p, const PcgScalars* sc, const int* restart, Bt batch) {
    z = slot_ptr(z, blockIdx.y, batch.fs);
    p = slot_ptr(p, blockIdx.y, batch.fs);
    sc += blockIdx.y;
    restart += blockIdx.y;
    if (sc->done) return;
    const int it = sc->iters;
    if (*restart) {  // p = z (not z + 0 p: p may hold non-finite values after a breakdown)
        for_each4(
            n,
            [&](int64_t i) {
                T zv[4];
                ld4(z + i, zv);
                st4(p + i, zv);
            },
            [&](int64_t i) { p[i] = z[i]; });
        return;
    }
    const T bt = T(-sc->alpha * sc->zq / sc->rz[(it + 1) & 1]);
    for_each4(
        n,
        [&](int64_t i) {
            T zv[4], pv[4];
            ld4(z + i, zv);
            ld4(p + i, pv);
#pragma unroll
            for (int e = 0; e < 4; ++e) pv[e] = zv[e] + bt * pv[e];
            st4(p + i, pv);
        },
        [&](int64_t i) { p[i] = z[i] + bt * p[i]; });
}

constexpr double kRecurrenceMargin = 0.5;  // (0.71 rtol)^2: the recurrence target, squared

template <class T>
__global__ void k_axpy(int64_t n, const T* p, const T* q, double* x, T* r, PcgScalars* sc, int* restart,
                       double* partials, unsigned* counter, Bt bt) {
    __shared__ double sm[VT / 32];
    {  // batch slot (grid.y)
        const int sl = blockIdx.y;
        p = slot_ptr(p, sl, bt.fs);
        q = slot_ptr(q, sl, bt.fs);
        x = slot_ptr(x, sl, bt.fs);
        r = slot_ptr(r, sl, bt.fs);
        sc += sl;
        restart += sl;
        partials = slot_ptr(partials, sl, bt.ps);
        counter += sl;
    }
    if (sc->done) return;
    const int it = sc->iters;
    const double pq = sc->pq;
    const double alpha = sc->rz[it & 1] / pq;
    const bool bad = !(pq > 0.0) || !isfinite(alpha);
    Sum<T> rr1[1];
    Sum<T>& rr = rr1[0];
    if (!bad) {
        const T at = T(alpha);
        for_each4(
            n,
            [&](int64_t i) {
                T pv[4], qv[4], rv[4];
                double xv[4];
                ld4(p + i, pv);
                ld4(q + i, qv);
                ld4(r + i, rv);
                ld4(x + i, xv);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    xv[e] = fma(alpha, (double)pv[e], xv[e]);
                    rv[e] = rv[e] - at * qv[e];
                    rr.prod(rv[e], rv[e]);
                }
                st4(x + i, xv);
                st4(r + i, rv);
            },
            [&](int64_t i) {
                x[i] = fma(alpha, (double)p[i], x[i]);
                const T ri = r[i] - at * q[i];
                r[i] = ri;
                rr.prod(ri, ri);
            });
    }
    __shared__ double res[1];
    if (finish_sums<1, VT>(rr1, blockIdx.x, gridDim.x, partials, counter, res, sm, threadIdx.x)) {
        if (threadIdx.x == 0) {
            sc->alpha = alpha;
            sc->rr = res[0];
            sc->iters = it + 1;
            *restart = 0;
            if (bad) {
                if (isfinite(pq) && isfinite(alpha)) sc->done = 4;
                else {
                    sc->done = 3;
                    sc->nonfinite = 1;
                }
            } else if (!isfinite(res[0])) {
                sc->done = 3;
                sc->nonfinite = 1;
            } else if (res[0] <= kRecurrenceMargin * sc->tol2) {
                // the recurrence residual drifts from the true one by a few tens of percent
                // in FP32; claiming convergence a little early would cost a failed
                // certification (one accurate residual) and a restart
                sc->done = 1;
            } else if (it + 1 >= sc->maxiter) {
                sc->done = 2;
            }
        }
    }
}

// ------------------------------------------------------------------ host side

template <class T>
static KeModal<T> modal_of(const anl_ctx* c);
template <>
KeModal<float> modal_of<float>(const anl_ctx* c) { return c->kmf; }
template <>
KeModal<double> modal_of<double>(const anl_ctx* c) { return c->kmd; }

// The K u passes of the finest level go to the tensor-core kernel (anl_kutc.cu) when the
// context enables it (FP32 contexts); every other level and precision uses the SIMT kernel.
template <class T>
static int ku_pass(anl_ctx* c, const Level& L, int mode, const KuArgs<T>& a, cudaStream_t s) {
    if constexpr (sizeof(T) == 4) {
        if (c->use_tc && c->rb == 1 && &L == &c->lev[0]) {
            KuArgs<float> t = a;
            t.diag = L.diag;
            return launch_kutc(mode, t, c->kmf, s);
        }
    }
    return launch_ku<T>(mode, a, modal_of<T>(c), s);
}

template <class T>
static KuArgs<T> ku_args(anl_ctx* c, const Level& L) {
    KuArgs<T> a;
    a.d = L.d;
    a.E = L.E;
    a.nmask = L.nmask;
    a.diag = L.diag;  // the Chebyshev passes' inverse diagonal
    a.kdiag = T(c->kdiag);
    a.partials = c->partials;
    a.counter = c->counter;
    a.partial_capacity = c->part_cap;
    a.nrhs = c->rb;
    a.vstride = L.vs;
    a.sc_bytes = (int)sizeof(PcgScalars);
    a.part_stride = c->part_stride;
    return a;
}

// the batch descriptor of a launch on level L (and its coarse level C for transfers)
static Bt bt_of(const anl_ctx* c, const Level& L, const Level* C = nullptr) {
    Bt b;
    b.nrhs = c->rb;
    b.fs = L.vs;
    b.cs = C ? C->vs : 0;
    b.sc_bytes = (int)sizeof(PcgScalars);
    b.ps = c->part_stride;
    return b;
}

// Points the single-vector state (level-0 right-hand side / residual, the FP64 solution and
// right-hand side, the float-pair right-hand side, the PCG scalars, the restart flag) at slot r.
static void set_slot(anl_ctx* c, int r) {
    c->slot = r;
    const int64_t vs0 = c->lev[0].vs;
    c->lev[0].b = (char*)c->b0_base + (size_t)r * vs0 * c->tsize;
    c->xbuf = c->xbuf_base + (size_t)r * vs0;
    c->bbuf = c->bbuf_base + (size_t)r * vs0;
    if (c->bdf_base) c->bdf = (DF*)c->bdf_base + (size_t)r * vs0;
    c->sc = c->sc_base + r;
}

template <class T>
static int apply_level(anl_ctx* c, const Level& L, const T* u, T* y, cudaStream_t s, double* dot_out = nullptr,
                       const int* done = nullptr) {
    KuArgs<T> a = ku_args<T>(c, L);
    a.u = u;
    a.y = y;
    a.done = done;
    a.red_out = dot_out;
    return ku_pass<T>(c, L, dot_out ? KU_APPLY_DOT : KU_APPLY, a, s);
}

static int level_index(const anl_ctx* c, const Level& L) { return (int)(&L - &c->lev[0]); }

// Chebyshev coefficients of a `degree`-step sweep of D^-1 K over [lo_frac, 1] x bound,
// where bound = lambda_max(Ke) / Ke_00 >= lambda_max(D^-1 K) on every level and for every
// design: out = {bound, c1_0, c2_0, c1_1, c2_1, ...}. A power-iteration estimate of the
// spectrum approaches lambda_max from below and misses the localised top modes of solid
// voxels inside void, which a sweep above its interval amplifies; the bound cannot.
void cheb_coefficients(double bound, double lo_frac, int degree, double* out) {
    const double hi = bound, lo = lo_frac * bound;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
    double rho_old = 1.0 / sigma;
    out[0] = bound;
    out[1] = 0.0;
    out[2] = 1.0 / theta;
    for (int k = 1; k < degree && k < kChebMax; ++k) {
        const double rho = 1.0 / (2.0 * sigma - rho_old);
        out[1 + 2 * k] = rho * rho_old;
        out[2 + 2 * k] = 2.0 * rho / delta;
        rho_old = rho;
    }
}

static int coarse_factor(anl_ctx* c, cudaStream_t s) {
    Level& L = c->lev.back();
    const int n = c->nc;
    const int64_t total = (int64_t)n * n;
    k_assemble_dense<<<(int)std::min<int64_t>(4096, (total + 255) / 256), 256, 0, s>>>(L.d, L.E, L.nmask, c->ke_d, n, c->A);
    ANL_LAUNCH_CHECK();
    ANL_CUDA(cudaMemsetAsync(c->flag_d, 0, sizeof(int), s));
    if (n <= kCholSmemN) {
        const int fb = n * n * (int)sizeof(double), ib = (n * n + 2 * n) * (int)sizeof(double);
        static bool attr = false;
        if (!attr) {
            ANL_CUDA(cudaFuncSetAttribute(k_cholesky_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          kCholSmemN * kCholSmemN * (int)sizeof(double)));
            ANL_CUDA(cudaFuncSetAttribute(k_chol_inverse_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (kCholSmemN * kCholSmemN + 2 * kCholSmemN) * (int)sizeof(double)));
            ANL_CUDA(cudaFuncSetAttribute(k_ldlt_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (kCholSmemN * kCholSmemN + kCholSmemN) * (int)sizeof(DF)));
            ANL_CUDA(cudaFuncSetAttribute(k_ldlt_inverse_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (kCholSmemN * kCholSmemN + 2 * kCholSmemN) * (int)sizeof(DF)));
            attr = true;
        }
        if (c->fp64) {
            k_cholesky_smem<<<1, 1024, fb, s>>>(c->A, n, c->flag_d);
            ANL_LAUNCH_CHECK();
            k_chol_inverse_smem<<<n, 256, ib, s>>>(c->A, c->Ainv, n);
            ANL_LAUNCH_CHECK();
        } else {  // the FP32 solver's preconditioner: double-float factor and inverse
            k_ldlt_df<<<1, 1024, (n * n + n) * (int)sizeof(DF), s>>>(c->A, n, c->flag_d);
            ANL_LAUNCH_CHECK();
            k_ldlt_inverse_df<<<n, 256, (n * n + 2 * n) * (int)sizeof(DF), s>>>(c->A, c->Ainv, n);
            ANL_LAUNCH_CHECK();
        }
    } else {
        k_cholesky<<<1, 1024, 0, s>>>(c->A, n, c->flag_d);
        ANL_LAUNCH_CHECK();
        k_chol_inverse<<<n, 128, n * sizeof(double), s>>>(c->A, c->Ainv, n);
        ANL_LAUNCH_CHECK();
    }
    if (c->tail_from >= 0) ANL_TRY(launch_ainv_split(c->Ainv, n, c->ainv_hi, c->ainv_lo, s));
    c->coarse_ready = true;
    return ANL_OK;
}

// Refresh the hierarchy's element scales from the level-0 scales; with `rebuild` also
// re-estimate the smoother spectra and refactor the coarsest grid.
template <class T>
static int update_hierarchy(anl_ctx* c, bool rebuild, cudaStream_t s) {
    for (size_t l = 0; l < c->lev.size(); ++l) {
        Level& L = c->lev[l];
        if (l > 0) {
            const Level& F = c->lev[l - 1];
            k_coarsen_E<<<vgrid(L.d.ne()), VT, 0, s>>>(F.d, L.d, F.E, L.E);
            ANL_LAUNCH_CHECK();
        }
        k_diag<<<vgrid(L.d.nn()), VT, 0, s>>>(L.d, L.E, (float)c->kdiag, L.diag);
        ANL_LAUNCH_CHECK();
    }
    // the coarsest grid's factor follows the design every solve: a stale one makes the
    // V-cycle a poor (even indefinite) preconditioner once the design has moved on
    (void)rebuild;
    if (c->dense_coarse) ANL_TRY(coarse_factor(c, s));
    else c->coarse_ready = true;
    return ANL_OK;
}

// degree Chebyshev steps on level L with the device coefficients of that level; x_is_zero
// uses the elementwise first step.
template <class T>
static int smooth(anl_ctx* c, Level& L, int degree, bool x_is_zero, const int* done, cudaStream_t s) {
    const double* cf = c->cheb_d + (size_t)level_index(c, L) * kChebStride + 1;  // (c1, c2) pairs
    int k0 = 0;
    if (x_is_zero && degree >= 2) {  // steps 0 and 1 in one pass: x1 = c2_0 D^-1 b is never stored
        KuArgs<T> a = ku_args<T>(c, L);
        a.b = (const T*)L.b;
        a.diag = L.diag;
        a.dv = (T*)L.dv;
        a.xout = (T*)L.x;
        a.cheb0 = cf;
        a.cheb = cf + 2;
        a.dv_keep = degree > 2;
        a.done = done;
        ANL_TRY(launch_ku<T>(KU_CHEB0, a, modal_of<T>(c), s));
        k0 = 2;
    } else if (x_is_zero) {
        k_cheb_first<T><<<dim3(vgrid(L.d.nn()), c->rb), VT, 0, s>>>(L.d.nn(), (const T*)L.b, L.diag, L.nmask, cf + 1,
                                                                     (T*)L.x, (T*)L.dv, done, bt_of(c, L));
        ANL_LAUNCH_CHECK();
        k0 = 1;
    }
    for (int k = k0; k < degree; ++k) {
        KuArgs<T> a = ku_args<T>(c, L);
        a.u = (const T*)L.x;
        a.b = (const T*)L.b;
        a.dv = (T*)L.dv;
        a.xout = (T*)L.xt;
        a.cheb = cf + 2 * k;
        a.c1_zero = k == 0;
        a.dv_keep = k + 1 < degree;
        a.done = done;
        ANL_TRY(ku_pass<T>(c, L, KU_CHEB, a, s));
        std::swap(L.x, L.xt);
    }
    return ANL_OK;
}

template <class T>
static int vcycle(anl_ctx* c, size_t l, const int* done, cudaStream_t s);

// One V-cycle step on a level the box kernels (anl_kbox.cu) smooth: the pre-smoothing sweep
// from x = 0 (its first two steps fused), the residual, the restriction, the coarser levels,
// then the post-smoothing sweep whose first step also adds the coarse-grid correction.
static int vcycle_box(anl_ctx* c, size_t l, int deg, const int* done, cudaStream_t s) {
    Level& L = c->lev[l];
    Level& C = c->lev[l + 1];
    const double* cf = c->cheb_d + l * kChebStride + 1;  // (c1, c2) pairs
    KbArgs base;
    base.d = L.d;
    base.E = L.E;
    base.nmask = L.nmask;
    base.diag = L.diag;
    base.b = (const float*)L.b;
    base.done = done;
    base.nrhs = c->rb;
    base.vstride = L.vs;
    base.cstride = C.vs;
    base.sc_bytes = (int)sizeof(PcgScalars);
    int k0 = 0;
    if (deg >= 2) {
        KbArgs a = base;
        a.cheb0 = cf;
        a.cheb = cf + 2;
        a.dv = (float*)L.dv;
        a.xout = (float*)L.x;
        a.dv_keep = deg > 2;
        ANL_TRY(launch_kbox(KB_CHEB0, a, c->kmf, s));
        k0 = 2;
    } else {
        k_cheb_first<float><<<dim3(vgrid(L.d.nn()), c->rb), VT, 0, s>>>(L.d.nn(), (const float*)L.b, L.diag, L.nmask, cf + 1,
                                                            (float*)L.x, (float*)L.dv, done, bt_of(c, L));
        ANL_LAUNCH_CHECK();
        k0 = 1;
    }
    for (int k = k0; k < deg; ++k) {
        KbArgs a = base;
        a.u = (const float*)L.x;
        a.dv = (float*)L.dv;
        a.xout = (float*)L.xt;
        a.cheb = cf + 2 * k;
        a.dv_keep = k + 1 < deg;
        ANL_TRY(launch_kbox(KB_CHEB, a, c->kmf, s));
        std::swap(L.x, L.xt);
    }
    {
        KbArgs a = base;
        a.u = (const float*)L.x;
        a.y = (float*)L.r;
        ANL_TRY(launch_kbox(KB_RESID, a, c->kmf, s));
    }
    k_restrict<float><<<transfer_grid(C.d, c->rb), dim3(TR_X, TR_Y), 0, s>>>(L.d, C.d, (const float*)L.r, C.nmask,
                                                                            (float*)C.b, done, bt_of(c, L, &C));
    ANL_LAUNCH_CHECK();
    ANL_TRY(vcycle<float>(c, l + 1, done, s));
    for (int k = 0; k < deg; ++k) {
        KbArgs a = base;
        a.u = (const float*)L.x;
        a.dv = (float*)L.dv;
        a.xout = (float*)L.xt;
        a.cheb = cf + 2 * k;
        a.c1_zero = k == 0;
        a.dv_keep = k + 1 < deg;
        if (k == 0) {
            a.dc = C.d;
            a.xc = (const float*)C.x;
        }
        ANL_TRY(launch_kbox(k == 0 ? KB_PCHEB : KB_CHEB, a, c->kmf, s));
        std::swap(L.x, L.xt);
    }
    return ANL_OK;
}

// The levels from tail_from down in one CTA per right-hand-side slot: b of level l in, its
// correction x out.
static int vcycle_tail(anl_ctx* c, size_t l, const int* done, cudaStream_t s) {
    TailArgs a;
    a.nlev = (int)(c->lev.size() - l);
    for (int q = 0; q < a.nlev; ++q) {
        const Level& Lq = c->lev[l + q];
        a.lev[q].d = Lq.d;
        a.lev[q].E = Lq.E;
        a.lev[q].nmask = Lq.nmask;
        a.lev[q].diag = Lq.diag;
        a.lev[q].cheb = c->cheb_d + (l + q) * kChebStride + 1;
    }
    a.degree = c->mg_degree_coarse;
    a.b0 = (const float*)c->lev[l].b;
    a.x0 = (float*)c->lev[l].x;
    a.ainv_hi = c->ainv_hi;
    a.ainv_lo = c->ainv_lo;
    a.nc = c->nc;
    a.done = done;
    a.km = c->kmf;
    a.nrhs = c->rb;
    a.vstride = c->lev[l].vs;
    a.sc_bytes = (int)sizeof(PcgScalars);
    return launch_vtail(a, s);
}

template <class T>
static int vcycle(anl_ctx* c, size_t l, const int* done, cudaStream_t s) {
    Level& L = c->lev[l];
    if (sizeof(T) == 4 && c->tail_from >= 0 && (int)l == c->tail_from) return vcycle_tail(c, l, done, s);
    if (l + 1 == c->lev.size()) {
        if (c->dense_coarse) {
            const int n = c->nc;
            k_coarse_apply<T><<<dim3(std::max(1, (n * 32 + 255) / 256), c->rb), 256, 0, s>>>(
                c->Ainv, n, (const T*)L.b, L.nmask, (T*)L.x, done, bt_of(c, L));
            ANL_LAUNCH_CHECK();
            return ANL_OK;
        }
        return smooth<T>(c, L, 16, true, done, s);
    }
    Level& C = c->lev[l + 1];
    const int deg = l >= 2 ? c->mg_degree_coarse : c->mg_degree;
    if (sizeof(T) == 4 && (int)l >= c->box_from) return vcycle_box(c, l, deg, done, s);
    ANL_TRY(smooth<T>(c, L, deg, true, done, s));
    KuArgs<T> a = ku_args<T>(c, L);
    a.u = (const T*)L.x;
    a.b = (const T*)L.b;
    a.y = (T*)L.r;
    a.done = done;
    ANL_TRY(ku_pass<T>(c, L, KU_RESID, a, s));
    k_restrict<T><<<transfer_grid(C.d, c->rb), dim3(TR_X, TR_Y), 0, s>>>(L.d, C.d, (const T*)L.r, C.nmask, (T*)C.b, done,
                                                                        bt_of(c, L, &C));
    ANL_LAUNCH_CHECK();
    ANL_TRY(vcycle<T>(c, l + 1, done, s));
    k_prolong_add<T><<<transfer_grid(C.d, c->rb), dim3(TR_X, TR_Y), 0, s>>>(L.d, C.d, (const T*)C.x, L.nmask, (T*)L.x,
                                                                            done, bt_of(c, L, &C));
    ANL_LAUNCH_CHECK();
    ANL_TRY(smooth<T>(c, L, deg, false, done, s));
    return ANL_OK;
}

// r = b - K x with x in FP64 (ctx->xbuf): the FP64 operator in FP64 mode. In FP32 mode either
// the same FP64 operator in double-float arithmetic (accurate: certifies any rtol down to
// about 1e-10) or the FP32 operator on x = hi + lo (plain: restarts the recurrence). Updates
// the CG state.
__global__ void k_resid_state(PcgScalars* sc, const double* rr, int set_state) {
    const double v = *rr;
    sc->rr_true = v;
    if (set_state) {
        sc->rr = v;
        if (!isfinite(v)) {
            sc->done = 3;
            sc->nonfinite = 1;
        } else {
            sc->done = v <= sc->tol2 ? 1 : 0;
        }
    }
}

template <class T>
static int true_residual(anl_ctx* c, int set_state, cudaStream_t s, bool accurate = true) {
    Level& L0 = c->lev[0];
    const int64_t n = 3 * L0.d.nn();
    T* r = (T*)L0.b;
    if (sizeof(T) == 8) {
        ANL_TRY(apply_level<T>(c, L0, (const T*)(const void*)c->xbuf, (T*)c->y1, s));
        k_true_resid<T><<<vgrid(n), VT, 0, s>>>(n, c->bbuf, (const T*)c->y1, nullptr, r, c->sc, set_state, c->partials,
                                                c->counter);
        ANL_LAUNCH_CHECK();
        return ANL_OK;
    }
    if (!accurate) {
        // plain FP32 evaluation of K x_hi + K x_lo: enough to restart the recurrence, not to
        // certify convergence (its rounding floor is ~eps |K| |dx|)
        k_split_hl<<<vgrid(n), VT, 0, s>>>(n, c->xbuf, (float*)c->xhi, (float*)c->xlo);
        ANL_LAUNCH_CHECK();
        ANL_TRY(apply_level<T>(c, L0, (const T*)c->xhi, (T*)c->y1, s));
        ANL_TRY(apply_level<T>(c, L0, (const T*)c->xlo, (T*)c->y2, s));
        k_true_resid_pair<<<vgrid(n), VT, 0, s>>>(n, (const DF*)c->bdf, (const float*)c->y1, (const float*)c->y2,
                                                  (float*)r, c->sc, set_state, c->partials, c->counter);
        ANL_LAUNCH_CHECK();
        return ANL_OK;
    }
    // r = b - K x of the FP64 modal operator in double-float arithmetic (FP32 residual out)
    k_split_df<<<vgrid(n), VT, 0, s>>>(n, c->xbuf, (DF*)c->xdf);
    ANL_LAUNCH_CHECK();
    KuArgs<DF> a;
    a.d = L0.d;
    a.E = L0.E;
    a.nmask = L0.nmask;
    a.u = (const DF*)c->xdf;
    a.b = (const DF*)c->bdf;
    a.y = (DF*)(void*)r;
    a.partials = c->partials;
    a.counter = c->counter;
    a.partial_capacity = c->part_cap;
    a.red_out = c->red_out + 8;
    ANL_TRY(launch_ku_resid_df(a, c->kmdf, s));
    k_resid_state<<<1, 1, 0, s>>>(c->sc, c->red_out + 8, set_state);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

// `chunk` CG iterations: V-cycle, r.z and z.q, direction update, q = K p with p.q, then the
// x / r update with ||r||^2. Every kernel returns early once the device "done" flag is set.
template <class T>
static int enqueue_chunk(anl_ctx* c, int chunk, cudaStream_t s) {
    Level& L0 = c->lev[0];
    const int64_t n = 3 * L0.d.nn();
    int* restart = c->restart_d + c->slot;
    const int* done = &c->sc->done;
    const Bt bt = bt_of(c, L0);
    const dim3 vg(vgrid(n), c->rb);
    for (int k = 0; k < chunk; ++k) {
        ANL_TRY(vcycle<T>(c, 0, done, s));
        const T* z = (const T*)L0.x;
        k_dots_rz_zq<T><<<vg, VT, 0, s>>>(n, (const T*)L0.b, z, (const T*)c->q, c->sc, restart, c->partials,
                                           c->counter, bt);
        ANL_LAUNCH_CHECK();
        k_pupdate<T><<<vg, VT, 0, s>>>(n, z, (T*)c->p, c->sc, restart, bt);
        ANL_LAUNCH_CHECK();
        ANL_TRY(apply_level<T>(c, L0, (const T*)c->p, (T*)c->q, s, &c->sc->pq, done));
        k_axpy<T><<<vg, VT, 0, s>>>(n, (const T*)c->p, (const T*)c->q, c->xbuf, (T*)L0.b, c->sc, restart,
                                    c->partials, c->counter, bt);
        ANL_LAUNCH_CHECK();
    }
    return ANL_OK;
}

// Captures enqueue_chunk into a graph on the context's own stream (the caller's stream may
// be the legacy default stream, which cannot be captured). The V-cycle's buffer swaps come
// back to their starting state after an even number of cycles, so the captured pointers
// stay valid for every replay.
template <class T>
static int capture_chunk(anl_ctx* c, int chunk) {
    if (c->cg_exec) {
        cudaGraphExecDestroy(c->cg_exec);
        c->cg_exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    ANL_CUDA(cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
    const int st = enqueue_chunk<T>(c, chunk, c->cap_stream);
    const cudaError_t e = cudaStreamEndCapture(c->cap_stream, &g);
    if (st != ANL_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) {
        set_error("CG graph capture failed: %s", cudaGetErrorString(e));
        return ANL_ERR_CUDA;
    }
    size_t nodes = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    const cudaError_t ei = cudaGraphInstantiate(&c->cg_exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        set_error("CG graph instantiation failed: %s", cudaGetErrorString(ei));
        c->cg_exec = nullptr;
        return ANL_ERR_CUDA;
    }
    c->cg_nodes = (int)nodes;
    c->cg_valid = true;
    c->cg_rb = c->rb;
    return ANL_OK;
}

template <class T>
static int pcg_one(anl_ctx* c, const double* f, double* x, double rtol, int maxiter, int* iters, double* relres,
                   cudaStream_t s) {
    Level& L0 = c->lev[0];
    const int64_t nn = L0.d.nn(), n = 3 * nn;
    int* restart = c->restart_d + c->slot;
    k_mask_copy_d<<<vgrid(nn), VT, 0, s>>>(nn, f, L0.nmask, c->bbuf);
    ANL_LAUNCH_CHECK();
    k_mask_copy_d<<<vgrid(nn), VT, 0, s>>>(nn, x, L0.nmask, c->xbuf);
    ANL_LAUNCH_CHECK();
    if (sizeof(T) == 4) {  // the right-hand side of the accurate residual, split once per solve
        k_split_df<<<vgrid(n), VT, 0, s>>>(n, c->bbuf, (DF*)c->bdf);
        ANL_LAUNCH_CHECK();
    }
    k_dot_d<<<vgrid(n), VT, 0, s>>>(n, c->bbuf, c->bbuf, c->partials, c->counter, c->red_out);
    ANL_LAUNCH_CHECK();
    k_init_scalars<<<1, 1, 0, s>>>(c->sc, rtol, maxiter, c->red_out);
    ANL_LAUNCH_CHECK();
    ANL_TRY(true_residual<T>(c, 1, s, false));
    const int one = 1;
    ANL_CUDA(cudaMemcpyAsync(restart, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    ANL_CUDA(cudaMemcpyAsync(c->sc_h, c->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
    ANL_CUDA(cudaStreamSynchronize(s));
    if (c->sc_h->done == 1 && sizeof(T) == 4) {  // certify an already-converged initial guess
        ANL_TRY(true_residual<T>(c, 1, s, true));
        ANL_CUDA(cudaMemcpyAsync(c->sc_h, c->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
        ANL_CUDA(cudaStreamSynchronize(s));
    }
    *iters = 0;
    if (c->sc_h->bb == 0.0) {
        ANL_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
        *relres = 0.0;
        return ANL_OK;
    }
    static const bool trace = std::getenv("ANL_TRACE") != nullptr;  // solver trace on stderr
    int last_replace = 0;
    double rr_replace = c->sc_h->rr;  // ||r||^2 at the last replacement
    double stag_ref = -1.0;            // true ||r||^2 when the recurrence first claimed convergence
    int status = ANL_OK;
    const int chunk = 4;  // even: the V-cycle buffer swaps return to their start (graph replay)
    // (done == 1 here: the initial guess already satisfies the tolerance)
    while (c->sc_h->done != 1) {
        if (c->sc_h->done == 0) {
            if (c->use_graph) {
                if (!c->cg_valid || c->cg_rb != c->rb) ANL_TRY(capture_chunk<T>(c, chunk));
                ANL_CUDA(cudaGraphLaunch(c->cg_exec, s));
                count_launches(c->cg_nodes);
            } else {
                ANL_TRY(enqueue_chunk<T>(c, chunk, s));
            }
            ANL_CUDA(cudaMemcpyAsync(c->sc_h, c->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
            ANL_CUDA(cudaStreamSynchronize(s));
        }
        const PcgScalars h = *c->sc_h;
        if (h.done == 3) {
            if (trace)
                std::fprintf(stderr, "[anl cg] it %d non-finite: rz %.3e pq %.3e zq %.3e rr %.3e alpha %.3e\n", h.iters,
                             h.rz[h.iters & 1], h.pq, h.zq, h.rr, h.alpha);
            status = ANL_ERR_NONFINITE;
            break;
        }
        // Replace the recurrence residual by the true one when the recurrence claims
        // convergence, runs out of iterations or breaks down, every 50 iterations, and
        // whenever ||r|| has dropped 1000x since the last replacement (reliable updates),
        // unless it is already within 10 rtol: the certification follows a few iterations
        // later and replaces it then.
        const bool want_check = h.done == 1 || h.done == 2 || h.done == 4 || h.iters - last_replace >= 50 ||
                                (h.rr <= 1e-6 * rr_replace && h.rr > 100.0 * h.tol2);
        if (!want_check) continue;
        // Every replacement takes the accurate residual of the FP64 operator. The FP32
        // operator differs from them by a few eps in every element force, which leaves a
        // residual of several rtol in high-frequency modes at the end of an FP32 recurrence.
        // Taking the accurate residual already at the mid-solve replacement lets the
        // iteration remove that part on the way, so the final certification passes at the
        // first attempt (with the plain residual there, the first certification failed in
        // every solve and cost a second certification and two more iterations).
        ANL_TRY(true_residual<T>(c, 1, s, true));
        ANL_CUDA(cudaMemcpyAsync(c->sc_h, c->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
        ANL_CUDA(cudaStreamSynchronize(s));
        const PcgScalars& t = *c->sc_h;
        if (trace)
            std::fprintf(stderr, "[anl cg] it %d state %d rec %.3e true %.3e (rel, tol %.1e)\n", t.iters, h.done,
                         std::sqrt(h.rr / t.bb), std::sqrt(t.rr_true / t.bb), rtol);
        last_replace = t.iters;
        rr_replace = t.rr_true;
        if (t.done == 1) break;  // certified on the true residual
        if (t.done == 3) {
            status = ANL_ERR_NONFINITE;
            break;
        }
        // At the attainable accuracy of the operator's arithmetic the true residual stops
        // falling while the recurrence keeps converging (the reference's scipy CG stops on
        // the recurrence alone and never sees this floor). In FP64 a solve is accepted once
        // a further round of iterations has not halved the true residual, if it is within
        // max(100 rtol, 1e-10) relative (the reported relres then exceeds rtol). An FP32
        // solve that stops falling above rtol returns ANL_ERR_STAGNATION instead, so the
        // caller can finish it in FP64: FP32 results always meet rtol.
        const double floor2 = std::max(1e4 * t.tol2, 1e-20 * t.bb);
        if (h.done == 1 || h.done == 4) {
            const bool stalled = stag_ref > 0 && t.rr_true >= 0.25 * stag_ref;
            if (stalled && sizeof(T) == 4) {
                status = ANL_ERR_STAGNATION;
                break;
            }
            if (stalled && t.rr_true <= floor2) break;
            if (stag_ref < 0 || t.rr_true < stag_ref) stag_ref = t.rr_true;
            if (h.done == 4 && t.rr_true > floor2) {
                status = ANL_ERR_BREAKDOWN;
                break;
            }
        }
        if (t.iters >= maxiter) {
            status = ANL_ERR_MAXITER;
            break;
        }
        // not converged: the replaced residual carries on; restart the directions after a
        // breakdown
        if (h.done == 4) {
            const int one_r = 1;
            ANL_CUDA(cudaMemcpyAsync(restart, &one_r, sizeof(int), cudaMemcpyHostToDevice, s));
        }
    }
    *iters = c->sc_h->iters;
    *relres = c->sc_h->bb > 0 ? std::sqrt(std::max(c->sc_h->rr_true, 0.0) / c->sc_h->bb) : 0.0;
    ANL_CUDA(cudaMemcpyAsync(x, c->xbuf, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return status;
}

// ------------------------------------------------------------------ entry points used by the C API

int solver_setup_domain(anl_ctx* c, const uint8_t* active, const uint8_t* fixed, cudaStream_t s) {
    Level& L0 = c->lev[0];
    ANL_CUDA(cudaMemcpyAsync(c->active, active, L0.d.ne(), cudaMemcpyDeviceToDevice, s));
    ANL_CUDA(cudaMemcpyAsync(L0.eact, active, L0.d.ne(), cudaMemcpyDeviceToDevice, s));
    k_mask_level0<<<vgrid(L0.d.nn()), VT, 0, s>>>(L0.d, active, fixed, L0.nmask);
    ANL_LAUNCH_CHECK();
    for (size_t l = 1; l < c->lev.size(); ++l) {
        Level& F = c->lev[l - 1];
        Level& C = c->lev[l];
        k_eact_coarse<<<vgrid(C.d.ne()), VT, 0, s>>>(F.d, C.d, F.eact, C.eact);
        ANL_LAUNCH_CHECK();
        k_mask_coarse<<<vgrid(C.d.nn()), VT, 0, s>>>(F.d, C.d, F.nmask, C.eact, C.nmask);
        ANL_LAUNCH_CHECK();
    }
    k_count_free<<<vgrid(L0.d.nn()), VT, 0, s>>>(L0.d.nn(), L0.nmask, c->partials, c->counter, c->red_out);
    ANL_LAUNCH_CHECK();
    ANL_CUDA(cudaMemcpyAsync(c->red_h, c->red_out, sizeof(double), cudaMemcpyDeviceToHost, s));
    ANL_CUDA(cudaStreamSynchronize(s));
    c->nfree = (int64_t)c->red_h[0];
    c->domain_set = true;
    c->coarse_ready = false;
    return ANL_OK;
}

int solver_set_escale(anl_ctx* c, const float* escale, cudaStream_t s) {
    Level& L0 = c->lev[0];
    k_level0_E<<<vgrid(L0.d.ne()), VT, 0, s>>>(L0.d.ne(), escale, c->active, (float)c->h, L0.E);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int solver_apply(anl_ctx* c, const float* escale, const void* u, void* y, cudaStream_t s) {
    ANL_TRY(solver_set_escale(c, escale, s));
    Level& L0 = c->lev[0];
    const int64_t nn = L0.d.nn();
    if (c->fp64) {
        k_mask_copy_t<double><<<vgrid(nn), VT, 0, s>>>(nn, (const double*)u, L0.nmask, (double*)c->tmp);
        ANL_LAUNCH_CHECK();
        return apply_level<double>(c, L0, (const double*)c->tmp, (double*)y, s);
    }
    k_mask_copy_t<float><<<vgrid(nn), VT, 0, s>>>(nn, (const float*)u, L0.nmask, (float*)c->tmp);
    ANL_LAUNCH_CHECK();
    return apply_level<float>(c, L0, (const float*)c->tmp, (float*)y, s);
}

// The R right-hand sides of a batch (FP32 contexts, R <= rmax) solved together: every kernel of
// the CG chunk (the V-cycle on all levels, the dot products, the direction and solution updates,
// q = K p) runs once for all slots, each slot with its own FP64 scalars, so one captured graph
// advances all of them in lockstep and a converged slot's kernels return at once. The
// per-slot steps outside the chunk (set-up, residual replacements, certification on the FP64
// operator's accurate residual, the acceptance rules) are those of pcg_one, slot by slot.
// statuses[r] receives each slot's status.
template <class T>
static int pcg_batch(anl_ctx* c, int R, const double* f, double* x, double rtol, int maxiter, int* iters,
                     double* relres, int* statuses, cudaStream_t s) {
    Level& L0 = c->lev[0];
    const int64_t nn = L0.d.nn(), n = 3 * nn;
    const int one = 1;
    struct SlotState {
        bool active = true;
        int last_replace = 0;
        double rr_replace = 0.0, stag_ref = -1.0;
        int status = ANL_OK;
    };
    std::vector<SlotState> st(R);
    for (int r = 0; r < R; ++r) {  // set-up, as pcg_one
        set_slot(c, r);
        k_mask_copy_d<<<vgrid(nn), VT, 0, s>>>(nn, f + r * n, L0.nmask, c->bbuf);
        ANL_LAUNCH_CHECK();
        k_mask_copy_d<<<vgrid(nn), VT, 0, s>>>(nn, x + r * n, L0.nmask, c->xbuf);
        ANL_LAUNCH_CHECK();
        k_split_df<<<vgrid(n), VT, 0, s>>>(n, c->bbuf, (DF*)c->bdf);
        ANL_LAUNCH_CHECK();
        k_dot_d<<<vgrid(n), VT, 0, s>>>(n, c->bbuf, c->bbuf, c->partials, c->counter, c->red_out);
        ANL_LAUNCH_CHECK();
        k_init_scalars<<<1, 1, 0, s>>>(c->sc, rtol, maxiter, c->red_out);
        ANL_LAUNCH_CHECK();
        ANL_TRY(true_residual<T>(c, 1, s, false));
        ANL_CUDA(cudaMemcpyAsync(c->restart_d + r, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    }
    set_slot(c, 0);
    auto fetch = [&](int r) -> int {  // host copy of slot r's scalars
        ANL_CUDA(cudaMemcpyAsync(c->sc_h + r, c->sc_base + r, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
        ANL_CUDA(cudaStreamSynchronize(s));
        return ANL_OK;
    };
    auto finish = [&](int r, int status) -> int {  // slot r leaves the batch: its kernels stop
        st[r].active = false;
        st[r].status = status;
        const int stop = 5;
        ANL_CUDA(cudaMemcpyAsync(&c->sc_base[r].done, &stop, sizeof(int), cudaMemcpyHostToDevice, s));
        return ANL_OK;
    };
    ANL_CUDA(cudaMemcpyAsync(c->sc_h, c->sc_base, R * sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
    ANL_CUDA(cudaStreamSynchronize(s));
    for (int r = 0; r < R; ++r) {
        PcgScalars& h = c->sc_h[r];
        if (h.bb == 0.0) {  // zero load: zero solution
            ANL_CUDA(cudaMemsetAsync(c->xbuf_base + r * L0.vs, 0, n * sizeof(double), s));
            ANL_TRY(finish(r, ANL_OK));
            continue;
        }
        if (h.done == 1) {  // certify an already-converged initial guess
            set_slot(c, r);
            ANL_TRY(true_residual<T>(c, 1, s, true));
            set_slot(c, 0);
            ANL_TRY(fetch(r));
            if (c->sc_h[r].done == 1) ANL_TRY(finish(r, ANL_OK));
        }
        st[r].rr_replace = c->sc_h[r].rr;
    }
    const int chunk = 4;  // even: the V-cycle buffer swaps return to their start (graph replay)
    while (true) {
        bool any_active = false, any_running = false;
        for (int r = 0; r < R; ++r)
            if (st[r].active) {
                any_active = true;
                any_running |= c->sc_h[r].done == 0;
            }
        if (!any_active) break;
        if (any_running) {
            c->rb = R;
            int e;
            if (c->use_graph) {
                e = ANL_OK;
                if (!c->cg_valid || c->cg_rb != c->rb) e = capture_chunk<T>(c, chunk);
                if (e == ANL_OK) {
                    const cudaError_t ce = cudaGraphLaunch(c->cg_exec, s);
                    if (ce != cudaSuccess) {
                        set_error("CG graph launch failed: %s", cudaGetErrorString(ce));
                        e = ANL_ERR_CUDA;
                    }
                    count_launches(c->cg_nodes);
                }
            } else {
                e = enqueue_chunk<T>(c, chunk, s);
            }
            c->rb = 1;
            ANL_TRY(e);
            ANL_CUDA(cudaMemcpyAsync(c->sc_h, c->sc_base, R * sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
            ANL_CUDA(cudaStreamSynchronize(s));
        }
        for (int r = 0; r < R; ++r) {
            if (!st[r].active) continue;
            const PcgScalars h = c->sc_h[r];
            if (h.done == 3) {
                ANL_TRY(finish(r, ANL_ERR_NONFINITE));
                continue;
            }
            const bool want_check = h.done == 1 || h.done == 2 || h.done == 4 || h.iters - st[r].last_replace >= 50 ||
                                    (h.rr <= 1e-6 * st[r].rr_replace && h.rr > 100.0 * h.tol2);
            if (!want_check) continue;
            set_slot(c, r);
            ANL_TRY(true_residual<T>(c, 1, s, true));
            set_slot(c, 0);
            ANL_TRY(fetch(r));
            const PcgScalars& t = c->sc_h[r];
            st[r].last_replace = t.iters;
            st[r].rr_replace = t.rr_true;
            if (t.done == 1) {
                st[r].active = false;  // certified (done stays 1: its kernels return)
                continue;
            }
            if (t.done == 3) {
                ANL_TRY(finish(r, ANL_ERR_NONFINITE));
                continue;
            }
            const double floor2 = std::max(1e4 * t.tol2, 1e-20 * t.bb);
            if (h.done == 1 || h.done == 4) {
                const bool stalled = st[r].stag_ref > 0 && t.rr_true >= 0.25 * st[r].stag_ref;
                if (stalled && sizeof(T) == 4) {
                    ANL_TRY(finish(r, ANL_ERR_STAGNATION));
                    continue;
                }
                if (stalled && t.rr_true <= floor2) {
                    ANL_TRY(finish(r, ANL_OK));
                    continue;
                }
                if (st[r].stag_ref < 0 || t.rr_true < st[r].stag_ref) st[r].stag_ref = t.rr_true;
                if (h.done == 4 && t.rr_true > floor2) {
                    ANL_TRY(finish(r, ANL_ERR_BREAKDOWN));
                    continue;
                }
            }
            if (t.iters >= maxiter) {
                ANL_TRY(finish(r, ANL_ERR_MAXITER));
                continue;
            }
            if (h.done == 4) ANL_CUDA(cudaMemcpyAsync(c->restart_d + r, &one, sizeof(int), cudaMemcpyHostToDevice, s));
        }
    }
    ANL_CUDA(cudaMemcpyAsync(c->sc_h, c->sc_base, R * sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
    ANL_CUDA(cudaStreamSynchronize(s));
    for (int r = 0; r < R; ++r) {
        const PcgScalars& h = c->sc_h[r];
        iters[r] = h.iters;
        relres[r] = h.bb > 0 ? std::sqrt(std::max(h.rr_true, 0.0) / h.bb) : 0.0;
        statuses[r] = st[r].status;
        ANL_CUDA(cudaMemcpyAsync(x + r * n, c->xbuf_base + r * L0.vs, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    return ANL_OK;
}

int solver_solve(anl_ctx* c, const float* escale, const double* f, double* x, int nrhs, double rtol, int maxiter,
                 int rebuild, int* iters, double* relres, cudaStream_t s) {
    ANL_TRY(solver_set_escale(c, escale, s));
    if (c->fp64) ANL_TRY(update_hierarchy<double>(c, rebuild != 0, s));
    else ANL_TRY(update_hierarchy<float>(c, rebuild != 0, s));
    const int64_t n = 3 * c->lev[0].d.nn();
    int worst = ANL_OK;
    set_slot(c, 0);
    if (!c->fp64 && nrhs > 1 && nrhs <= c->rmax) {
        std::vector<int> sts(nrhs, ANL_OK);
        ANL_TRY(pcg_batch<float>(c, nrhs, f, x, rtol, maxiter, iters, relres, sts.data(), s));
        for (int k = 0; k < nrhs; ++k)
            if (sts[k] != ANL_OK && worst == ANL_OK) worst = sts[k];
        c->last_status.assign(sts.begin(), sts.end());
    } else {
        c->last_status.assign(nrhs, ANL_OK);
        for (int k = 0; k < nrhs; ++k) {
            int st = c->fp64 ? pcg_one<double>(c, f + k * n, x + k * n, rtol, maxiter, iters + k, relres + k, s)
                             : pcg_one<float>(c, f + k * n, x + k * n, rtol, maxiter, iters + k, relres + k, s);
            if (st == ANL_ERR_CUDA) return st;
            c->last_status[k] = st;
            if (st != ANL_OK && worst == ANL_OK) worst = st;
        }
    }
    if (worst == ANL_ERR_MAXITER) set_error("CG did not reach rtol %.3g in %d iterations", rtol, maxiter);
    if (worst == ANL_ERR_NONFINITE) set_error("a non-finite value appeared in CG");
    if (worst == ANL_ERR_BREAKDOWN) set_error("CG breakdown: the operator is not positive definite on the free DOFs");
    if (worst == ANL_ERR_STAGNATION)
        set_error("FP32 CG stopped improving above rtol %.3g (finish the solve in FP64)", rtol);
    return worst;
}

// Times one finest-level pass of the solve, `reps` launches between two CUDA events on s, on
// the context's own work vectors (their contents are whatever the last solve left; the timed
// passes overwrite the V-cycle scratch, which the next solve re-initialises). FP32 contexts.
int solver_profile_pass(anl_ctx* c, int pass, int reps, double* ms, cudaStream_t s) {
    if (c->fp64) {
        set_error("profile pass: FP32 contexts only");
        return ANL_ERR_BADARG;
    }
    Level& L = c->lev[0];
    const double* cf = c->cheb_d + 1;  // level 0 (c1, c2) pairs
    KuArgs<float> a = ku_args<float>(c, L);
    int mode = KU_APPLY;
    switch (pass) {
        case 0: a.u = (const float*)c->p; a.y = (float*)c->q; mode = KU_APPLY; break;
        case 1: a.u = (const float*)c->p; a.y = (float*)c->q; a.red_out = c->red_out + 12; mode = KU_APPLY_DOT; break;
        case 2: a.u = (const float*)L.x; a.b = (const float*)L.b; a.y = (float*)L.r; mode = KU_RESID; break;
        case 3:
            a.u = (const float*)L.x; a.b = (const float*)L.b; a.dv = (float*)L.dv; a.xout = (float*)L.xt;
            a.cheb = cf + 2; a.c1_zero = 0; a.dv_keep = 0; mode = KU_CHEB;  // the last step of a sweep
            break;
        case 5:
            a.u = (const float*)L.x; a.b = (const float*)L.b; a.dv = (float*)L.dv; a.xout = (float*)L.xt;
            a.cheb = cf; a.c1_zero = 1; a.dv_keep = 1; mode = KU_CHEB;  // the first step of a sweep from x != 0
            break;
        case 4:
            a.b = (const float*)L.b; a.diag = L.diag; a.dv = (float*)L.dv; a.xout = (float*)L.x;
            // as the V-cycle runs it: the direction is kept only for a sweep of more than 2 steps
            a.cheb0 = cf; a.cheb = cf + 2; a.dv_keep = c->mg_degree > 2; mode = KU_CHEB0;
            break;
        default: set_error("profile pass: unknown pass %d", pass); return ANL_ERR_BADARG;
    }
    cudaEvent_t e0, e1;
    ANL_CUDA(cudaEventCreate(&e0));
    ANL_CUDA(cudaEventCreate(&e1));
    ANL_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < reps; ++r) ANL_TRY(ku_pass<float>(c, L, mode, a, s));
    ANL_CUDA(cudaEventRecord(e1, s));
    ANL_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    ANL_CUDA(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = (double)t / reps;
    return ANL_OK;
}

int solver_profile_apply(anl_ctx* c, const void* u, void* y, int reps, double* ms, cudaStream_t s) {
    cudaEvent_t e0, e1;
    ANL_CUDA(cudaEventCreate(&e0));
    ANL_CUDA(cudaEventCreate(&e1));
    ANL_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < reps; ++r) {
        int st = c->fp64 ? apply_level<double>(c, c->lev[0], (const double*)u, (double*)y, s)
                         : apply_level<float>(c, c->lev[0], (const float*)u, (float*)y, s);
        if (st != ANL_OK) return st;
    }
    ANL_CUDA(cudaEventRecord(e1, s));
    ANL_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    ANL_CUDA(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = (double)t / reps;
    return ANL_OK;
}

int solver_dot(anl_ctx* c, const double* a, const double* b, double* out, cudaStream_t s) {
    const int64_t n = 3 * c->lev[0].d.nn();
    k_dot_d<<<vgrid(n), VT, 0, s>>>(n, a, b, c->partials, c->counter, c->red_out);
    ANL_LAUNCH_CHECK();
    ANL_CUDA(cudaMemcpyAsync(c->red_h, c->red_out, sizeof(double), cudaMemcpyDeviceToHost, s));
    ANL_CUDA(cudaStreamSynchronize(s));
    *out = c->red_h[0];
    return ANL_OK;
}

ANL_DEBUG_UNIT(solver)

}  // namespace anl
