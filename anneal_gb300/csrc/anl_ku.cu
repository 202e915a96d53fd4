// anl_ku.cu -- matrix-free hex8 operator K u and the kernels fused with it.
//
// Replaces the assembled CSR matrix of FEM.assemble (fem.py:198-201) and its SpMV inside
// scipy's CG (fem.py:224). K = sum_e E_e Ke acts node by node (gather form, no atomics):
//
//   (K u)_n = sum_{octants o} E_o * S_o * sum_{delta != 0} B0(delta) * S_o * (u_{n + o.delta} - u_n)
//
// o in {-1,+1}^3 picks the element around node n, S_o = diag(o), B0 are the 8 base 3x3
// blocks of Ke (anl_common.cuh). The difference form uses the zero block-row sums of Ke;
// it keeps FP32 products proportional to the local strain rather than to |u|, which is
// what lets the FP32 operator resolve residuals far below |K| |u| eps.
//
// Tiling: a CTA of 32x8 threads owns a 32x8 column of nodes and marches up a chunk of
// z-layers, keeping three node planes (with a one-node halo) and two element planes in
// shared memory. HBM traffic is u once, y once, E once and the node mask once.
#include <algorithm>

#include "anl_common.cuh"
#include "anl_kernels.cuh"

namespace anl {

constexpr int KU_BX = 32, KU_BY = 8;
constexpr int KU_HX = KU_BX + 2, KU_HY = KU_BY + 2;
constexpr int KU_EX = KU_BX + 1, KU_EY = KU_BY + 1;
constexpr int KU_NT = KU_BX * KU_BY;

template <class T>
struct DotAcc;
template <>
struct DotAcc<float> {
    Acc2 a;
    __device__ void add(float x, float y) { a.add_prod(x, y); }
    __device__ double value() const { return a.value(); }
};
template <>
struct DotAcc<double> {
    double s = 0.0;
    __device__ void add(double x, double y) { s = fma(x, y, s); }
    __device__ double value() const { return s; }
};

constexpr int KU_NSLOT = 4;                                            // node-plane ring
constexpr int KU_ESLOT = 3;                                            // element-layer ring
constexpr int KU_PLANE = KU_HY * KU_HX * 3;                            // values per node plane
constexpr int KU_EPLANE = KU_EY * KU_EX;                               // values per element layer
constexpr int KU_NLOAD = (KU_PLANE + KU_NT - 1) / KU_NT;               // loads per thread per plane
constexpr int KU_ELOAD = (KU_EPLANE + KU_NT - 1) / KU_NT;

// Pipelining: while a CTA computes node layer k it holds layers k-1..k+1 (and element layers
// k-1, k) in a 4-slot / 3-slot ring, and the loads of layer k+2 (element layer k+1) are in
// flight into registers; they are stored into the free slot after the compute, and one
// barrier per layer publishes them. Each thread's load slots (shared-memory index and offset
// within a plane) are computed once.
#ifndef KU_MINB
#define KU_MINB 3  // resident CTAs per SM the register allocation is sized for
#endif

template <class T, int MODE>
__global__ void __launch_bounds__(KU_NT, (sizeof(T) == 8 ? 2 : KU_MINB)) ku_kernel(KuArgs<T> a, KeBlocks<T> kb) {
    __shared__ T su[KU_NSLOT][KU_PLANE];
    __shared__ float sE[KU_ESLOT][KU_EPLANE];
    __shared__ double sred[KU_NT / 32];
    if (a.done != nullptr && *a.done) return;

    const Dims d = a.d;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * KU_BX + tx;
    const int i0 = blockIdx.x * KU_BX, j0 = blockIdx.y * KU_BY, k0 = blockIdx.z * a.kz;
    const int NXn = d.nx + 1, NYn = d.ny + 1, NZn = d.nz + 1;
    const int64_t nplane = 3 * (int64_t)NXn * NYn, eplane = (int64_t)d.nx * d.ny;

    int noff[KU_NLOAD];   // offset within a node plane (3*node + c), -1 outside the grid
    int eoff[KU_ELOAD];   // offset within an element layer, -1 outside
#pragma unroll
    for (int q = 0; q < KU_NLOAD; ++q) {
        const int f = tid + q * KU_NT;
        noff[q] = -1;
        if (f < KU_PLANE) {
            const int row = f / (KU_HX * 3), w = f - row * (KU_HX * 3);
            const int c = w / 3, comp = w - 3 * c;
            const int gi = i0 - 1 + c, gj = j0 - 1 + row;
            if (gi >= 0 && gi < NXn && gj >= 0 && gj < NYn) noff[q] = 3 * (gi + NXn * gj) + comp;
        }
    }
#pragma unroll
    for (int q = 0; q < KU_ELOAD; ++q) {
        const int f = tid + q * KU_NT;
        eoff[q] = -1;
        if (f < KU_EPLANE) {
            const int row = f / KU_EX, c = f - row * KU_EX;
            const int gi = i0 - 1 + c, gj = j0 - 1 + row;
            if (gi >= 0 && gi < d.nx && gj >= 0 && gj < d.ny) eoff[q] = gi + d.nx * gj;
        }
    }
    T rn[KU_NLOAD];
    float re[KU_ELOAD];
    auto fetch = [&](int kk, int ke) {
        const bool kin = kk >= 0 && kk < NZn, ein = ke >= 0 && ke < d.nz;
        const T* up = a.u + (int64_t)kk * nplane;
        const float* ep = a.E + (int64_t)ke * eplane;
#pragma unroll
        for (int q = 0; q < KU_NLOAD; ++q) rn[q] = (kin && noff[q] >= 0) ? up[noff[q]] : T(0);
#pragma unroll
        for (int q = 0; q < KU_ELOAD; ++q) re[q] = (ein && eoff[q] >= 0) ? ep[eoff[q]] : 0.f;
    };
    auto store_nodes = [&](int slot) {
#pragma unroll
        for (int q = 0; q < KU_NLOAD; ++q)
            if (tid + q * KU_NT < KU_PLANE) su[slot][tid + q * KU_NT] = rn[q];
    };
    auto store_elems = [&](int slot) {
#pragma unroll
        for (int q = 0; q < KU_ELOAD; ++q)
            if (tid + q * KU_NT < KU_EPLANE) sE[slot][tid + q * KU_NT] = re[q];
    };

    // prologue: node planes k0-1, k0, k0+1 -> slots 0, 1, 2; element layers k0-1, k0 -> 0, 1
    fetch(k0 - 1, k0 - 1);
    store_nodes(0);
    store_elems(0);
    fetch(k0, k0);
    store_nodes(1);
    store_elems(1);
    fetch(k0 + 1, -1);
    store_nodes(2);
    __syncthreads();

    DotAcc<T> dot;
    const int i = i0 + tx, j = j0 + ty;
    const int kend = min(k0 + a.kz, NZn);
    for (int k = k0; k < kend; ++k) {
        const int r = k - k0;
        const int s_lo = r & 3, s_mid = (r + 1) & 3, s_hi = (r + 2) & 3, s_next = (r + 3) & 3;
        const int e_lo = r % 3, e_hi = (r + 1) % 3, e_next = (r + 2) % 3;
        const bool more = k + 1 < kend;
        if (more) fetch(k + 2, k + 1);   // in flight during the compute below
        if (i < NXn && j < NYn) {
            const T* base[3] = {su[s_lo], su[s_mid], su[s_hi]};
            const float* Elo = sE[e_lo];
            const float* Ehi = sE[e_hi];
            T un[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) un[c] = base[1][((ty + 1) * KU_HX + tx + 1) * 3 + c];
            T dl[3][3][3][3];
#pragma unroll
            for (int mz = 0; mz < 3; ++mz)
#pragma unroll
                for (int my = 0; my < 3; ++my)
#pragma unroll
                    for (int mx = 0; mx < 3; ++mx) {
                        const T* p = base[mz] + ((ty + my) * KU_HX + (tx + mx)) * 3;
#pragma unroll
                        for (int c = 0; c < 3; ++c) dl[mz][my][mx][c] = p[c] - un[c];
                    }
            T y[3] = {T(0), T(0), T(0)};
            float esum = 0.f;
#pragma unroll
            for (int oct = 0; oct < 8; ++oct) {
                const int sx = (oct & 1) ? 1 : -1, sy = (oct & 2) ? 1 : -1, sz = (oct & 4) ? 1 : -1;
                const float Eo = (sz > 0 ? Ehi : Elo)[(ty + (sy > 0 ? 1 : 0)) * KU_EX + tx + (sx > 0 ? 1 : 0)];
                esum += Eo;
                T w[3] = {T(0), T(0), T(0)};
#pragma unroll
                for (int dlt = 1; dlt < 8; ++dlt) {
                    const int dx = dlt & 1, dy = (dlt >> 1) & 1, dz = (dlt >> 2) & 1;
                    const T* dv = dl[1 + sz * dz][1 + sy * dy][1 + sx * dx];
                    const T t0 = sx > 0 ? dv[0] : -dv[0];
                    const T t1 = sy > 0 ? dv[1] : -dv[1];
                    const T t2 = sz > 0 ? dv[2] : -dv[2];
                    const T* B = kb.blk[dlt];
#pragma unroll
                    for (int rr = 0; rr < 3; ++rr) w[rr] += B[3 * rr] * t0 + B[3 * rr + 1] * t1 + B[3 * rr + 2] * t2;
                }
                const T Et = T(Eo);
                y[0] += sx > 0 ? Et * w[0] : -Et * w[0];
                y[1] += sy > 0 ? Et * w[1] : -Et * w[1];
                y[2] += sz > 0 ? Et * w[2] : -Et * w[2];
            }
            const int64_t n = d.node(i, j, k);
            const uint8_t nm = a.nmask[n];
            if (MODE == KU_APPLY || MODE == KU_APPLY_DOT) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const T v = (nm >> c) & 1 ? y[c] : T(0);
                    a.y[3 * n + c] = v;
                    if (MODE == KU_APPLY_DOT) dot.add(un[c], v);
                }
            } else if (MODE == KU_RESID) {
#pragma unroll
                for (int c = 0; c < 3; ++c) a.y[3 * n + c] = (nm >> c) & 1 ? a.b[3 * n + c] - y[c] : T(0);
            } else if (MODE == KU_CHEB) {
                const T inv = esum > 0.f ? T(1) / (a.kdiag * T(esum)) : T(0);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    T dn = T(0), xn = T(0);
                    if ((nm >> c) & 1) {
                        const T rc = a.b[3 * n + c] - y[c];
                        dn = (a.c1 != T(0) ? a.c1 * a.dv[3 * n + c] : T(0)) + a.c2 * rc * inv;
                        xn = un[c] + dn;
                    }
                    a.dv[3 * n + c] = dn;
                    a.xout[3 * n + c] = xn;
                }
            }
        }
        if (more) {
            store_nodes(s_next);
            store_elems(e_next);
        }
        __syncthreads();
    }
    if (MODE == KU_APPLY_DOT) {
        double v[1] = {dot.value()};
        block_sum<1, KU_NT>(v, sred, tid);
        const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        finish_reduction<1, KU_NT>(v, bid, gridDim.x * gridDim.y * gridDim.z, a.partials, a.counter, a.red_out, tid,
                                   sred);
    }
}

// z-chunking: the CTA count is a near multiple of the resident CTAs (occupancy x SMs), so
// the last wave is full; chunks stay at least 4 layers deep (2 halo layers per chunk).
template <class T, int MODE>
static int ku_chunks(int columns, int NZn) {
    static int resident = 0;
    if (resident == 0) {
        int dev = 0, sms = 1, occ = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ku_kernel<T, MODE>, KU_NT, 0);
        resident = std::max(1, sms * std::max(1, occ));
    }
    int best = 1;
    double best_score = -1.0;
    for (int c = 1; c <= std::max(1, NZn / 4); ++c) {
        const int kz = ceil_div(NZn, c);
        const int64_t blocks = (int64_t)columns * ceil_div(NZn, kz);
        const double waves = (double)blocks / resident;
        const double eff = waves / std::ceil(waves);                 // last-wave fill
        const double halo = (double)kz / (kz + 2);                    // halo-plane overhead
        const double score = eff * halo * std::min(1.0, waves);        // need at least one wave
        if (score > best_score + 1e-9) {
            best_score = score;
            best = c;
        }
    }
    return best;
}

// Evaluates the occupancy of every K u variant once (outside any stream capture).
void ku_prepare() {
    ku_chunks<float, KU_APPLY>(1, 8);
    ku_chunks<float, KU_APPLY_DOT>(1, 8);
    ku_chunks<float, KU_RESID>(1, 8);
    ku_chunks<float, KU_CHEB>(1, 8);
    ku_chunks<double, KU_APPLY>(1, 8);
    ku_chunks<double, KU_APPLY_DOT>(1, 8);
    ku_chunks<double, KU_RESID>(1, 8);
    ku_chunks<double, KU_CHEB>(1, 8);
}

template <class T>
int launch_ku(int mode, const KuArgs<T>& args, const KeBlocks<T>& kb, cudaStream_t s) {
    KuArgs<T> a = args;
    const Dims& d = a.d;
    const int NXn = d.nx + 1, NYn = d.ny + 1, NZn = d.nz + 1;
    const int gx = ceil_div(NXn, KU_BX), gy = ceil_div(NYn, KU_BY);
    int chunks = 1;
    switch (mode) {
        case KU_APPLY: chunks = ku_chunks<T, KU_APPLY>(gx * gy, NZn); break;
        case KU_APPLY_DOT: chunks = ku_chunks<T, KU_APPLY_DOT>(gx * gy, NZn); break;
        case KU_RESID: chunks = ku_chunks<T, KU_RESID>(gx * gy, NZn); break;
        case KU_CHEB: chunks = ku_chunks<T, KU_CHEB>(gx * gy, NZn); break;
        default: return ANL_ERR_BADARG;
    }
    a.kz = ceil_div(NZn, chunks);
    dim3 grid(gx, gy, ceil_div(NZn, a.kz));
    dim3 block(KU_BX, KU_BY);
    if (mode == KU_APPLY_DOT && (int64_t)grid.x * grid.y * grid.z > a.partial_capacity) {
        set_error("K u dot: %d blocks exceed the reduction scratch (%d)", grid.x * grid.y * grid.z,
                  a.partial_capacity);
        return ANL_ERR_BADARG;
    }
    switch (mode) {
        case KU_APPLY: ku_kernel<T, KU_APPLY><<<grid, block, 0, s>>>(a, kb); break;
        case KU_APPLY_DOT: ku_kernel<T, KU_APPLY_DOT><<<grid, block, 0, s>>>(a, kb); break;
        case KU_RESID: ku_kernel<T, KU_RESID><<<grid, block, 0, s>>>(a, kb); break;
        case KU_CHEB: ku_kernel<T, KU_CHEB><<<grid, block, 0, s>>>(a, kb); break;
        default: return ANL_ERR_BADARG;
    }
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

// ------------------------------------------------------------------ accurate residual
//
// r = b - K32 x for x held in FP64 (as the pair x_hi + x_lo of floats), where K32 is the
// FP32 operator above (the element blocks rounded to FP32). Differences, products and sums
// are carried as unevaluated float pairs (TwoSum / TwoProd), so the result is accurate to
// about eps^2 of the summed terms: the FP32 CG can certify ||b - K32 x|| <= rtol ||b||
// far below the FP32 rounding floor of a plain evaluation (eps |K| |x|), at a fraction of
// the cost of FP64 arithmetic on this part.

struct F2 {
    float s, c;
};

__device__ __forceinline__ void f2_add(F2& a, float p) {
    float t, e;
    two_sum(a.s, p, t, e);
    a.s = t;
    a.c += e;
}

__global__ void __launch_bounds__(KU_NT, 1) ku_resid_hp_kernel(ResidHpArgs a, KeBlocks<float> kb) {
    __shared__ float sh[3][KU_HY][KU_HX][3];
    __shared__ float sl[3][KU_HY][KU_HX][3];
    __shared__ float sE[2][KU_EY][KU_EX];
    __shared__ double sred[KU_NT / 32];
    const Dims d = a.d;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * KU_BX + tx;
    const int i0 = blockIdx.x * KU_BX, j0 = blockIdx.y * KU_BY, k0 = blockIdx.z * a.kz;
    const int NXn = d.nx + 1, NYn = d.ny + 1, NZn = d.nz + 1;

    auto load_nodes = [&](int slot, int kk) {
        const bool kin = kk >= 0 && kk < NZn;
        for (int f = tid; f < KU_HY * KU_HX * 3; f += KU_NT) {
            const int row = f / (KU_HX * 3);
            const int w = f - row * (KU_HX * 3);
            const int c = w / 3, comp = w - 3 * c;
            const int gi = i0 - 1 + c, gj = j0 - 1 + row;
            float vh = 0.f, vl = 0.f;
            if (kin && gi >= 0 && gi < NXn && gj >= 0 && gj < NYn) {
                const int64_t g = 3 * d.node(gi, gj, kk) + comp;
                vh = a.xhi[g];
                vl = a.xlo[g];
            }
            sh[slot][row][c][comp] = vh;
            sl[slot][row][c][comp] = vl;
        }
    };
    auto load_elems = [&](int slot, int ke) {
        const bool kin = ke >= 0 && ke < d.nz;
        for (int f = tid; f < KU_EY * KU_EX; f += KU_NT) {
            const int row = f / KU_EX, c = f - row * KU_EX;
            const int gi = i0 - 1 + c, gj = j0 - 1 + row;
            float v = 0.f;
            if (kin && gi >= 0 && gi < d.nx && gj >= 0 && gj < d.ny) v = a.E[d.elem(gi, gj, ke)];
            sE[slot][row][c] = v;
        }
    };

    load_nodes(0, k0 - 1);
    load_nodes(1, k0);
    load_elems(0, k0 - 1);
    double rr = 0.0;
    const int i = i0 + tx, j = j0 + ty;
    const int kend = min(k0 + a.kz, NZn);
    for (int k = k0; k < kend; ++k) {
        const int r = k - k0;
        const int sl3[3] = {r % 3, (r + 1) % 3, (r + 2) % 3};
        const int e_lo = r & 1, e_hi = (r + 1) & 1;
        load_nodes(sl3[2], k + 1);
        load_elems(e_hi, k);
        __syncthreads();
        if (i < NXn && j < NYn) {
            float uh[3], ul[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                uh[c] = sh[sl3[1]][ty + 1][tx + 1][c];
                ul[c] = sl[sl3[1]][ty + 1][tx + 1][c];
            }
            F2 y[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll 1
            for (int oct = 0; oct < 8; ++oct) {
                const int sx = (oct & 1) ? 1 : -1, sy = (oct & 2) ? 1 : -1, sz = (oct & 4) ? 1 : -1;
                const float Eo = sE[sz > 0 ? e_hi : e_lo][ty + (sy > 0 ? 1 : 0)][tx + (sx > 0 ? 1 : 0)];
                if (Eo == 0.f) continue;
                F2 w[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
                for (int dlt = 1; dlt < 8; ++dlt) {
                    const int mx = sx * (dlt & 1), my = sy * ((dlt >> 1) & 1), mz = sz * ((dlt >> 2) & 1);
                    const int slot = sl3[mz + 1];
                    float th[3], tc[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float sg = c == 0 ? (float)sx : (c == 1 ? (float)sy : (float)sz);
                        float dh, de;
                        two_sum(sh[slot][ty + 1 + my][tx + 1 + mx][c], -uh[c], dh, de);
                        const float dl = sl[slot][ty + 1 + my][tx + 1 + mx][c] - ul[c];
                        th[c] = sg * dh;
                        tc[c] = sg * (de + dl);
                    }
                    const float* B = kb.blk[dlt];
#pragma unroll
                    for (int rr3 = 0; rr3 < 3; ++rr3)
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            float p, e;
                            two_prod(B[3 * rr3 + c], th[c], p, e);
                            f2_add(w[rr3], p);
                            w[rr3].c += e + B[3 * rr3 + c] * tc[c];
                        }
                }
#pragma unroll
                for (int rr3 = 0; rr3 < 3; ++rr3) {
                    const float sg = rr3 == 0 ? (float)sx : (rr3 == 1 ? (float)sy : (float)sz);
                    float p, e;
                    two_prod(sg * Eo, w[rr3].s, p, e);
                    f2_add(y[rr3], p);
                    y[rr3].c += e + sg * Eo * w[rr3].c;
                }
            }
            const int64_t n = d.node(i, j, k);
            const uint8_t nm = a.nmask[n];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                double rc = 0.0;
                if ((nm >> c) & 1) rc = a.b[3 * n + c] - ((double)y[c].s + (double)y[c].c);
                a.r[3 * n + c] = (float)rc;
                rr = fma(rc, rc, rr);
            }
        }
        __syncthreads();
    }
    double v[1] = {rr};
    block_sum<1, KU_NT>(v, sred, tid);
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const int nb = gridDim.x * gridDim.y * gridDim.z;
    __shared__ double res[1];
    if (finish_reduction<1, KU_NT>(v, bid, nb, a.partials, a.counter, res, tid, sred)) {
        if (tid == 0) *a.rr_out = res[0];
    }
}

int launch_resid_hp(const ResidHpArgs& args, const KeBlocks<float>& kb, cudaStream_t s) {
    ResidHpArgs a = args;
    const Dims& d = a.d;
    const int NXn = d.nx + 1, NYn = d.ny + 1, NZn = d.nz + 1;
    const int chunks = ceil_div(NZn, 16);
    a.kz = ceil_div(NZn, chunks);
    dim3 grid(ceil_div(NXn, KU_BX), ceil_div(NYn, KU_BY), ceil_div(NZn, a.kz));
    if ((int64_t)grid.x * grid.y * grid.z > a.partial_capacity) {
        set_error("accurate residual: %d blocks exceed the reduction scratch (%d)", grid.x * grid.y * grid.z,
                  a.partial_capacity);
        return ANL_ERR_BADARG;
    }
    ku_resid_hp_kernel<<<grid, dim3(KU_BX, KU_BY), 0, s>>>(a, kb);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

// Upper bound of the K u grid (chunks of at least 4 layers): sizes the reduction scratch.
int ku_grid_blocks(const Dims& d) {
    const int NXn = d.nx + 1, NYn = d.ny + 1, NZn = d.nz + 1;
    return ceil_div(NXn, KU_BX) * ceil_div(NYn, KU_BY) * std::max(1, NZn / 4 + 1);
}

template int launch_ku<float>(int, const KuArgs<float>&, const KeBlocks<float>&, cudaStream_t);
template int launch_ku<double>(int, const KuArgs<double>&, const KeBlocks<double>&, cudaStream_t);

}  // namespace anl
