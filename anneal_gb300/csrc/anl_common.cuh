// anl_common.cuh -- shared definitions of the anneal_gb300 CUDA library (sm_103a).
//
// Grid conventions follow the anneal voxel grid (fem.py:87-127): element
// e = i + nx*(j + ny*k), node n = i + (nx+1)*(j + (ny+1)*k), DOF = 3*n + c. Nodal vectors
// are stored interleaved (the three components of a node are adjacent), element fields
// are stored on the full grid with zeros on inactive elements.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <mutex>

#include "../../include/anneal_gb300.h"

namespace anl {

// ------------------------------------------------------------------ errors

#define ANL_CUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t _e = (call);                                                           \
        if (_e != cudaSuccess) {                                                           \
            anl::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
            return ANL_ERR_CUDA;                                                           \
        }                                                                                  \
    } while (0)

// Every kernel launch of the library is followed by exactly one ANL_LAUNCH_CHECK, which
// also counts it (anl_launch_count).
#define ANL_LAUNCH_CHECK()                                                                 \
    do {                                                                                   \
        anl::count_launch();                                                               \
        cudaError_t _e = cudaGetLastError();                                               \
        if (_e != cudaSuccess) {                                                           \
            anl::set_error("%s:%d launch: %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
            return ANL_ERR_CUDA;                                                           \
        }                                                                                  \
    } while (0)

#define ANL_TRY(expr)                 \
    do {                              \
        int _s = (expr);              \
        if (_s != ANL_OK) return _s;  \
    } while (0)

void set_error(const char* fmt, ...);

// ------------------------------------------------------------------ debug bounds checks
//
// ANL_IN_RANGE(i, n) is `true` in the normal build. In the debug build (-DANL_DEBUG=1,
// `python -m anneal_gb300.build --debug`, loaded with ANL_DEBUG_LIB=1) it tests 0 <= i < n for
// a global-memory index before the access; a miss is counted in this translation unit's
// device record (the first miss keeps its index, extent and source line) and the caller skips
// the access, so a bad index is reported instead of touching memory out of range.
// anl_debug_oob collects the records of every unit. Without relocatable device code each
// unit has its own record: ANL_DEBUG_UNIT(name) defines the unit's reader.
#if ANL_DEBUG
struct OobRecord {
    unsigned long long count;
    long long index, extent, line;
};
static __device__ OobRecord g_oob;
__device__ __forceinline__ bool debug_in_range(long long i, long long n, int line) {
    if (i >= 0 && i < n) return true;
    if (atomicAdd(&g_oob.count, 1ull) == 0ull) {
        g_oob.index = i;
        g_oob.extent = n;
        g_oob.line = line;
    }
    return false;
}
#define ANL_IN_RANGE(i, n) ::anl::debug_in_range((long long)(i), (long long)(n), __LINE__)
// reads and clears this unit's record (host)
#define ANL_DEBUG_UNIT(name)                                                        \
    int debug_take_##name(unsigned long long* count, long long* first) {          \
        OobRecord r{}, z{};                                                          \
        ANL_CUDA(cudaMemcpyFromSymbol(&r, g_oob, sizeof(r)));                       \
        ANL_CUDA(cudaMemcpyToSymbol(g_oob, &z, sizeof(z)));                         \
        *count += r.count;                                                           \
        if (r.count && first[2] == 0) {                                              \
            first[0] = r.index;                                                      \
            first[1] = r.extent;                                                     \
            first[2] = r.line;                                                       \
        }                                                                            \
        return ANL_OK;                                                               \
    }
#else
#define ANL_IN_RANGE(i, n) true
#define ANL_DEBUG_UNIT(name)
#endif

// Held while a stream is captured into a CUDA graph and around every call that synchronises
// the whole device (cudaFree, cudaFreeHost, context set-up): such a call from another host
// thread would invalidate an ongoing capture, and several contexts may run in parallel
// threads (one per load case or per part).
std::recursive_mutex& device_sync_mutex();
void count_launch();
void count_launches(long long n);  // kernels replayed by a CUDA graph

// Grows a device buffer to at least `need` elements of `elem` bytes (contents are not kept).
template <class P>
inline int grow(P*& p, size_t& cap, size_t need, size_t elem) {
    if (need <= cap) return ANL_OK;
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t n = std::max<size_t>(need, 1);
    if (cudaMalloc((void**)&p, n * elem) != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMalloc of %zu bytes failed", n * elem);
        return ANL_ERR_NOMEM;
    }
    cap = n;
    return ANL_OK;
}

// ------------------------------------------------------------------ grid

struct Dims {
    int nx, ny, nz;  // elements
    __host__ __device__ int64_t ne() const { return (int64_t)nx * ny * nz; }
    __host__ __device__ int64_t nn() const { return (int64_t)(nx + 1) * (ny + 1) * (nz + 1); }
    __host__ __device__ int64_t node(int i, int j, int k) const {
        return (int64_t)i + (int64_t)(nx + 1) * ((int64_t)j + (int64_t)(ny + 1) * k);
    }
    __host__ __device__ int64_t elem(int i, int j, int k) const {
        return (int64_t)i + (int64_t)nx * ((int64_t)j + (int64_t)ny * k);
    }
};

// Node mask bits: bit c (c = 0,1,2) set when DOF c of the node is free; bit 3 set when the
// node is touched by an active element (fem.py:145-150).
enum : uint8_t { NODE_FREE_X = 1, NODE_FREE_Y = 2, NODE_FREE_Z = 4, NODE_USED = 8 };

// ------------------------------------------------------------------ element matrix

// The 24x24 hex8 stiffness of a unit cube (E = 1) has the reflection structure
//   Ke[a][b] (3x3 block) = S_a * B0(|p_b - p_a|) * S_a,   S_a = diag(1 - 2 p_a),
// with p_a the local position of node a in {0,1}^3, and every block row sums to zero
// (rigid translations store no energy). So 8 blocks B0(delta), delta in {0,1}^3, carry
// the whole matrix. blk[d] is B0(delta) with d = dx + 2 dy + 4 dz, row-major 3x3.
template <class T>
struct KeBlocks {
    T blk[8][9];
};

// Host: fills ke[576] (row-major) for a cube of side h (fem.py:71-84).
void hex8_ke(double nu, double h, double* ke);
// Host: extracts the 8 base blocks from ke and checks the reflection structure; returns
// the largest deviation found.
double ke_blocks(const double* ke, KeBlocks<double>* out);

// The same Ke in the basis of the 8 trilinear modes of a brick. A displacement component
// on the 8 corners p in {0,1}^3 is a combination of 1, sx, sy, sz, sx sy, sy sz, sz sx,
// sx sy sz (s = 2p - 1); its mode amplitudes beta_m = sum_p s_m(p) u_p are a Walsh-Hadamard
// transform. Ke u = T (KA / 64) T^T u with KA = T^T Ke T, and for an isotropic material KA
// is sparse: 45 non-zeros in 24 x 24, set by 8 numbers (the rigid translations, mode 1, carry
// none). So one element costs about 200 flops instead of the 1152 of the dense 24 x 24
// product, and the transform can be taken from edge differences u(p + e_d) - u(p), which
// keeps FP32 products proportional to the local strain, not to |u|.
// Constants (of KA / 64; modes x y z xy yz zx xyz = 1..7, components x y z):
//   g1x = A b1x + B (b2y + b3z)   and cyclic      -> ab = A - B, b = B (trace form)
//   g1y = g2x = C (b1y + b2x)     and cyclic      -> c
//   g4x = D b4x + F b5z, g5z = F b4x + D b5z, ... -> d, f
//   g4z = G b4z + H (b5x + b6y)   and cyclic      -> gh = G - H, h = H
//   g7c = J b7c                                   -> j
template <class T>
struct KeModal {
    T ab, b, c, d, f, gh, h, j;
};

// Host: the modal constants of ke (unit E); returns the largest deviation between ke and
// the matrix that modal_element applies, relative to max |ke| (a full 24 x 24 check).
double ke_modal(const double* ke, KeModal<double>* out);

// A nodal 3-vector: x and y as a pair, z alone. In FP32 the pair is a float2 driven by the
// packed f32x2 instructions of sm_100+ (one instruction for both lanes), which takes a third
// of the instructions out of the element transforms; in FP64 it is two doubles.
struct dpair {
    double x, y;
};
template <class T>
struct PairOf;
template <>
struct PairOf<float> {
    using type = float2;
};
template <>
struct PairOf<double> {
    using type = dpair;
};
template <class T>
struct V3 {
    typename PairOf<T>::type xy;
    T z;
};

__host__ __device__ __forceinline__ dpair padd(dpair a, dpair b) { return {a.x + b.x, a.y + b.y}; }
__host__ __device__ __forceinline__ dpair psub(dpair a, dpair b) { return {a.x - b.x, a.y - b.y}; }
__host__ __device__ __forceinline__ dpair pscale(double s, dpair a) { return {s * a.x, s * a.y}; }
#ifdef __CUDACC__
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) {  // a - b, one rounding
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ float2 pscale(float s, float2 a) { return __fmul2_rn(make_float2(s, s), a); }
#endif

#pragma nv_exec_check_disable
template <class T>
__host__ __device__ __forceinline__ V3<T> operator+(const V3<T>& a, const V3<T>& b) {
    return V3<T>{padd(a.xy, b.xy), a.z + b.z};
}
#pragma nv_exec_check_disable
template <class T>
__host__ __device__ __forceinline__ V3<T> operator-(const V3<T>& a, const V3<T>& b) {
    return V3<T>{psub(a.xy, b.xy), a.z - b.z};
}
#pragma nv_exec_check_disable
template <class T>
__host__ __device__ __forceinline__ V3<T> operator*(T s, const V3<T>& a) {
    return V3<T>{pscale(s, a.xy), s * a.z};
}
template <class T>
__host__ __device__ __forceinline__ V3<T> v3zero() {
    V3<T> v;
    v.xy.x = T(0);
    v.xy.y = T(0);
    v.z = T(0);
    return v;
}

// E Ke u_e of one brick from its edge differences (p = corner in {0,1}^3):
//   dxb[py] = u(1,py,0) - u(0,py,0),  dxt[py] = u(1,py,1) - u(0,py,1)
//   dyb[px] = u(px,1,0) - u(px,0,0),  dyt[px] = u(px,1,1) - u(px,0,1)
//   dz[px][py] = u(px,py,1) - u(px,py,0)
// and writes the corner forces f[px][py][pz].
// Mode amplitudes b1..b7 (x y z xy yz zx xyz) of a brick from its edge differences: the
// Walsh-Hadamard transform of the corner values, taken through the edges.
#pragma nv_exec_check_disable
template <class T>
__host__ __device__ __forceinline__ void modal_amplitudes(const V3<T> (&dxb)[2], const V3<T> (&dxt)[2],
                                                          const V3<T> (&dyb)[2], const V3<T> (&dyt)[2],
                                                          const V3<T> (&dz)[2][2], V3<T> (&b)[8]) {
    const V3<T> s0 = dxb[0] + dxb[1], s1 = dxt[0] + dxt[1];
    b[1] = s0 + s1;
    b[6] = s1 - s0;
    const V3<T> p0 = dxb[1] - dxb[0], p1 = dxt[1] - dxt[0];
    b[4] = p0 + p1;
    b[7] = p1 - p0;
    const V3<T> t0 = dyb[0] + dyb[1], t1 = dyt[0] + dyt[1];
    b[2] = t0 + t1;
    b[5] = t1 - t0;
    b[3] = (dz[0][0] + dz[1][0]) + (dz[0][1] + dz[1][1]);
}

// u_e^T Ke u_e (unit E) from the mode amplitudes: beta^T (KA / 64) beta written as sums of
// squares in which every rigid rotation cancels inside a square (b1y + b2x for a rotation
// about z, ...), so FP32 keeps the energy of an element that turns a lot but strains little.
#pragma nv_exec_check_disable
template <class T>
__host__ __device__ __forceinline__ T modal_energy(const KeModal<T>& k, const V3<T> (&b)[8]) {
    const T b1x = b[1].xy.x, b1y = b[1].xy.y, b1z = b[1].z, b2x = b[2].xy.x, b2y = b[2].xy.y, b2z = b[2].z;
    const T b3x = b[3].xy.x, b3y = b[3].xy.y, b3z = b[3].z, b4x = b[4].xy.x, b4y = b[4].xy.y, b4z = b[4].z;
    const T b5x = b[5].xy.x, b5y = b[5].xy.y, b5z = b[5].z, b6x = b[6].xy.x, b6y = b[6].xy.y, b6z = b[6].z;
    const T tr = b1x + b2y + b3z, s3 = b4z + b5x + b6y;
    const T q1 = b1y + b2x, q2 = b1z + b3x, q3 = b2z + b3y;
    T e = k.ab * (b1x * b1x + b2y * b2y + b3z * b3z) + k.b * tr * tr + k.c * (q1 * q1 + q2 * q2 + q3 * q3);
    e += k.d * (b4x * b4x + b5z * b5z + b4y * b4y + b6z * b6z + b5y * b5y + b6x * b6x);
    e += T(2) * k.f * (b4x * b5z + b4y * b6z + b5y * b6x);
    e += k.gh * (b4z * b4z + b5x * b5x + b6y * b6y) + k.h * s3 * s3;
    e += k.j * (b[7].xy.x * b[7].xy.x + b[7].xy.y * b[7].xy.y + b[7].z * b[7].z);
    return e;
}

#pragma nv_exec_check_disable
template <class T>
__host__ __device__ __forceinline__ void modal_element(const KeModal<T>& k, T E, const V3<T> (&dxb)[2],
                                                       const V3<T> (&dxt)[2], const V3<T> (&dyb)[2],
                                                       const V3<T> (&dyt)[2], const V3<T> (&dz)[2][2],
                                                       V3<T> (&f)[2][2][2]) {
    // mode amplitudes (Walsh-Hadamard transform through the edges)
    V3<T> bm[8];
    modal_amplitudes<T>(dxb, dxt, dyb, dyt, dz, bm);
    const V3<T>& b1 = bm[1];
    const V3<T>& b2 = bm[2];
    const V3<T>& b3 = bm[3];
    const V3<T>& b4 = bm[4];
    const V3<T>& b5 = bm[5];
    const V3<T>& b6 = bm[6];
    const V3<T>& b7 = bm[7];
    // the sparse modal stiffness, scaled by E
    const T ab = E * k.ab, bb = E * k.b, cc = E * k.c, dd = E * k.d, ff = E * k.f, gh = E * k.gh, hh = E * k.h,
            jj = E * k.j;
    V3<T> g1, g2, g3, g4, g5, g6;
    const T tr = b1.xy.x + b2.xy.y + b3.z;
    g1.xy.x = ab * b1.xy.x + bb * tr;
    g2.xy.y = ab * b2.xy.y + bb * tr;
    g3.z = ab * b3.z + bb * tr;
    g1.xy.y = g2.xy.x = cc * (b1.xy.y + b2.xy.x);
    g1.z = g3.xy.x = cc * (b1.z + b3.xy.x);
    g2.z = g3.xy.y = cc * (b2.z + b3.xy.y);
    g4.xy.x = dd * b4.xy.x + ff * b5.z;
    g5.z = ff * b4.xy.x + dd * b5.z;
    g4.xy.y = dd * b4.xy.y + ff * b6.z;
    g6.z = ff * b4.xy.y + dd * b6.z;
    g5.xy.y = dd * b5.xy.y + ff * b6.xy.x;
    g6.xy.x = ff * b5.xy.y + dd * b6.xy.x;
    const T s3 = b4.z + b5.xy.x + b6.xy.y;
    g4.z = gh * b4.z + hh * s3;
    g5.xy.x = gh * b5.xy.x + hh * s3;
    g6.xy.y = gh * b6.xy.y + hh * s3;
    const V3<T> g7 = jj * b7;
    // back to the corners: f(p) = sum_m s_m(p) g_m = A(py,pz) + sx B(py,pz)
    const V3<T> am = g2 - g5, ap = g2 + g5;
    const V3<T> n00 = am + g3, a10 = am - g3, a01 = g3 - ap, a11 = ap + g3;  // A(0,0) = -n00
    const V3<T> cm = g1 - g6, cp = g1 + g6, dm = g4 - g7, dp = g4 + g7;
    const V3<T> q00 = cm - dm, q10 = cm + dm, q01 = cp - dp, q11 = cp + dp;
    f[0][0][0] = v3zero<T>() - (n00 + q00);
    f[1][0][0] = q00 - n00;
    f[0][1][0] = a10 - q10;
    f[1][1][0] = a10 + q10;
    f[0][0][1] = a01 - q01;
    f[1][0][1] = a01 + q01;
    f[0][1][1] = a11 - q11;
    f[1][1][1] = a11 + q11;
}

// ------------------------------------------------------------------ reductions

// Deterministic two-stage reductions: every block writes its partial sums to a scratch
// array; the last block to finish (ticket counter) adds the partials in block order and
// writes the result. Nothing depends on atomic ordering, so reruns are bit-identical.
struct RedScratch {
    double* partials;    // capacity_blocks * max_vals
    unsigned* counter;   // one ticket counter per concurrent reduction slot
    int capacity_blocks;
    int max_vals;
};

constexpr int kMaxRedVals = 16;
constexpr int kRedBlocks = 1216;  // 152 SMs x 8: grid of the grid-stride vector kernels

// Sum of `val` over the block, for NV values; result valid in the thread with flat index 0.
// `tid` is the flat thread index (threadIdx.x for 1D blocks).
template <int NV, int NT>
__device__ __forceinline__ void block_sum(double (&val)[NV], double* smem /* NV*NT/32 */, int tid) {
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double s = val[v];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) smem[v * (NT / 32) + warp] = s;
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            double s = 0;
            for (int w = 0; w < NT / 32; ++w) s += smem[v * (NT / 32) + w];
            val[v] = s;
        }
    }
}

// The same block sum for values given as unevaluated float pairs (s + c) per thread: the warp
// tree adds pairs with TwoSum on the FP32 pipes (FP64 arithmetic on this part runs at a small
// fraction of FP32, and a tree of FP64 adds over every thread of a full grid costs microseconds),
// each warp's pair becomes one double, and thread 0 adds the warps' doubles in order. About 48
// significant bits; deterministic. Result valid in the thread with flat index 0.
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// Block sum of NV float pairs (hi + lo per thread), entirely on the FP32 pipes: the warp tree
// adds pairs with TwoSum, then thread 0 adds the warps' pairs in order. FP64 arithmetic on this
// part runs at a small fraction of the FP32 rate: even a few FP64 instructions per warp, in every
// block of a 1,216-block reduction, cost several microseconds. Result in thread 0 (in place).
template <int NV, int NT>
__device__ __forceinline__ void block_pair_sum(float (&hi)[NV], float (&lo)[NV], float2* smem /* NV*NT/32 */,
                                               int tid) {
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        float h = hi[v], l = lo[v];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float h2 = __shfl_down_sync(0xffffffffu, h, o), l2 = __shfl_down_sync(0xffffffffu, l, o);
            float t, e;
            two_sum_f(h, h2, t, e);
            h = t;
            l += l2 + e;
        }
        if (lane == 0) smem[v * (NT / 32) + warp] = make_float2(h, l);
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            float2 a = smem[v * (NT / 32)];
            for (int w = 1; w < NT / 32; ++w) {
                const float2 b = smem[v * (NT / 32) + w];
                float t, e;
                two_sum_f(a.x, b.x, t, e);
                a = make_float2(t, a.y + b.y + e);
            }
            hi[v] = a.x;
            lo[v] = a.y;
        }
    }
}

// The same block sum with the result as doubles (thread 0), for finish_reduction.
template <int NV, int NT>
__device__ __forceinline__ void block_sum_f2(const float (&s)[NV], const float (&c)[NV], double (&val)[NV],
                                             double* smem /* NV*NT/32 */, int tid) {
    float h[NV], l[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        h[v] = s[v];
        l[v] = c[v];
    }
    block_pair_sum<NV, NT>(h, l, reinterpret_cast<float2*>(smem), tid);
    if (tid == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) val[v] = (double)h[v] + (double)l[v];
    }
}

// finish_reduction for float pairs (after block_pair_sum, the pairs valid in thread 0): each
// block stores its pairs in the 8-byte partial slots, the last block adds them in the fixed
// order of finish_reduction with TwoSum and block_pair_sum, and thread 0 writes
// out[v] = hi + lo as a double. Returns true in the block that wrote the result.
template <int NV, int NT>
__device__ __forceinline__ bool finish_pair_reduction(const float (&hi)[NV], const float (&lo)[NV], int bid,
                                                      int nblocks, double* partials, unsigned* counter, double* out,
                                                      int tid, float2* smem /* NV*NT/32 */) {
    __shared__ bool last;
    float2* p = reinterpret_cast<float2*>(partials);
    __syncthreads();  // smem of block_pair_sum is reused below
    if (tid == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) p[(int64_t)bid * NV + v] = make_float2(hi[v], lo[v]);
        __threadfence();
        const unsigned t = atomicAdd(counter, 1u);
        last = (t == (unsigned)nblocks - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    float h[NV], l[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        h[v] = 0.f;
        l[v] = 0.f;
        for (int b = tid; b < nblocks; b += NT) {
            const float2 q = __ldcg(p + (int64_t)b * NV + v);
            float t, e;
            two_sum_f(h[v], q.x, t, e);
            h[v] = t;
            l[v] += q.y + e;
        }
    }
    block_pair_sum<NV, NT>(h, l, smem, tid);
    if (tid == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) out[v] = (double)h[v] + (double)l[v];
        *counter = 0u;
    }
    return true;
}

// Finishes a reduction: block `bid` of `nblocks` stores its NV partials; the last block to
// arrive adds them and writes out[0..NV) (from thread 0). The last block sums in parallel:
// thread t adds partials t, t+NT, t+2NT, ... in order, then a fixed tree combines the
// threads, so the result depends only on the partials, never on which block came last.
// Call with every thread of the block after block_sum (val valid in thread 0); `smem` holds
// NV*NT/32 doubles. Returns true in the block that wrote the result.
template <int NV, int NT>
__device__ __forceinline__ bool finish_reduction(const double (&val)[NV], int bid, int nblocks, double* partials,
                                                 unsigned* counter, double* out, int tid, double* smem) {
    __shared__ bool last;
    __syncthreads();  // smem of block_sum is reused below
    if (tid == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) partials[(int64_t)bid * NV + v] = val[v];
        __threadfence();
        unsigned t = atomicAdd(counter, 1u);
        last = (t == (unsigned)nblocks - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double s = 0.0;
        for (int b = tid; b < nblocks; b += NT) s += __ldcg(partials + (int64_t)b * NV + v);
        acc[v] = s;
    }
    block_sum<NV, NT>(acc, smem, tid);
    if (tid == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) out[v] = acc[v];
        *counter = 0u;
    }
    return true;
}

// Error-free product and sum (Dekker/Knuth): exact s + e == a*b, a+b in FP32. Used for
// dot products whose per-thread partials must carry ~FP48 accuracy before they are
// promoted to FP64 (FP64 arithmetic on this part runs at a small fraction of FP32).
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = a * b;
    e = fmaf(a, b, -p);
}
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// A double-float: the unevaluated sum hi + lo of two floats, about 48 significant bits.
// Sums and products cost a few FP32 instructions (TwoSum, FMA-based TwoProd), far less than
// FP64 arithmetic on this part. Used for the accurate residual of the FP64 operator.
struct alignas(8) DF {
    float hi, lo;
    DF() = default;
    __host__ __device__ constexpr DF(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr DF(float v) : hi(v), lo(0.f) {}
    __host__ __device__ explicit constexpr DF(int v) : hi((float)v), lo(0.f) {}
    __host__ __device__ explicit DF(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    __host__ __device__ explicit operator float() const { return hi + lo; }
    __host__ __device__ double value() const { return (double)hi + (double)lo; }
};
#ifdef __CUDACC__
__device__ __forceinline__ DF df_norm(float s, float e) {  // |s| >= |e|
    const float h = s + e;
    return DF(h, e - (h - s));
}
__device__ __forceinline__ DF operator+(DF a, DF b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    return df_norm(s, e);
}
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + DF(-b.hi, -b.lo); }
__device__ __forceinline__ DF operator*(DF a, DF b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_norm(p, e);
}
__device__ __forceinline__ DF operator/(DF a, DF b) { return DF(a.value() / b.value()); }  // not on a hot path
// 1 / a to about 48 bits: the FP32 reciprocal refined by one Newton step in pair arithmetic
// (r + r (1 - a r) doubles the number of correct bits)
__device__ __forceinline__ DF df_recip(DF a) {
    const float r0 = 1.f / a.hi;
    const DF e = DF(1.f) - a * DF(r0);
    return DF(r0) + DF(r0) * e;
}
__device__ __forceinline__ DF& operator+=(DF& a, DF b) { return a = a + b; }
__device__ __forceinline__ bool operator>(DF a, DF b) { return a.value() > b.value(); }
#endif
#ifdef __CUDACC__
// A double as an unevaluated float pair hi + lo, by integer and FP32 operations only (FP64
// arithmetic on this part runs at a small fraction of the FP32 rate, and a conversion per
// value is FP64 work): hi keeps the leading 24 significant bits (truncated), lo the next 29
// rounded to 24, so hi + lo is within 2^-48 of d. |d| below 2^-120 becomes (signed) zero and
// |d| beyond the float range takes the FP64 path; neither occurs in the fields split here.
__device__ __forceinline__ void split_double(double d, float& hi, float& lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FF);
    if (e < 1023 - 120) {
        hi = __uint_as_float(sign);
        lo = 0.f;
        return;
    }
    if (e > 1023 + 127) {
        hi = (float)d;
        lo = 0.f;
        return;
    }
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | (unsigned)(m >> 29));
    const unsigned r = (unsigned)(m & 0x1FFFFFFFull);  // the 29 bits below hi, weight 2^(e - 1075)
    const float scale = e > 948 ? __uint_as_float((unsigned)(e - 948) << 23) : 0.f;
    const float l = __uint2float_rn(r) * scale;
    lo = sign ? -l : l;
}
// (a_hi + a_lo) - (b_hi + b_lo) rounded to FP32
__device__ __forceinline__ float df_diff(float ah, float al, float bh, float bl) {
    float s, e;
    two_sum(ah, -bh, s, e);
    return s + (e + (al - bl));
}
#endif
struct dfpair {
    DF x, y;
};
template <>
struct PairOf<DF> {
    using type = dfpair;
};
#ifdef __CUDACC__
__device__ __forceinline__ dfpair padd(dfpair a, dfpair b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ dfpair psub(dfpair a, dfpair b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ dfpair pscale(DF s, dfpair a) { return {s * a.x, s * a.y}; }
#endif

// Compensated accumulator: adds a*b exactly up to FP32 rounding of the error terms.
struct Acc2 {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add_prod(float a, float b) {
        float p, e, t, f;
        two_prod(a, b, p, e);
        two_sum(s, p, t, f);
        s = t;
        c += f + e;
    }
    __device__ __forceinline__ void add_prod(double a, double b) {  // FP64 inputs
        add_d(a * b);
    }
    __device__ __forceinline__ void add_d(double v) {
        float hi = (float)v;
        float lo = (float)(v - (double)hi);
        float t, f;
        two_sum(s, hi, t, f);
        s = t;
        c += f + lo;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// ------------------------------------------------------------------ PCG device scalars

struct PcgScalars {
    double rz[2];   // r.z of the current / next iteration (ping-pong on iteration parity)
    double pq;      // p.K p
    double zq;      // z_new.q (flexible beta)
    double rr;      // ||r||^2
    double bb;      // ||b||^2
    double alpha;
    double tol2;    // (rtol ||b||)^2
    double rr_true; // ||b - K x||^2 from the last residual replacement
    int done;       // 0 running, 1 converged, 2 maxiter, 3 non-finite, 4 breakdown; every
                    // kernel of the CG loop returns early while it is non-zero
    int iters;      // iterations performed
    int nonfinite;  // a non-finite scalar was seen
    int maxiter;
};

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

}  // namespace anl
