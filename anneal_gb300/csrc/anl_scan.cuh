// anl_scan.cuh -- deterministic exclusive scans over device arrays (int, int64, int2).
#pragma once

#include <algorithm>

#include "anl_common.cuh"

namespace anl {

// ------------------------------------------------------------------ scan (deterministic)

// Exclusive scan in three passes over a fixed grid: block sums, a one-block scan of those,
// then each block rescans its chunk from its offset. No atomics: results are reproducible.
constexpr int SCAN_BLOCKS = 1216;
constexpr int SCAN_T = 512;

template <class V>
struct ScanOps;
template <>
struct ScanOps<int> {
    __device__ static int zero() { return 0; }
    __device__ static int add(int a, int b) { return a + b; }
    __device__ static int sub(int a, int b) { return a - b; }
    __device__ static int shfl_up(int v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
};
template <>
struct ScanOps<long long> {
    __device__ static long long zero() { return 0; }
    __device__ static long long add(long long a, long long b) { return a + b; }
    __device__ static long long sub(long long a, long long b) { return a - b; }
    __device__ static long long shfl_up(long long v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
};
template <>
struct ScanOps<int2> {
    __device__ static int2 zero() { return make_int2(0, 0); }
    __device__ static int2 add(int2 a, int2 b) { return make_int2(a.x + b.x, a.y + b.y); }
    __device__ static int2 sub(int2 a, int2 b) { return make_int2(a.x - b.x, a.y - b.y); }
    __device__ static int2 shfl_up(int2 v, int d) {
        return make_int2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
    }
};

// inclusive scan of one value per thread across the block; returns the block total in *tot
template <class V>
__device__ V block_scan_incl(V v, V* sm, V* tot) {
    using O = ScanOps<V>;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const V u = O::shfl_up(v, d);
        if (lane >= d) v = O::add(v, u);
    }
    if (lane == 31) sm[warp] = v;
    __syncthreads();
    if (warp == 0) {
        V w = lane < SCAN_T / 32 ? sm[lane] : O::zero();
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const V u = O::shfl_up(w, d);
            if (lane >= d) w = O::add(w, u);
        }
        if (lane < SCAN_T / 32) sm[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v = O::add(v, sm[warp - 1]);
    *tot = sm[SCAN_T / 32 - 1];
    __syncthreads();
    return v;
}

template <class V>
__global__ void __launch_bounds__(SCAN_T) k_scan_reduce(const V* in, int64_t n, int64_t chunk, V* part) {
    using O = ScanOps<V>;
    __shared__ V sm[SCAN_T / 32];
    const int64_t b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    V acc = O::zero();
    for (int64_t i = b0 + threadIdx.x; i < b1; i += SCAN_T) acc = O::add(acc, in[i]);
    V tot;
    block_scan_incl<V>(acc, sm, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// turns the block sums into inclusive prefix sums (one block); *total = the grand total
template <class V>
__global__ void __launch_bounds__(SCAN_T) k_scan_top(V* part, int nb, V* total) {
    using O = ScanOps<V>;
    __shared__ V sm[SCAN_T / 32];
    V base = O::zero();
    for (int b0 = 0; b0 < nb; b0 += SCAN_T) {
        const int i = b0 + threadIdx.x;
        const V v = i < nb ? part[i] : O::zero();
        V tot;
        const V incl = block_scan_incl<V>(v, sm, &tot);
        if (i < nb) part[i] = O::add(base, incl);
        base = O::add(base, tot);
    }
    if (threadIdx.x == 0) *total = base;
}

template <class V>
__global__ void __launch_bounds__(SCAN_T) k_scan_down(const V* in, int64_t n, int64_t chunk, const V* part_incl,
                                                      V* out) {
    using O = ScanOps<V>;
    __shared__ V sm[SCAN_T / 32];
    const int64_t b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    V base = blockIdx.x > 0 ? part_incl[blockIdx.x - 1] : O::zero();
    for (int64_t t0 = b0; t0 < b1; t0 += SCAN_T) {
        const int64_t i = t0 + threadIdx.x;
        const V v = i < b1 ? in[i] : O::zero();
        V tot;
        const V incl = block_scan_incl<V>(v, sm, &tot);
        if (i < b1) out[i] = O::sub(O::add(base, incl), v);
        base = O::add(base, tot);
    }
}

// exclusive scan of n values: out[i] = in[0] + ... + in[i-1]; *total_d = the sum (device)
template <class V>
static inline int scan_exclusive(const V* in, int64_t n, V* out, V* part, V* total_d, cudaStream_t s) {
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(SCAN_BLOCKS, (n + SCAN_T - 1) / SCAN_T));
    const int64_t chunk = (n + nb - 1) / nb;
    k_scan_reduce<V><<<nb, SCAN_T, 0, s>>>(in, n, chunk, part);
    ANL_LAUNCH_CHECK();
    k_scan_top<V><<<1, SCAN_T, 0, s>>>(part, nb, total_d);
    ANL_LAUNCH_CHECK();
    k_scan_down<V><<<nb, SCAN_T, 0, s>>>(in, n, chunk, part, out);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

}  // namespace anl
