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
void count_launch();
void count_launches(long long n);  // kernels replayed by a CUDA graph

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

constexpr int kMaxRedVals = 8;
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
