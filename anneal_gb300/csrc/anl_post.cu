// anl_post.cu -- the steps between the optimised density and the exported surface.
//
// Replaces, from export.py:
//  - output_field (export.py:8-14): the printed field from the design, the design-space
//    fill, the keep-solid and keep-out fills and the frozen elements (elementwise);
//  - choose_level (export.py:17-28): the iso level whose super-level set holds the design's
//    volume, by 40 bisection steps on count(f > t). Each device pass settles 8 steps at once:
//    the 255 thresholds those steps can visit (the in-order nodes of the bisection subtree,
//    each computed along its own path with the reference's arithmetic) are counted in one
//    read of the field (a rank histogram), then one thread walks the subtree with the counts;
//  - the connectivity test of keep_load_paths (export.py:31-118, ndimage.label of f > need,
//    6-connectivity): union-find with atomicMin hooking. Every component ends up labelled
//    with its smallest element index whatever the order of the hooks, so the labels are
//    deterministic. The path repair (Dijkstra) stays on the host;
//  - the distance transform of member_thickness (export.py:150-158,
//    ndimage.distance_transform_edt of the padded solid): exact squared Euclidean distances by
//    three separable passes of the lower envelope of parabolas (Felzenszwalb and Huttenlocher,
//    "Distance transforms of sampled functions", 2012), one thread per grid line. Squared
//    distances are integers, so the square roots equal scipy's.
#include "anl_common.cuh"

namespace anl {

constexpr int POST_T = 256;
constexpr int LEVEL_DEPTH = 8;                       // bisection steps per pass
constexpr int LEVEL_NODES = (1 << LEVEL_DEPTH) - 1;  // thresholds per pass

inline int post_blocks(int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + POST_T - 1) / POST_T, 152 * 8));
}

__global__ void __launch_bounds__(POST_T) k_output_field(int64_t n, const double* __restrict__ x,
                                                         const double* __restrict__ fill,
                                                         const uint8_t* __restrict__ active,
                                                         const double* __restrict__ solid,
                                                         const double* __restrict__ voidf,
                                                         const uint8_t* __restrict__ frozen, double* __restrict__ f) {
    for (int64_t e = blockIdx.x * (int64_t)POST_T + threadIdx.x; e < n; e += (int64_t)gridDim.x * POST_T) {
        double v = x[e] * fill[e];
        v = fmax(v, active[e] ? solid[e] : 0.0);
        v = fmin(v, 1.0 - voidf[e]);
        if (frozen[e]) v = fmax(v, fill[e]);
        f[e] = v;
    }
}

// st[0] = lo, st[1] = hi of the bisection; the node j of the current subtree (in-order, depth
// `depth`) has the threshold reached by walking to it from the root
__device__ __forceinline__ double level_node(double lo, double hi, int j, int depth) {
    int idx = (1 << (depth - 1)) - 1, step = depth >= 2 ? 1 << (depth - 2) : 0;
    for (int d = 0; d < depth; ++d) {
        const double t = 0.5 * (lo + hi);
        if (j == idx) return t;
        if (j < idx) {
            hi = t;
            idx -= step;
        } else {
            lo = t;
            idx += step;
        }
        step >>= 1;
    }
    return 0.5 * (lo + hi);  // not reached for 0 <= j < 2^depth - 1
}

// per element: r = number of subtree thresholds below f; hist[r] += 1
__global__ void __launch_bounds__(POST_T) k_level_count(const double* __restrict__ f, int64_t n,
                                                        const double* __restrict__ st, int depth,
                                                        unsigned long long* __restrict__ hist) {
    __shared__ double T[LEVEL_NODES];
    __shared__ unsigned H[LEVEL_NODES + 1];
    const int nodes = (1 << depth) - 1;
    const double lo = st[0], hi = st[1];
    for (int j = threadIdx.x; j < nodes; j += POST_T) T[j] = level_node(lo, hi, j, depth);
    for (int j = threadIdx.x; j <= nodes; j += POST_T) H[j] = 0;
    __syncthreads();
    for (int64_t e = blockIdx.x * (int64_t)POST_T + threadIdx.x; e < n; e += (int64_t)gridDim.x * POST_T) {
        const double v = f[e];
        int a = 0, b = nodes;  // first j with !(T[j] < v)
        while (a < b) {
            const int m = (a + b) >> 1;
            if (T[m] < v)
                a = m + 1;
            else
                b = m;
        }
        atomicAdd(&H[a], 1u);
    }
    __syncthreads();
    for (int j = threadIdx.x; j <= nodes; j += POST_T)
        if (H[j]) atomicAdd(&hist[j], (unsigned long long)H[j]);
}

// one thread: walk the subtree; count(f > T[j]) = sum of hist[r] for r > j (export.py:21-27)
__global__ void k_level_walk(double* st, int depth, double target, unsigned long long* hist) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int nodes = (1 << depth) - 1;
    unsigned long long above[LEVEL_NODES];
    unsigned long long acc = 0;
    for (int j = nodes - 1; j >= 0; --j) {
        acc += hist[j + 1];
        above[j] = acc;
    }
    double lo = st[0], hi = st[1];
    int idx = (1 << (depth - 1)) - 1, step = depth >= 2 ? 1 << (depth - 2) : 0;
    for (int d = 0; d < depth; ++d) {
        const double t = 0.5 * (lo + hi);
        const double v = (double)above[idx];
        if (v > target) {
            lo = t;
            idx += step;
        } else {
            hi = t;
            idx -= step;
        }
        step >>= 1;
    }
    st[0] = lo;
    st[1] = hi;
    for (int j = 0; j <= nodes; ++j) hist[j] = 0;
}

// ------------------------------------------------------------------ labelling

// Labels only decrease, and every value a label ever holds is an element of the same
// component with a smaller or equal index, so a stale read still leads towards the root and
// the atomicMin below sees the true value. Reads during the hooking kernel bypass L1.
__device__ __forceinline__ int uf_find(const volatile int* lab, int x) {
    int p = lab[x];
    while (p != x) {
        x = p;
        p = lab[x];
    }
    return x;
}

__device__ void uf_union(int* lab, int a, int b) {
    while (true) {
        a = uf_find(lab, a);
        b = uf_find(lab, b);
        if (a == b) return;
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicMin(&lab[b], a);
        if (old == b) return;  // b was a root and now hangs below a
        b = old;
    }
}

__global__ void __launch_bounds__(POST_T) k_label_init(const double* __restrict__ f, int64_t n, double thr,
                                                       int* __restrict__ lab) {
    for (int64_t e = blockIdx.x * (int64_t)POST_T + threadIdx.x; e < n; e += (int64_t)gridDim.x * POST_T)
        lab[e] = f[e] > thr ? (int)e : -1;
}

__global__ void __launch_bounds__(POST_T) k_label_union(int nx, int ny, int nz, int* lab) {
    const int64_t n = (int64_t)nx * ny * nz;
    for (int64_t e = blockIdx.x * (int64_t)POST_T + threadIdx.x; e < n; e += (int64_t)gridDim.x * POST_T) {
        if (lab[e] < 0) continue;
        const int i = (int)(e % nx);
        const int64_t r = e / nx;
        const int j = (int)(r % ny), k = (int)(r / ny);
        if (i > 0 && lab[e - 1] >= 0) uf_union(lab, (int)e, (int)(e - 1));
        if (j > 0 && lab[e - nx] >= 0) uf_union(lab, (int)e, (int)(e - nx));
        if (k > 0 && lab[e - (int64_t)nx * ny] >= 0) uf_union(lab, (int)e, (int)(e - (int64_t)nx * ny));
    }
}

__global__ void __launch_bounds__(POST_T) k_label_flatten(int64_t n, int* lab) {
    for (int64_t e = blockIdx.x * (int64_t)POST_T + threadIdx.x; e < n; e += (int64_t)gridDim.x * POST_T)
        if (lab[e] >= 0) lab[e] = uf_find(lab, (int)e);
}

// ------------------------------------------------------------------ distance transform

constexpr double EDT_INF = 1e20;
constexpr int EDT_MAXN = 4096;

// One line of the separable transform: d_out(q) = min_p ((q - p)^2 + d_in(p)) over the line,
// the lower envelope of parabolas. Line of n values at base + i * stride (element units).
// First pass (axis 0): d_in is 0 on background and EDT_INF on foreground.
template <bool FIRST>
__global__ void __launch_bounds__(128) k_edt_pass(const uint8_t* __restrict__ solid, double* __restrict__ d,
                                                  int nx, int ny, int nz, int axis, int* __restrict__ vbuf,
                                                  double* __restrict__ zbuf, double* __restrict__ gbuf) {
    const int n = axis == 0 ? nx : axis == 1 ? ny : nz;
    const int64_t lines = (int64_t)nx * ny * nz / n;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (tid >= lines) return;
    int64_t base, stride;
    if (axis == 0) {
        base = tid * nx;
        stride = 1;
    } else if (axis == 1) {
        const int64_t i = tid % nx, k = tid / nx;
        base = i + (int64_t)nx * ny * k;
        stride = nx;
    } else {
        base = tid;
        stride = (int64_t)nx * ny;
    }
    int* v = vbuf + tid * n;          // parabola apexes of the envelope
    double* z = zbuf + tid * (n + 1);  // envelope breakpoints
    double* g = gbuf + tid * n;        // the line's input
    for (int q = 0; q < n; ++q) {
        const int64_t e = base + q * stride;
        g[q] = FIRST ? (solid[e] ? EDT_INF : 0.0) : d[e];
    }
    int k = -1;
    for (int q = 0; q < n; ++q) {
        if (g[q] >= EDT_INF) continue;
        const double fq = g[q] + (double)q * q;
        while (k >= 0) {
            const int p = v[k];
            const double s = (fq - (g[p] + (double)p * p)) / (2.0 * (q - p));
            if (s <= z[k]) {
                --k;
            } else {
                break;
            }
        }
        ++k;
        v[k] = q;
        z[k] = k == 0 ? -EDT_INF : (fq - (g[v[k - 1]] + (double)v[k - 1] * v[k - 1])) / (2.0 * (q - v[k - 1]));
        z[k + 1] = EDT_INF;
    }
    if (k < 0) {  // no finite value on the line
        for (int q = 0; q < n; ++q) d[base + q * stride] = EDT_INF;
        return;
    }
    int j = 0;
    for (int q = 0; q < n; ++q) {
        while (z[j + 1] < (double)q) ++j;
        const int p = v[j];
        const double dq = (double)(q - p);
        d[base + q * stride] = dq * dq + g[p];
    }
}

__global__ void __launch_bounds__(POST_T) k_edt_sqrt(int64_t n, double* d) {
    for (int64_t e = blockIdx.x * (int64_t)POST_T + threadIdx.x; e < n; e += (int64_t)gridDim.x * POST_T)
        d[e] = sqrt(d[e]);
}

}  // namespace anl

using namespace anl;

extern "C" {

int anl_output_field(const double* x, const double* fill, const uint8_t* active, const double* solid_fill,
                     const double* void_fill, const uint8_t* frozen, int64_t n, double* f, anl_stream_t stream) {
    if (!x || !fill || !active || !solid_fill || !void_fill || !frozen || !f || n < 0) {
        set_error("anl_output_field: bad argument");
        return ANL_ERR_BADARG;
    }
    if (n == 0) return ANL_OK;
    k_output_field<<<post_blocks(n), POST_T, 0, (cudaStream_t)stream>>>(n, x, fill, active, solid_fill, void_fill,
                                                                         frozen, f);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int anl_choose_level(const double* f, int64_t n, double target, double lo, double hi, int steps, double* state,
                     unsigned long long* hist, double* lo_hi_h, anl_stream_t stream) {
    if (!f || n < 1 || steps < 0 || steps > 1000 || !state || !hist || !lo_hi_h) {
        set_error("anl_choose_level: bad argument");
        return ANL_ERR_BADARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const double init[2] = {lo, hi};
    ANL_CUDA(cudaMemcpyAsync(state, init, sizeof(init), cudaMemcpyHostToDevice, s));
    ANL_CUDA(cudaMemsetAsync(hist, 0, (LEVEL_NODES + 1) * sizeof(unsigned long long), s));
    for (int done = 0; done < steps; done += LEVEL_DEPTH) {
        const int depth = std::min(LEVEL_DEPTH, steps - done);
        k_level_count<<<post_blocks(n), POST_T, 0, s>>>(f, n, state, depth, hist);
        ANL_LAUNCH_CHECK();
        k_level_walk<<<1, 32, 0, s>>>(state, depth, target, hist);
        ANL_LAUNCH_CHECK();
    }
    ANL_CUDA(cudaMemcpyAsync(lo_hi_h, state, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    ANL_CUDA(cudaStreamSynchronize(s));
    return ANL_OK;
}

int anl_label_above(const double* f, int nx, int ny, int nz, double thr, int32_t* labels, anl_stream_t stream) {
    const int64_t n = (int64_t)nx * ny * nz;
    if (!f || !labels || nx < 1 || ny < 1 || nz < 1 || n >= ((int64_t)1 << 31)) {
        set_error("anl_label_above: bad argument");
        return ANL_ERR_BADARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    k_label_init<<<post_blocks(n), POST_T, 0, s>>>(f, n, thr, labels);
    ANL_LAUNCH_CHECK();
    k_label_union<<<post_blocks(n), POST_T, 0, s>>>(nx, ny, nz, labels);
    ANL_LAUNCH_CHECK();
    k_label_flatten<<<post_blocks(n), POST_T, 0, s>>>(n, labels);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int anl_edt(const uint8_t* solid, int nx, int ny, int nz, double* dist, void* scratch, size_t scratch_bytes,
            anl_stream_t stream) {
    const int64_t n = (int64_t)nx * ny * nz;
    if (!solid || !dist || nx < 1 || ny < 1 || nz < 1 || nx > EDT_MAXN || ny > EDT_MAXN || nz > EDT_MAXN) {
        set_error("anl_edt: bad argument");
        return ANL_ERR_BADARG;
    }
    // per line: n ints (apexes), n + 1 doubles (breakpoints), n doubles (input)
    const size_t need = (((size_t)n * sizeof(int) + 15) & ~(size_t)15) + (size_t)n * 2 * sizeof(double) +
                        (size_t)std::max({(int64_t)ny * nz, (int64_t)nx * nz, (int64_t)nx * ny}) * sizeof(double);
    if (!scratch || scratch_bytes < need) {
        set_error("anl_edt: scratch of %zu bytes needed", need);
        return ANL_ERR_BADARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    for (int axis = 0; axis < 3; ++axis) {
        const int len = axis == 0 ? nx : axis == 1 ? ny : nz;
        const int64_t lines = n / len;
        int* vb = (int*)scratch;
        double* zb = (double*)((char*)scratch + (((size_t)n * sizeof(int) + 15) & ~(size_t)15));
        double* gb = zb + (n + lines);
        const int blocks = (int)((lines + 127) / 128);
        if (axis == 0)
            k_edt_pass<true><<<blocks, 128, 0, s>>>(solid, dist, nx, ny, nz, axis, vb, zb, gb);
        else
            k_edt_pass<false><<<blocks, 128, 0, s>>>(solid, dist, nx, ny, nz, axis, vb, zb, gb);
        ANL_LAUNCH_CHECK();
    }
    k_edt_sqrt<<<post_blocks(n), POST_T, 0, s>>>(n, dist);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

}  // extern "C"
