// anl_vox.cu -- the voxeliser: the fill fraction of every grid element inside a closed
// triangle mesh.
//
// Replaces geometry.voxel_fill (geometry.py:89-149). The method is the reference's: s x s x s
// sample points per element, a ray along +z through every (x, y) sample column, a sample is
// inside when an odd number of the column's triangle crossings lie below it, and the fill
// fraction is the inside share of the element's samples. The reference gathers every
// crossing as a key (column index + normalised height), sorts all keys and counts the keys
// below each sample by binary search. Here nothing is sorted:
//  1. k_vox_zrange: the lowest and highest vertex z (they normalise the crossing heights);
//  2. k_vox_axes: the sample coordinates along x and y and the normalised sample heights;
//  3. k_vox_count: per triangle, the sample columns inside its xy bounding box (binary
//     search on the sample axes); an exclusive scan gives every (triangle, column) pair a slot;
//  4. k_vox_hits: one thread per pair runs the barycentric test. A crossing flips the bit of
//     the lowest sample above it in the column's bit row (atomicXor), so that
//  5. k_vox_parity: a prefix XOR along each column turns the flips into inside bits, and
//  6. k_vox_fill: the popcount of an element's s^3 sample bits, divided by s^3.
// Every number that decides a crossing or a comparison is the reference's FP64 expression,
// evaluated one rounded operation at a time (__dmul_rn, __dadd_rn, __dsub_rn: nothing is
// contracted into an FMA; FP64 division is correctly rounded). A crossing is counted below
// a sample exactly when the reference's sorted search counts it, so the inside bits and the
// fill fractions are the reference's, bit for bit.
#include <new>

#include "anl_common.cuh"
#include "anl_scan.cuh"

namespace anl {

constexpr int VOX_T = 256;
constexpr int VOX_MAX_S = 16;

struct VoxGrid {
    int nx, ny, nz, s;
    int nxs, nys, nzs;  // sample counts per axis (n * s)
    int64_t ncol;       // nxs * nys
    int W;              // 32-bit words per column bit row
    double h, ox, oy, oz;
};

// doubles ordered as unsigned integers (atomicMin/atomicMax on finite values)
__device__ __forceinline__ unsigned long long dkey(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dunkey(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// zmm[0] = key of min z, zmm[1] = key of max z (initialised to ~0 and 0)
__global__ void __launch_bounds__(VOX_T) k_vox_zrange(const double* __restrict__ tri, int64_t ntri,
                                                      unsigned long long* zmm) {
    unsigned long long lo = ~0ull, hi = 0ull;
    for (int64_t v = blockIdx.x * (int64_t)VOX_T + threadIdx.x; v < 3 * ntri; v += (int64_t)gridDim.x * VOX_T) {
        const unsigned long long k = dkey(tri[3 * v + 2]);
        lo = min(lo, k);
        hi = max(hi, k);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(zmm, lo);
        atomicMax(zmm + 1, hi);
    }
}

// xs, ys: sample coordinates (geometry.py:91-94); zq: normalised, clipped sample heights
// (geometry.py:144); zs_out[0..1] = zlo, zr
__global__ void __launch_bounds__(VOX_T) k_vox_axes(VoxGrid G, const unsigned long long* zmm, double* xs,
                                                    double* ys, double* zq, double* zs_out) {
    const double zlo = dunkey(zmm[0]), zhi = dunkey(zmm[1]);
    const double zr = __dadd_rn(__dmul_rn(__dsub_rn(zhi, zlo), 1.001), 1e-9);
    const int n = G.nxs + G.nys + G.nzs;
    for (int t = blockIdx.x * VOX_T + threadIdx.x; t < n; t += gridDim.x * VOX_T) {
        int axis, m = t;
        if (m < G.nxs) {
            axis = 0;
        } else if ((m -= G.nxs) < G.nys) {
            axis = 1;
        } else {
            m -= G.nys;
            axis = 2;
        }
        const int i = m / G.s, a = m - i * G.s;
        const double sub = ((double)a + 0.5) / (double)G.s;
        const double o = axis == 0 ? G.ox : axis == 1 ? G.oy : G.oz;
        const double c = __dadd_rn(o, __dmul_rn(G.h, __dadd_rn((double)i, sub)));
        if (axis == 0) {
            xs[m] = __dadd_rn(c, __dmul_rn(G.h, 6.18e-6));
        } else if (axis == 1) {
            ys[m] = __dadd_rn(c, __dmul_rn(G.h, 4.14e-6));
        } else {
            const double q = __dsub_rn(c, zlo) / zr;
            zq[m] = fmin(fmax(q, 0.0), 0.999999);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        zs_out[0] = zlo;
        zs_out[1] = zr;
    }
}

// first index with a[i] >= v (right = false) or a[i] > v (right = true): numpy searchsorted
__device__ __forceinline__ int vox_search(const double* __restrict__ a, int n, double v, bool right) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const double x = a[mid];
        if (right ? (x <= v) : (x < v))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// per triangle: the first sample column along x and y inside its bounding box and the box
// width; cnt = the number of columns in the box (geometry.py:99-105)
__global__ void __launch_bounds__(VOX_T) k_vox_count(const double* __restrict__ tri, int64_t ntri, VoxGrid G,
                                                     const double* __restrict__ xs, const double* __restrict__ ys,
                                                     int4* __restrict__ box, long long* __restrict__ cnt) {
    for (int64_t t = blockIdx.x * (int64_t)VOX_T + threadIdx.x; t < ntri; t += (int64_t)gridDim.x * VOX_T) {
        const double* v = tri + 9 * t;
        const double xmin = fmin(fmin(v[0], v[3]), v[6]), xmax = fmax(fmax(v[0], v[3]), v[6]);
        const double ymin = fmin(fmin(v[1], v[4]), v[7]), ymax = fmax(fmax(v[1], v[4]), v[7]);
        const int ix0 = vox_search(xs, G.nxs, xmin, false), ix1 = vox_search(xs, G.nxs, xmax, true);
        const int iy0 = vox_search(ys, G.nys, ymin, false), iy1 = vox_search(ys, G.nys, ymax, true);
        const int nxr = max(ix1 - ix0, 0), nyr = max(iy1 - iy0, 0);
        box[t] = make_int4(ix0, iy0, nxr, 0);
        cnt[t] = (long long)nxr * nyr;
    }
}

// one thread per (triangle, column) pair: the barycentric test of geometry.py:124-131 and the
// flip of the lowest sample the crossing lies below (geometry.py:139-146)
__global__ void __launch_bounds__(VOX_T) k_vox_hits(const double* __restrict__ tri, int64_t ntri, VoxGrid G,
                                                    const double* __restrict__ xs, const double* __restrict__ ys,
                                                    const double* __restrict__ zq, const double* __restrict__ zs,
                                                    const int4* __restrict__ box, const long long* __restrict__ off,
                                                    const long long* __restrict__ total, unsigned* __restrict__ bits,
                                                    unsigned long long* __restrict__ nhits) {
    const long long np = *total;
    const double zlo = zs[0], zr = zs[1];
    unsigned long long mine = 0;
    for (long long p = blockIdx.x * (long long)VOX_T + threadIdx.x; p < np; p += (long long)gridDim.x * VOX_T) {
        // the triangle: the last t with off[t] <= p (triangles without columns have no slot)
        int64_t lo = 0, hi = ntri;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (off[mid] <= p)
                lo = mid + 1;
            else
                hi = mid;
        }
        const int64_t t = lo - 1;
        const int4 b = box[t];
        const long long local = p - off[t];
        const int lx = (int)(local % b.z), ly = (int)(local / b.z);
        const int cx = b.x + lx, cy = b.y + ly;
        const double px = xs[cx], py = ys[cy];
        const double* v = tri + 9 * t;
        const double x0 = v[0], y0 = v[1], z0 = v[2], x1 = v[3], y1 = v[4], z1 = v[5], x2 = v[6], y2 = v[7],
                     z2 = v[8];
        const double y12 = __dsub_rn(y1, y2), x21 = __dsub_rn(x2, x1), x02 = __dsub_rn(x0, x2);
        const double d = __dadd_rn(__dmul_rn(y12, x02), __dmul_rn(x21, __dsub_rn(y0, y2)));
        if (d == 0.0) continue;
        const double pxd = __dsub_rn(px, x2), pyd = __dsub_rn(py, y2);
        const double l0 = __dadd_rn(__dmul_rn(y12, pxd), __dmul_rn(x21, pyd)) / d;
        const double l1 = __dadd_rn(__dmul_rn(__dsub_rn(y2, y0), pxd), __dmul_rn(x02, pyd)) / d;
        const double l2 = __dsub_rn(__dsub_rn(1.0, l0), l1);
        if (!(l0 >= 0.0 && l1 >= 0.0 && l2 >= 0.0)) continue;
        const double z = __dadd_rn(__dadd_rn(__dmul_rn(l0, z0), __dmul_rn(l1, z1)), __dmul_rn(l2, z2));
        const double zn = __dsub_rn(z, zlo) / zr;
        // The reference sorts keys col + zn and counts, for sample m of column c, the keys in
        // [c, c + zq[m]) (both ends rounded to FP64 like the keys). A key that rounds below its
        // own column is therefore counted nowhere, and one that reaches the next column's
        // range belongs to that column.
        int64_t c = cx + (int64_t)G.nxs * cy;
        const double key = __dadd_rn((double)c, zn);
        if (key < (double)c) continue;
        if (key >= (double)(c + 1)) {
            if (++c >= G.ncol) continue;
        }
        ++mine;
        int mlo = 0, mhi = G.nzs;  // the lowest sample m with c + zq[m] > key
        const double cd = (double)c;
        while (mlo < mhi) {
            const int mid = (mlo + mhi) >> 1;
            if (__dadd_rn(cd, zq[mid]) > key)
                mhi = mid;
            else
                mlo = mid + 1;
        }
        if (mlo < G.nzs) atomicXor(bits + (int64_t)(mlo >> 5) * G.ncol + c, 1u << (mlo & 31));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(nhits, mine);
}

// bit rows of flips -> inside bits (prefix XOR along z); rows are word-major: bits[w*ncol + c]
__global__ void __launch_bounds__(VOX_T) k_vox_parity(VoxGrid G, unsigned* __restrict__ bits) {
    for (int64_t c = blockIdx.x * (int64_t)VOX_T + threadIdx.x; c < G.ncol; c += (int64_t)gridDim.x * VOX_T) {
        unsigned carry = 0;
        for (int w = 0; w < G.W; ++w) {
            unsigned x = bits[(int64_t)w * G.ncol + c];
            x ^= x << 1;
            x ^= x << 2;
            x ^= x << 4;
            x ^= x << 8;
            x ^= x << 16;
            x ^= carry;
            carry = (x >> 31) ? ~0u : 0u;
            bits[(int64_t)w * G.ncol + c] = x;
        }
    }
}

// fill fraction per element (x fastest): inside samples / s^3 (geometry.py:147-149)
__global__ void __launch_bounds__(VOX_T) k_vox_fill(VoxGrid G, const unsigned* __restrict__ bits,
                                                    double* __restrict__ fill) {
    const int64_t ne = (int64_t)G.nx * G.ny * G.nz;
    const unsigned mask = (G.s >= 32) ? ~0u : ((1u << G.s) - 1u);
    const double n3 = (double)(G.s * G.s * G.s);
    for (int64_t e = blockIdx.x * (int64_t)VOX_T + threadIdx.x; e < ne; e += (int64_t)gridDim.x * VOX_T) {
        const int i = (int)(e % G.nx);
        const int64_t r = e / G.nx;
        const int j = (int)(r % G.ny), k = (int)(r / G.ny);
        const int m = k * G.s, w = m >> 5, sh = m & 31;
        const bool two = sh + G.s > 32;
        int count = 0;
        for (int b = 0; b < G.s; ++b)
            for (int a = 0; a < G.s; ++a) {
                const int64_t c = (int64_t)(i * G.s + a) + (int64_t)G.nxs * (j * G.s + b);
                unsigned x = bits[(int64_t)w * G.ncol + c] >> sh;
                if (two) x |= bits[(int64_t)(w + 1) * G.ncol + c] << (32 - sh);
                count += __popc(x & mask);
            }
        fill[e] = (double)count / n3;
    }
}

inline int vox_blocks(int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + VOX_T - 1) / VOX_T, 152 * 16));
}

}  // namespace anl

using namespace anl;

struct anl_vox {
    int4* box = nullptr;
    size_t box_cap = 0;
    long long* cnt = nullptr;
    size_t cnt_cap = 0;
    long long* off = nullptr;
    size_t off_cap = 0;
    double* axes = nullptr;  // xs | ys | zq
    size_t axes_cap = 0;
    unsigned* bits = nullptr;
    size_t bits_cap = 0;
    long long* part = nullptr;  // SCAN_BLOCKS
    // scalars: [0..1] z range keys, [2] pair total, [3] hits, then zlo, zr as doubles
    unsigned long long* sc = nullptr;
    unsigned long long* host = nullptr;
};

namespace {

void vox_free(anl_vox* v) {
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    cudaFree(v->box);
    cudaFree(v->cnt);
    cudaFree(v->off);
    cudaFree(v->axes);
    cudaFree(v->bits);
    cudaFree(v->part);
    cudaFree(v->sc);
    if (v->host) cudaFreeHost(v->host);
    delete v;
}

}  // namespace

extern "C" {

int anl_vox_create(anl_vox** out) {
    if (!out) {
        set_error("anl_vox_create: null argument");
        return ANL_ERR_BADARG;
    }
    *out = nullptr;
    anl_vox* v = new (std::nothrow) anl_vox();
    if (!v) return ANL_ERR_NOMEM;
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    if (cudaMalloc((void**)&v->part, SCAN_BLOCKS * sizeof(long long)) != cudaSuccess ||
        cudaMalloc((void**)&v->sc, 8 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMallocHost((void**)&v->host, 8 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        set_error("anl_vox_create: allocation failed");
        vox_free(v);
        return ANL_ERR_NOMEM;
    }
    *out = v;
    return ANL_OK;
}

void anl_vox_destroy(anl_vox* v) {
    if (v) vox_free(v);
}

int anl_voxel_fill(anl_vox* v, const double* tri, int64_t ntri, int nx, int ny, int nz, double h,
                   const double* origin_h, int s, double* fill, int64_t* stats_h, anl_stream_t stream) {
    if (!v || !tri || !origin_h || !fill || ntri < 1 || nx < 1 || ny < 1 || nz < 1 || s < 1 || s > VOX_MAX_S ||
        !(h > 0) || !std::isfinite(h)) {
        set_error("anl_voxel_fill: bad argument%s", ntri < 1 ? " (the mesh has no triangles)" : "");
        return ANL_ERR_BADARG;
    }
    const int64_t nxs = (int64_t)nx * s, nys = (int64_t)ny * s, nzs = (int64_t)nz * s;
    if (nxs > (1 << 28) || nys > (1 << 28) || nzs > (1 << 28) || nxs * nys > ((int64_t)1 << 40) ||
        ntri > ((int64_t)1 << 40)) {
        set_error("anl_voxel_fill: grid or mesh too large");
        return ANL_ERR_BADARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    VoxGrid G;
    G.nx = nx, G.ny = ny, G.nz = nz, G.s = s;
    G.nxs = (int)nxs, G.nys = (int)nys, G.nzs = (int)nzs;
    G.ncol = nxs * nys;
    G.W = (int)((nzs + 31) / 32);
    G.h = h, G.ox = origin_h[0], G.oy = origin_h[1], G.oz = origin_h[2];
    const size_t nbits = (size_t)G.W * (size_t)G.ncol;
    ANL_TRY(grow(v->box, v->box_cap, (size_t)ntri, sizeof(int4)));
    ANL_TRY(grow(v->cnt, v->cnt_cap, (size_t)ntri, sizeof(long long)));
    ANL_TRY(grow(v->off, v->off_cap, (size_t)ntri, sizeof(long long)));
    ANL_TRY(grow(v->axes, v->axes_cap, (size_t)(nxs + nys + nzs), sizeof(double)));
    ANL_TRY(grow(v->bits, v->bits_cap, nbits, sizeof(unsigned)));
    double* xs = v->axes;
    double* ys = xs + nxs;
    double* zq = ys + nys;
    double* zs = (double*)(v->sc + 4);
    ANL_CUDA(cudaMemsetAsync(v->sc, 0xff, sizeof(unsigned long long), st));
    ANL_CUDA(cudaMemsetAsync(v->sc + 1, 0, 3 * sizeof(unsigned long long), st));
    ANL_CUDA(cudaMemsetAsync(v->bits, 0, nbits * sizeof(unsigned), st));
    k_vox_zrange<<<vox_blocks(3 * ntri), VOX_T, 0, st>>>(tri, ntri, v->sc);
    ANL_LAUNCH_CHECK();
    k_vox_axes<<<vox_blocks(nxs + nys + nzs), VOX_T, 0, st>>>(G, v->sc, xs, ys, zq, zs);
    ANL_LAUNCH_CHECK();
    k_vox_count<<<vox_blocks(ntri), VOX_T, 0, st>>>(tri, ntri, G, xs, ys, v->box, v->cnt);
    ANL_LAUNCH_CHECK();
    ANL_TRY(scan_exclusive<long long>(v->cnt, ntri, v->off, v->part, (long long*)(v->sc + 2), st));
    k_vox_hits<<<152 * 8, VOX_T, 0, st>>>(tri, ntri, G, xs, ys, zq, zs, v->box, v->off, (const long long*)(v->sc + 2),
                                          v->bits, v->sc + 3);
    ANL_LAUNCH_CHECK();
    k_vox_parity<<<vox_blocks(G.ncol), VOX_T, 0, st>>>(G, v->bits);
    ANL_LAUNCH_CHECK();
    k_vox_fill<<<vox_blocks((int64_t)nx * ny * nz), VOX_T, 0, st>>>(G, v->bits, fill);
    ANL_LAUNCH_CHECK();
    if (stats_h) {
        ANL_CUDA(cudaMemcpyAsync(v->host, v->sc + 2, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        ANL_CUDA(cudaStreamSynchronize(st));
        stats_h[0] = (int64_t)v->host[0];
        stats_h[1] = (int64_t)v->host[1];
    }
    return ANL_OK;
}

}  // extern "C"
