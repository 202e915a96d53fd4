// anl_kutc.cu -- the fine-grid K u family on the tensor cores (tcgen05, FP32 through a
// three-product TF32 split).
//
// The element product f_e = E_e Ke u_e is written in the edge-difference basis: Ke annihilates
// translations, so Ke u_e = G w_e with w_e the 7 corner displacements relative to corner 0 and
// those in turn sums of 7 edge differences of the element (Dx(i), Dy(i), Dz(i), Dy(i+1),
// Dz(i+1), Dz(i, j+1), Dz(i+1, j+1) for the element whose corner 0 is node (i, j, k)). G is the
// constant 24 x 21 matrix that maps the edge differences to the 24 corner forces. Products then
// scale with the local strain, not with |u|, as in the modal SIMT kernel (anl_ku.cu).
//
// For a row of 128 elements along x (one MMA, M = 128) every edge difference is an entry of a
// per-node-row array, and element i reads entry i or i + 1 of it. The MMA's A operand is such
// an array in shared memory, read through a descriptor whose rows are 16 bytes apart (one
// padded 3-vector per node): the shift by one node is a 16-byte change of the start address,
// so no per-element gather exists. Each MMA takes two 16-byte K chunks (8 TF32 values): four
// MMAs cover the seven edges, with B = G^T (N = 32: 8 corners x 4 padded components).
//
// Precision: A = A_hi + A_lo and B = B_hi + B_lo, each part exactly representable in TF32;
// A_hi B_hi + A_lo B_hi + A_hi B_lo with FP32 accumulation keeps about 21 bits of the product,
// the accuracy of the FP32 SIMT kernel.
//
// Tiling: a CTA owns 128 node columns in x (plus node nx when its tile ends the grid), 7 node
// rows in y (it computes 8 element rows: the row below its first node row is a halo row) and a
// z-segment of node planes, marching up one element layer at a time:
//   1. producers (warps 4-7) stage node planes with cp.async (4-plane ring), then build the
//      difference arrays of the layer (hi and lo parts) and the forces of element x0 - 1 (the
//      neighbouring tile's last element, by the modal SIMT product) for lane 0 of warp 0;
//   2. one thread issues the 96 MMAs of the layer (8 rows x 4 K steps x 3 split products) into
//      TMEM and commits them to an mbarrier;
//   3. the epilogue warps (0-3, thread t = element x0 + t) read their row accumulators from
//      TMEM, scale by E, and sum the corner forces onto nodes: across x by a shuffle (lane 0 of
//      warps 1-3 through shared memory), across y and z in registers (each thread walks its
//      rows in order and carries the upper corners to the next row and layer).
#include <algorithm>
#include <cmath>
#include <vector>

#include "anl_common.cuh"
#include "anl_kernels.cuh"
#include "anl_tc.cuh"

namespace anl {

namespace {

using namespace tc;

constexpr int TX = 128;       // elements per x-tile (the MMA's M)
constexpr int RY = 8;         // element rows per CTA (row 0 is the halo row)
constexpr int OY = RY - 1;    // owned node rows
constexpr int NR = RY + 1;    // node rows a layer reads
constexpr int DE = 130;       // difference entries per row: nodes x0 .. x0 + 129
constexpr int NT = 256;       // threads: warps 0-3 epilogue, 4-7 producers
constexpr int NP = 128;       // producer threads
constexpr int NBUF = 2;       // operand buffers and TMEM accumulator slots
constexpr int NXB = 4;        // x hand-over buffers

constexpr int DROW = DE * 16;                   // bytes per difference row (float4 entries)
constexpr int NDROW = RY + RY + NR + 1;         // Dx[RY], Dy[RY], Dz[NR], one padding row
constexpr int DPART = NDROW * DROW;             // one split part of one buffer
constexpr int DBUF = 2 * DPART;                 // hi and lo parts
constexpr int OFF_D = 0;                        // [NBUF][hi, lo][DPART]
constexpr int OFF_BHI = OFF_D + NBUF * DBUF;    // B = G^T: 32 x 32 TF32, 4 KB per part
constexpr int OFF_BLO = OFF_BHI + 4096;
constexpr int OFF_XCH = OFF_BLO + 4096;         // corner px = 1 forces of element x0 - 1: [NXB][RY][12]
constexpr int OFF_XEP = OFF_XCH + NXB * RY * 12 * 4;  // lane 31 -> lane 0 of the next epilogue warp: [RY][4][12]
constexpr int OFF_BAR = OFF_XEP + RY * 4 * 12 * 4;
constexpr int SMEM_BYTES = OFF_BAR + 128;
static_assert(OFF_BHI % 16 == 0 && OFF_XCH % 16 == 0 && OFF_BAR % 8 == 0, "alignment");
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");

// difference-row indices inside a part
__host__ __device__ constexpr int drow_x(int r) { return r; }
__host__ __device__ constexpr int drow_y(int r) { return RY + r; }
__host__ __device__ constexpr int drow_z(int r) { return 2 * RY + r; }

constexpr uint32_t kWaitLimit = 1u << 20;  // mbarrier polls before a wait gives up (well over a second)

// B = G^T in the K-major core-matrix layout: core matrix (row group g of 8 outputs, K chunk c)
// at byte (4 c + g) * 128, row n % 8 at 16 (n % 8) within it.
__host__ __device__ constexpr int b_index(int n, int kk) {  // float index of B[n][kk]
    return (((kk >> 2) * 4 + (n >> 3)) * 128 + (n & 7) * 16) / 4 + (kk & 3);
}

struct TcConst {
    float bhi[1024];  // B parts in the smem layout
    float blo[1024];
};

__device__ __forceinline__ float tf32_hi(float v) { return __uint_as_float(__float_as_uint(v) & 0xFFFFE000u); }

// node-value load of the layer's source field, zero outside the grid; with `diag` set (the
// fused first two Chebyshev steps) the field is x1 = c2_0 D^-1 b, formed from b on the fly
struct NodeSrc {
    const float* f;
    int NXn, NYn, NZn;
    int64_t plane;
    const float* diag;
    float c20;
    __device__ __forceinline__ void get(int i, int j, int k, float (&v)[3]) const {
        if (i >= 0 && j >= 0 && k >= 0 && i < NXn && j < NYn && k < NZn) {
            const int64_t n = (int64_t)i + (int64_t)NXn * j + plane * k;
            const float* p = f + 3 * n;
            const float s = diag ? c20 * __ldg(diag + n) : 1.f;
            v[0] = s * __ldg(p);
            v[1] = s * __ldg(p + 1);
            v[2] = s * __ldg(p + 2);
        } else {
            v[0] = v[1] = v[2] = 0.f;
        }
    }
};

template <int MODE>
__global__ void __launch_bounds__(NT, 1) kutc_kernel(KuArgs<float> a, KeModal<float> km, const TcConst* __restrict__ cst,
                                                      int* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    float* xch = reinterpret_cast<float*>(smem + OFF_XCH);
    float* xep = reinterpret_cast<float*>(smem + OFF_XEP);
    uint64_t* bar_full = reinterpret_cast<uint64_t*>(smem + OFF_BAR);      // [NBUF] MMAs of a layer done
    uint64_t* bar_tfree = bar_full + NBUF;                                // [NBUF] epilogue done with a slot
    uint64_t* bar_xfull = bar_tfree + NBUF;                               // [NXB] producers' hand-over written
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_xfull + NXB);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    volatile int* ep_abort = abort_flag + 1;  // the epilogue's snapshot of abort_flag
    __shared__ double sred[NT / 32];
    if (a.done != nullptr && *a.done) return;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const Dims d = a.d;
    const int NXn = d.nx + 1, NYn = d.ny + 1, NZn = d.nz + 1;
    const int gxt = (d.nx + TX - 1) / TX, gyt = (NYn + OY - 1) / OY;
    const int ncol = gxt * gyt;
    const int col = blockIdx.x % ncol, seg = blockIdx.x / ncol;
    const int x0 = TX * (col % gxt), j0 = OY * (col / gxt);
    const int k0 = seg * a.kz, kend = min(NZn, k0 + a.kz);
    const int nlayer = kend - (k0 - 1);   // layers k0 - 1 .. kend - 1 (the first one is a halo layer)
    const bool last_x = x0 + TX >= d.nx;
    const int64_t plane_n = (int64_t)NXn * NYn;

    // ---- set-up: B parts, padding rows, barriers, TMEM (512 columns: two slots of 8 x 32)
    for (int q = tid; q < 1024; q += NT) {
        reinterpret_cast<float*>(smem + OFF_BHI)[q] = cst->bhi[q];
        reinterpret_cast<float*>(smem + OFF_BLO)[q] = cst->blo[q];
    }
    for (int q = tid; q < NBUF * 2 * DE * 4; q += NT) {  // the padding row of every part
        const int part = q / (DE * 4), w = q - part * (DE * 4);
        reinterpret_cast<float*>(smem + OFF_D + part * DPART + (NDROW - 1) * DROW)[w] = 0.f;
    }
    if (tid == 0) {
        for (int b = 0; b < NBUF; ++b) {
            mbar_init(bar_full + b, 1);
            mbar_init(bar_tfree + b, 4);
        }
        for (int b = 0; b < NXB; ++b) mbar_init(bar_xfull + b, NP);
        *abort_flag = 0;
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    fence_proxy_async_smem();
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t sbase = smem_u32(smem);
    DotAcc<float> dot;

    if (warp >= 4) {
        // ================================================================ producers
        // Producer thread pt owns difference entry e = pt (node column x0 + e) of every row and
        // marches up the planes with it: plane k of its column is carried in registers, plane
        // k + 1 is loaded one layer ahead, the x neighbour comes from the next lane by a shuffle
        // (lane 31 loads the next warp's first column itself; thread 127 also writes entry 128,
        // which the shifted operand reads of element 127 need).
        const int pt = tid - (NT - NP), e = pt, i = x0 + e;
        const float* src = MODE == KU_CHEB0 ? a.b : a.u;
        const NodeSrc U{src, NXn, NYn, NZn, plane_n, MODE == KU_CHEB0 ? a.diag : nullptr,
                        MODE == KU_CHEB0 ? (float)a.cheb0[1] : 1.f};
        const uint32_t idesc = idesc_tf32(128, 32);
        float cur[NR][3], nxt[NR][3];
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            U.get(i, j0 - 1 + r, k0 - 1, cur[r]);
            U.get(i, j0 - 1 + r, k0, nxt[r]);
        }
        auto put = [&](unsigned char* D, int row, int ent, const float (&v)[3]) {
            float4 hi, lo;
            hi = make_float4(tf32_hi(v[0]), tf32_hi(v[1]), tf32_hi(v[2]), 0.f);
            lo = make_float4(v[0] - hi.x, v[1] - hi.y, v[2] - hi.z, 0.f);
            *reinterpret_cast<float4*>(D + row * DROW + ent * 16) = hi;
            *reinterpret_cast<float4*>(D + DPART + row * DROW + ent * 16) = lo;
        };
        // Every producer runs all nlayer iterations and reaches every named barrier: after a wait
        // gave up (abort_flag), the waits and MMAs are skipped, never the barriers.
        for (int it = 0; it < nlayer; ++it) {
            const int k = k0 - 1 + it, b = it & 1, xb = it & (NXB - 1);
            // the next column at plane k (lane 31) and, for entry 128, at plane k + 1 (thread 127)
            float nx0[NR][3], nx1[NR][3];
            if (lane == 31) {
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    U.get(i + 1, j0 - 1 + r, k, nx0[r]);
                    if (pt == NP - 1) U.get(i + 1, j0 - 1 + r, k + 1, nx1[r]);
                }
            }
            // plane k + 2 of this column, for the next layer
            float nn2[NR][3];
#pragma unroll
            for (int r = 0; r < NR; ++r) U.get(i, j0 - 1 + r, k + 2, nn2[r]);
            // corner px = 1 forces of element x0 - 1 (modal SIMT product) for lane 0 of epilogue
            // warp 0, one row per lane 0..7 of warp 4
            if (warp == 4 && lane < RY) {
                const int r = lane, ii = x0 - 1, j = j0 - 1 + r;
                float* h = xch + (xb * RY + r) * 12;
                const float Ee = (ii >= 0 && ii < d.nx && j >= 0 && j < d.ny && k >= 0 && k < d.nz)
                                     ? __ldg(a.E + d.elem(ii, j, k)) : 0.f;
                V3<float> f[2][2][2];
                if (Ee != 0.f) {
                    V3<float> c[2][2][2];
#pragma unroll
                    for (int px = 0; px < 2; ++px)
#pragma unroll
                        for (int py = 0; py < 2; ++py)
#pragma unroll
                            for (int pz = 0; pz < 2; ++pz) {
                                float v[3];
                                U.get(ii + px, j + py, k + pz, v);
                                c[px][py][pz].xy = make_float2(v[0], v[1]);
                                c[px][py][pz].z = v[2];
                            }
                    V3<float> dxb[2], dxt[2], dyb[2], dyt[2], dz[2][2];
#pragma unroll
                    for (int q2 = 0; q2 < 2; ++q2) {
                        dxb[q2] = c[1][q2][0] - c[0][q2][0];
                        dxt[q2] = c[1][q2][1] - c[0][q2][1];
                        dyb[q2] = c[q2][1][0] - c[q2][0][0];
                        dyt[q2] = c[q2][1][1] - c[q2][0][1];
                    }
#pragma unroll
                    for (int px = 0; px < 2; ++px)
#pragma unroll
                        for (int py = 0; py < 2; ++py) dz[px][py] = c[px][py][1] - c[px][py][0];
                    modal_element<float>(km, Ee, dxb, dxt, dyb, dyt, dz, f);
                } else {
#pragma unroll
                    for (int q2 = 0; q2 < 8; ++q2) (&f[0][0][0])[q2] = v3zero<float>();
                }
#pragma unroll
                for (int pz = 0; pz < 2; ++pz)
#pragma unroll
                    for (int py = 0; py < 2; ++py) {
                        const int cc = py + 2 * pz;
                        h[cc * 3] = f[1][py][pz].xy.x;
                        h[cc * 3 + 1] = f[1][py][pz].xy.y;
                        h[cc * 3 + 2] = f[1][py][pz].z;
                    }
            }
            if (it >= NBUF && !*abort_flag && !mbar_wait(bar_full + b, ((it >> 1) - 1) & 1, kWaitLimit)) {
                atomicExch(err, 1);  // the MMAs of layer k - 2 never completed
                *abort_flag = 1;
            }
            unsigned char* D = smem + OFF_D + b * DBUF;
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                float dz[3], dx[3], dy[3], xn[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    xn[c] = __shfl_down_sync(0xffffffffu, cur[r][c], 1);
                    if (lane == 31) xn[c] = nx0[r][c];
                    dz[c] = nxt[r][c] - cur[r][c];
                    dx[c] = xn[c] - cur[r][c];
                    if (r < RY) dy[c] = cur[r + 1][c] - cur[r][c];
                }
                put(D, drow_z(r), e, dz);
                if (r < RY) {
                    put(D, drow_x(r), e, dx);
                    put(D, drow_y(r), e, dy);
                }
                if (pt == NP - 1) {  // entry 128: Dy and Dz of node column x0 + 128
                    float ez[3], ey[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        ez[c] = nx1[r][c] - nx0[r][c];
                        if (r < RY) ey[c] = nx0[r + 1][c] - nx0[r][c];
                    }
                    put(D, drow_z(r), TX, ez);
                    if (r < RY) put(D, drow_y(r), TX, ey);
                }
            }
#pragma unroll
            for (int r = 0; r < NR; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    cur[r][c] = nxt[r][c];
                    nxt[r][c] = nn2[r][c];
                }
            fence_proxy_async_smem();
            mbar_arrive(bar_xfull + xb);
            asm volatile("bar.sync 2, 128;\n" ::: "memory");  // every producer's operands are written
            if (pt == 0 && !*abort_flag) {  // the MMA issuer: 8 rows x 4 K steps x 3 split products into slot b
                bool ok = true;
                if (it >= NBUF) ok = mbar_wait(bar_tfree + b, ((it >> 1) - 1) & 1, kWaitLimit);  // epilogue k - 2
                if (!ok) {
                    atomicExch(err, 1);
                    *abort_flag = 1;
                } else {
                    tc_fence_after_sync();
                    const uint32_t dhi = sbase + OFF_D + b * DBUF, dlo = dhi + DPART;
                    uint64_t ah[4], al[4], bh[4], bl[4];
                    const uint32_t st[4] = {(uint32_t)(drow_x(0) * DROW), (uint32_t)(drow_z(0) * DROW),
                                            (uint32_t)(drow_y(0) * DROW + 16), (uint32_t)(drow_z(1) * DROW + 16)};
                    const uint32_t lb[4] = {(uint32_t)((drow_y(0) - drow_x(0)) * DROW), (uint32_t)DROW,
                                            (uint32_t)((drow_z(0) - drow_y(0)) * DROW), (uint32_t)DROW};
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        ah[p] = smem_desc(dhi + st[p], lb[p], 128);
                        al[p] = smem_desc(dlo + st[p], lb[p], 128);
                        bh[p] = smem_desc(sbase + OFF_BHI + 1024 * p, 512, 128);
                        bl[p] = smem_desc(sbase + OFF_BLO + 1024 * p, 512, 128);
                    }
#pragma unroll
                    for (int r = 0; r < RY; ++r) {
                        const uint32_t dcol = tmem + b * 256 + 32 * r;
                        const uint64_t dr = (uint64_t)((r * DROW) >> 4);
#pragma unroll
                        for (int p = 0; p < 4; ++p) {
                            mma_tf32(dcol, ah[p] + dr, bh[p], idesc, p > 0 ? 1u : 0u);
                            mma_tf32(dcol, al[p] + dr, bh[p], idesc, 1u);
                            mma_tf32(dcol, ah[p] + dr, bl[p], idesc, 1u);
                        }
                    }
                    mma_commit(bar_full + b);
                }
            }
            __syncwarp();
        }
    } else {
        // ================================================================ epilogue
        const int et = tid, ex = x0 + et;
        // node nx has no element to its right: when the grid ends exactly at this tile's last
        // element, that element's thread also emits node nx
        const bool extra = last_x && et == TX - 1 && ex == d.nx - 1;
        float zc[OY][3], zce[OY][3];
#pragma unroll
        for (int o = 0; o < OY; ++o)
#pragma unroll
            for (int c = 0; c < 3; ++c) zc[o][c] = zce[o][c] = 0.f;
        const uint32_t tl = tmem + ((uint32_t)(32 * warp) << 16);
        for (int it = 0; it < nlayer; ++it) {
            const int k = k0 - 1 + it, b = it & 1, xb = it & (NXB - 1);
            // The four epilogue warps meet at a named barrier every row, so they leave the loop
            // together: thread 0 snapshots the abort flag, the barrier publishes the snapshot.
            if (tid == 0) *ep_abort = *abort_flag;
            asm volatile("bar.sync 1, 128;\n" ::: "memory");
            if (*ep_abort) break;
            // element scales and node masks of the layer (loaded before the waits)
            float Er[RY];
            uint8_t nmr[RY];
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                const int j = j0 - 1 + r;
                Er[r] = (ex < d.nx && j >= 0 && j < d.ny && k >= 0 && k < d.nz) ? __ldg(a.E + d.elem(ex, j, k)) : 0.f;
                nmr[r] = (r >= 1 && k >= k0 && ex < NXn && j < NYn) ? __ldg(a.nmask + (int64_t)ex + (int64_t)NXn * j +
                                                                              plane_n * k)
                                                                    : (uint8_t)0;
            }
            const bool got = mbar_wait(bar_full + b, (it >> 1) & 1, kWaitLimit) &&
                             mbar_wait(bar_xfull + xb, (it >> 2) & 1, kWaitLimit);
            if (!got) {  // the layer's results are not there: finish the layer (every warp reaches
                         // the row barriers) and leave at the next snapshot
                atomicExch(err, 1);
                *abort_flag = 1;
            }
            tc_fence_after_sync();
            const float* hx = xch + xb * RY * 12;  // element x0 - 1 (warp 0 only)
            float hc[2][3] = {}, hce[2][3] = {};
            uint32_t va[32], vb[32];
            tmem_ld32_raw(tl + b * 256, va);
            tmem_wait_ld32(va);
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                uint32_t(&cur)[32] = (r & 1) ? vb : va;
                uint32_t(&nxt)[32] = (r & 1) ? va : vb;
                if (r + 1 < RY) tmem_ld32_raw(tl + b * 256 + 32 * (r + 1), nxt);
                float g[4][3], ge[4][3];
                // lane 31 hands its px = 1 corners to lane 0 of the next warp (through shared
                // memory, one named barrier of the four epilogue warps per row)
                if (lane == 31 && warp < 3) {
                    float* hw = xep + (r * 4 + warp + 1) * 12;
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc)
#pragma unroll
                        for (int c = 0; c < 3; ++c) hw[cc * 3 + c] = Er[r] * __uint_as_float(cur[16 + 4 * cc + c]);
                }
                asm volatile("bar.sync 1, 128;\n" ::: "memory");
                const float* h = warp == 0 ? hx + r * 12 : xep + (r * 4 + warp) * 12;
#pragma unroll
                for (int cc = 0; cc < 4; ++cc)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float f0 = Er[r] * __uint_as_float(cur[4 * cc + c]);
                        const float f1 = Er[r] * __uint_as_float(cur[16 + 4 * cc + c]);
                        float up = __shfl_up_sync(0xffffffffu, f1, 1);
                        if (lane == 0) up = h[cc * 3 + c];
                        g[cc][c] = f0 + up;
                        ge[cc][c] = f1;
                    }
                if (r == 0) {
#pragma unroll
                    for (int pz = 0; pz < 2; ++pz)
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            hc[pz][c] = g[1 + 2 * pz][c];
                            hce[pz][c] = ge[1 + 2 * pz][c];
                        }
                } else {
                    float tot[3], tote[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float y0 = g[0][c] + hc[0][c], y1 = g[2][c] + hc[1][c];
                        const float e0 = ge[0][c] + hce[0][c], e1 = ge[2][c] + hce[1][c];
                        hc[0][c] = g[1][c];
                        hc[1][c] = g[3][c];
                        hce[0][c] = ge[1][c];
                        hce[1][c] = ge[3][c];
                        tot[c] = y0 + zc[r - 1][c];
                        zc[r - 1][c] = y1;
                        tote[c] = e0 + zce[r - 1][c];
                        zce[r - 1][c] = e1;
                    }
                    const int j = j0 - 1 + r;
                    if (k >= k0 && j < NYn) {
                        auto emit = [&](int xi, const float (&y)[3], uint8_t nm) {
                            const int64_t n = (int64_t)xi + (int64_t)NXn * j + plane_n * k;
                            if (MODE == KU_APPLY || MODE == KU_APPLY_DOT) {
                                float* yp = a.y + 3 * n;
#pragma unroll
                                for (int c = 0; c < 3; ++c) {
                                    const float vv = (nm >> c) & 1 ? y[c] : 0.f;
                                    yp[c] = vv;
                                    if (MODE == KU_APPLY_DOT) dot.add(__ldg(a.u + 3 * n + c), vv);
                                }
                            } else if (MODE == KU_RESID) {
                                float* yp = a.y + 3 * n;
#pragma unroll
                                for (int c = 0; c < 3; ++c) yp[c] = (nm >> c) & 1 ? a.b[3 * n + c] - y[c] : 0.f;
                            } else {  // KU_CHEB, KU_CHEB0
                                const float inv = a.diag[n];
                                const float c1 = a.cheb ? (float)a.cheb[0] : a.c1, c2 = a.cheb ? (float)a.cheb[1] : a.c2;
                                const float c20 = MODE == KU_CHEB0 ? (float)a.cheb0[1] : 0.f;
                                float* dp = a.dv + n;  // component-major: dp[c * N_n]
                                const int64_t nnode = a.d.nn();
                                float* xp = a.xout + 3 * n;
#pragma unroll
                                for (int c = 0; c < 3; ++c) {
                                    float dn = 0.f, xn = 0.f;
                                    if ((nm >> c) & 1) {
                                        const float bc = a.b[3 * n + c];
                                        // the iterate: x1 = c2_0 D^-1 b (which is also the first
                                        // direction) in the fused pass, else the staged field
                                        const float uc = MODE == KU_CHEB0 ? c20 * inv * bc : __ldg(a.u + 3 * n + c);
                                        const float dprev = MODE == KU_CHEB0 ? uc : (a.c1_zero ? 0.f : dp[c * nnode]);
                                        dn = c1 * dprev + c2 * (bc - y[c]) * inv;
                                        xn = uc + dn;
                                    }
                                    if (a.dv_keep) dp[c * nnode] = dn;
                                    xp[c] = xn;
                                }
                            }
                        };
                        if (ex < NXn) emit(ex, tot, nmr[r]);
                        if (extra) emit(d.nx, tote, __ldg(a.nmask + (int64_t)d.nx + (int64_t)NXn * j + plane_n * k));
                    }
                }
                if (r + 1 < RY) tmem_wait_ld32(nxt);
            }
            tc_fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar_tfree + b);
        }
    }
    tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after_sync();
        tmem_dealloc(tmem, 512);
    }
    if (MODE == KU_APPLY_DOT) {
        float h[1] = {dot.a.s}, l[1] = {dot.a.c};
        float2* sp = reinterpret_cast<float2*>(sred);
        block_pair_sum<1, NT>(h, l, sp, tid);
        finish_pair_reduction<1, NT>(h, l, blockIdx.x, gridDim.x, a.partials, a.counter, a.red_out, tid, sp);
    }
}

TcConst* g_const[64] = {};
int* g_err[64] = {};

}  // namespace

// The constant B = G^T parts for Ke of a unit cube (the element scale carries h): built on the
// host in FP64 from ke (row-major 24 x 24, DOF order 3 a + c with a the LOCAL corner of
// fem.py:20-21), split into TF32 hi and lo parts.
static void build_tc_const(const double* ke, TcConst* out) {
    // LOCAL corner index of the corner (px, py, pz)
    auto local = [](int px, int py, int pz) { return (pz << 2) | (py ? (px ? 2 : 3) : (px ? 1 : 0)); };
    // edges (K chunks): 0 Dx(i), 1 Dy(i), 2 Dz(i), 3 Dz(i, j+1), 4 Dy(i+1), 5 Dz(i+1), 6 Dz(i+1, j+1)
    // corner displacements relative to corner (0,0,0) as sums of edges
    int uses[8][3];  // per corner (px + 2 py + 4 pz): up to 3 edges, -1 = none
    for (int q = 0; q < 8; ++q) uses[q][0] = uses[q][1] = uses[q][2] = -1;
    auto set = [&](int px, int py, int pz, int e0, int e1, int e2) {
        int* u = uses[px + 2 * py + 4 * pz];
        u[0] = e0, u[1] = e1, u[2] = e2;
    };
    set(1, 0, 0, 0, -1, -1);
    set(0, 1, 0, 1, -1, -1);
    set(0, 0, 1, 2, -1, -1);
    set(1, 1, 0, 0, 4, -1);
    set(1, 0, 1, 0, 5, -1);
    set(0, 1, 1, 1, 3, -1);
    set(1, 1, 1, 0, 4, 6);
    double G[32][32] = {};  // [output n][K index]
    for (int px = 0; px < 2; ++px)
        for (int py = 0; py < 2; ++py)
            for (int pz = 0; pz < 2; ++pz) {
                // output corner (px', py', pz') = (px, py, pz) at column 4 (4 px + py + 2 pz) + comp
                const int a_loc = local(px, py, pz);
                const int n0 = 4 * (4 * px + py + 2 * pz);
                for (int qx = 0; qx < 2; ++qx)
                    for (int qy = 0; qy < 2; ++qy)
                        for (int qz = 0; qz < 2; ++qz) {
                            const int* u = uses[qx + 2 * qy + 4 * qz];
                            const int b_loc = local(qx, qy, qz);
                            for (int t = 0; t < 3; ++t) {
                                if (u[t] < 0) continue;
                                for (int ci = 0; ci < 3; ++ci)
                                    for (int cj = 0; cj < 3; ++cj)
                                        G[n0 + ci][4 * u[t] + cj] += ke[(3 * a_loc + ci) * 24 + 3 * b_loc + cj];
                            }
                        }
            }
    auto tf32 = [](double v) {  // round to TF32 (10 explicit mantissa bits), as an FP32 value
        const float f = (float)v;
        if (f == 0.f || !std::isfinite(f)) return f;
        int e;
        const double m = std::frexp((double)f, &e);  // f = m 2^e, 0.5 <= |m| < 1
        const double s = std::ldexp(std::nearbyint(std::ldexp(m, 11)), e - 11);
        return (float)s;
    };
    for (int n = 0; n < 32; ++n)
        for (int kk = 0; kk < 32; ++kk) {
            const float hi = tf32(G[n][kk]);
            const float lo = tf32(G[n][kk] - (double)hi);
            out->bhi[b_index(n, kk)] = hi;
            out->blo[b_index(n, kk)] = lo;
        }
}

int kutc_prepare(const double* ke) {
    int dev = 0;
    ANL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return ANL_ERR_BADARG;
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    if (g_const[dev]) return ANL_OK;
    TcConst h;
    build_tc_const(ke, &h);
    TcConst* dcst = nullptr;
    int* derr = nullptr;
    ANL_CUDA(cudaMalloc((void**)&dcst, sizeof(TcConst)));
    ANL_CUDA(cudaMalloc((void**)&derr, sizeof(int)));
    ANL_CUDA(cudaMemcpy(dcst, &h, sizeof(TcConst), cudaMemcpyHostToDevice));
    ANL_CUDA(cudaMemset(derr, 0, sizeof(int)));
    ANL_CUDA(cudaFuncSetAttribute(kutc_kernel<KU_APPLY>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    ANL_CUDA(cudaFuncSetAttribute(kutc_kernel<KU_APPLY_DOT>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    ANL_CUDA(cudaFuncSetAttribute(kutc_kernel<KU_RESID>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    ANL_CUDA(cudaFuncSetAttribute(kutc_kernel<KU_CHEB>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    ANL_CUDA(cudaFuncSetAttribute(kutc_kernel<KU_CHEB0>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    g_const[dev] = dcst;
    g_err[dev] = derr;
    return ANL_OK;
}

int kutc_error_flag(int* out_h) {
    int dev = 0;
    ANL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !g_err[dev]) {
        *out_h = 0;
        return ANL_OK;
    }
    ANL_CUDA(cudaMemcpy(out_h, g_err[dev], sizeof(int), cudaMemcpyDeviceToHost));
    return ANL_OK;
}

// Launch: the CTAs are (x-tile, y-tile, z-segment) triples, one per SM.
int launch_kutc(int mode, const KuArgs<float>& args, const KeModal<float>& km, cudaStream_t s) {
    int dev = 0;
    ANL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !g_const[dev]) {
        set_error("tensor-core K u used before kutc_prepare");
        return ANL_ERR_STATE;
    }
    KuArgs<float> a = args;
    const Dims& d = a.d;
    const int gxt = (d.nx + TX - 1) / TX, gyt = (d.ny + 1 + OY - 1) / OY;
    const int ncol = gxt * gyt;
    int sms = 1;
    ANL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int NZn = d.nz + 1;
    const int nseg = std::max(1, std::min(NZn, (sms + ncol - 1) / ncol));
    a.kz = (NZn + nseg - 1) / nseg;
    const int segs = (NZn + a.kz - 1) / a.kz;
    const int blocks = ncol * segs;
    if (mode == KU_APPLY_DOT && blocks > a.partial_capacity) {
        set_error("tensor-core K u dot: %d blocks exceed the reduction scratch (%d)", blocks, a.partial_capacity);
        return ANL_ERR_BADARG;
    }
    switch (mode) {
        case KU_APPLY: kutc_kernel<KU_APPLY><<<blocks, NT, SMEM_BYTES, s>>>(a, km, g_const[dev], g_err[dev]); break;
        case KU_APPLY_DOT:
            kutc_kernel<KU_APPLY_DOT><<<blocks, NT, SMEM_BYTES, s>>>(a, km, g_const[dev], g_err[dev]);
            break;
        case KU_RESID: kutc_kernel<KU_RESID><<<blocks, NT, SMEM_BYTES, s>>>(a, km, g_const[dev], g_err[dev]); break;
        case KU_CHEB: kutc_kernel<KU_CHEB><<<blocks, NT, SMEM_BYTES, s>>>(a, km, g_const[dev], g_err[dev]); break;
        case KU_CHEB0: kutc_kernel<KU_CHEB0><<<blocks, NT, SMEM_BYTES, s>>>(a, km, g_const[dev], g_err[dev]); break;
        default: return ANL_ERR_BADARG;
    }
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

}  // namespace anl
