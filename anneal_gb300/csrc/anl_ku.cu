// anl_ku.cu -- matrix-free hex8 operator K u and the kernels fused with it.
//
// Replaces the assembled CSR matrix of FEM.assemble (fem.py:198-201) and its SpMV inside
// scipy's CG (fem.py:224). K = sum_e E_e Ke is applied element by element in the basis of the
// trilinear modes (modal_element, anl_common.cuh): about 200 flops per element instead of the
// 1152 of the dense 24 x 24 product, taken from edge differences so that FP32 products scale
// with the local strain, not with |u|.
//
// Tiling. A CTA is 32 lanes (x) by NW warps (y) and marches up a chunk of z-layers. Lane l of
// warp w computes the element column (ie, je) = (30 bx - 1 + l, (NW-1) by - 1 + w): it loads
// its own two nodes (ie, je) and (ie, je + 1) of each node plane and takes the nodes of column
// ie + 1 from lane l + 1 by a shuffle. Corner forces are summed onto nodes without atomics:
// across x by a shuffle from lane l - 1, across y through shared memory from warp w - 1, and
// across z in registers from the previous layer. So lanes 1..30 of warps 1..NW-1 own complete
// nodes; the outer lanes and warp 0 compute the halo elements of the tile (a 13 % overlap
// at NW = 16). Edge differences of the lower node plane are carried from the previous layer,
// and warps whose 32 elements are all void skip the element arithmetic.
// HBM traffic is u once, y once, E once and the node mask once (halo re-reads hit L2).
//
// The same kernel in double-float arithmetic (T = DF, residual mode only) evaluates the FP64
// operator's residual b - K x for the FP32 solver's certification: every difference, product
// and sum is an unevaluated float pair, accurate to about 2^-48 of the terms, at a fraction
// of the cost of FP64 arithmetic on this part.
#include <algorithm>
#include <type_traits>

#include "anl_common.cuh"
#include "anl_kernels.cuh"

namespace anl {

#ifndef KU_NW32
#define KU_NW32 16  // warps per CTA of the FP32 K u kernel
#endif
#ifndef KU_MINB32
#define KU_MINB32 1  // resident CTAs per SM its registers are sized for
#endif
#ifndef KU_DEPTH
#define KU_DEPTH 3  // layers staged ahead by cp.async
#endif
#define KU_RING (KU_DEPTH + 1)

__host__ __device__ constexpr int ceil_div_d(int a, int b) { return (a + b - 1) / b; }

// node-field loads of the epilogue
__device__ __forceinline__ float ldg_t(const float* p) { return __ldg(p); }
__device__ __forceinline__ double ldg_t(const double* p) { return __ldg(p); }
__device__ __forceinline__ DF ldg_t(const DF* p) {
    const float2 t = __ldg(reinterpret_cast<const float2*>(p));
    return DF(t.x, t.y);
}

__device__ __forceinline__ float shfl_dn(float v) { return __shfl_down_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ double shfl_dn(double v) { return __shfl_down_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ DF shfl_dn(DF v) { return DF(shfl_dn(v.hi), shfl_dn(v.lo)); }
__device__ __forceinline__ float shfl_upv(float v) { return __shfl_up_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ double shfl_upv(double v) { return __shfl_up_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ DF shfl_upv(DF v) { return DF(shfl_upv(v.hi), shfl_upv(v.lo)); }

// warps per CTA: 16 in FP32 (15 owned node rows), 8 in FP64 (shared memory and registers)
template <class T>
struct KmCfg {
    static constexpr int NW = sizeof(T) == 4 ? KU_NW32 : 8;
    static constexpr int NT = 32 * NW;
    static constexpr int OX = 30;      // node columns owned per CTA
    static constexpr int OY = NW - 1;  // node rows owned per CTA
    static constexpr int MINB = sizeof(T) == 4 ? KU_MINB32 : 1;
};

constexpr unsigned FULL = 0xffffffffu;

template <class T>
__device__ __forceinline__ V3<T> shfl_down3(const V3<T>& v) {
    V3<T> r;
    r.xy.x = shfl_dn(v.xy.x);
    r.xy.y = shfl_dn(v.xy.y);
    r.z = shfl_dn(v.z);
    return r;
}
template <class T>
__device__ __forceinline__ V3<T> shfl_up3(const V3<T>& v) {
    V3<T> r;
    r.xy.x = shfl_upv(v.xy.x);
    r.xy.y = shfl_upv(v.xy.y);
    r.z = shfl_upv(v.z);
    return r;
}

// state carried from one element layer to the next (lower node plane of the next layer)
template <class T>
struct KuCarry {
    V3<T> ub[2];   // own nodes (ie, je) and (ie, je + 1)
    V3<T> dxb[2];  // Dx of rows je, je + 1
    V3<T> dyb[2];  // Dy of columns ie, ie + 1
    V3<T> acc;     // forces of the layer below on node (ie, je)
    V3<T> braw;    // CHEB0: b at node (ie, je), as staged (before the D^-1 scaling)
    float dg;      // CHEB0: the inverse diagonal at node (ie, je), as staged
};
// epilogue inputs of the next output node, loaded one layer ahead
template <class T>
struct KuEpi {
    uint8_t nm;
    T b[3], dv[3];
    float dg;  // CHEB: the inverse diagonal of the output node (level's diag array)
};

__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Shared memory of one CTA: a ring of KU_RING staged (node plane, element layer) pairs filled
// by cp.async KU_DEPTH layers ahead, and the double-buffered y hand-over between warps (row
// w + 1 is written by warp w; row 0 stays zero for warp 0).
template <class T, int MODE>
struct KuSmem {
    static constexpr int NW = KmCfg<T>::NW;
    static constexpr bool CH = MODE == KU_CHEB || MODE == KU_CHEB0;
    static constexpr int NV = 6;           // values passed to the next warp
    T u[KU_RING][NW + 1][32][3];           // staged node values (b in CHEB0)
    float E[KU_RING][NW][32];
    float D[MODE == KU_CHEB0 ? KU_RING : 1][NW + 1][32];  // CHEB0: staged inverse diagonal
    T x[2][NW + 1][NV][32];
};
static_assert((KU_RING & (KU_RING - 1)) == 0, "the cp.async ring length must be a power of two");

template <class T, int MODE>
struct KuTile {
    static constexpr int NW = KmCfg<T>::NW;
    using Smem = KuSmem<T, MODE>;
    static constexpr uint32_t SLOT_U = sizeof(T) * (NW + 1) * 32 * 3;  // bytes per ring slot
    static constexpr uint32_t SLOT_E = sizeof(float) * NW * 32;
    const KuArgs<T>& a;
    const KeModal<T>& km;
    Smem& sm;
    int lane, w;
    int NXn, NYn, NZn;
    int64_t plane, eplane;
    uint32_t s_u, s_uN, s_E;  // shared addresses of this thread's ring entries in slot 0
    uint32_t s_D, s_DN;       // CHEB0: the inverse diagonal's ring entries
    const T* src_base;        // staged node field: u, or b in CHEB0
    T c2_0 = T(0);            // CHEB0: x1 = c2_0 D^-1 b
    T c1s = T(0), c2s = T(0); // CHEB, CHEB0: the step's coefficients (read and converted once)
    const float* iD = nullptr;
    // segment geometry
    bool r0in, rNin, ein, owner;
    int64_t n0, e0;
    // staging cursor: next layer ik; sources of node plane ik + 1 and element layer ik
    int ik;
    const T* iu;
    const float* iE;

    __device__ KuTile(const KuArgs<T>& a_, const KeModal<T>& km_, Smem& sm_) : a(a_), km(km_), sm(sm_) {
        lane = threadIdx.x;
        w = threadIdx.y;
        NXn = a.d.nx + 1;
        NYn = a.d.ny + 1;
        NZn = a.d.nz + 1;
        plane = (int64_t)NXn * NYn;
        eplane = (int64_t)a.d.nx * a.d.ny;
        s_u = (uint32_t)__cvta_generic_to_shared(&sm.u[0][w][lane][0]);
        s_uN = (uint32_t)__cvta_generic_to_shared(&sm.u[0][NW][lane][0]);
        s_E = (uint32_t)__cvta_generic_to_shared(&sm.E[0][w][lane]);
        s_D = (uint32_t)__cvta_generic_to_shared(&sm.D[0][w][lane]);
        s_DN = (uint32_t)__cvta_generic_to_shared(&sm.D[0][NW][lane]);
        src_base = MODE == KU_CHEB0 ? a.b : a.u;
        if (MODE == KU_CHEB0) c2_0 = T(a.cheb0[1]);
        if (MODE == KU_CHEB || MODE == KU_CHEB0) {
            c1s = a.cheb ? T(a.cheb[0]) : a.c1;
            c2s = a.cheb ? T(a.cheb[1]) : a.c2;
        }
    }

    __device__ void set_column(int bx, int by, int k0) {
        const int ie = bx * KmCfg<T>::OX - 1 + lane, je = by * KmCfg<T>::OY - 1 + w;
        const bool xin = ie >= 0 && ie < NXn;
        r0in = xin && je >= 0 && je < NYn;
        rNin = xin && by * KmCfg<T>::OY - 1 + NW < NYn;  // the extra row of the last warp
        ein = ie >= 0 && ie < a.d.nx && je >= 0 && je < a.d.ny;
        owner = lane >= 1 && lane <= KmCfg<T>::OX && w >= 1 && xin && je < NYn;
        n0 = (int64_t)ie + (int64_t)NXn * je;
        e0 = (int64_t)ie + (int64_t)a.d.nx * je;
        ik = k0 - 2;
        iu = src_base + 3 * (n0 + (int64_t)(ik + 1) * plane);
        iE = a.E + e0 + (int64_t)ik * eplane;
        if (MODE == KU_CHEB0) iD = a.diag + n0 + (int64_t)(ik + 1) * plane;
    }

    // stages layer ik (node plane ik + 1, element layer ik) into its ring slot (zeros outside
    // the grid) when ik < kend, then advances the cursor; one commit group either way
    __device__ __forceinline__ void issue_next(int kend) {
        if (ik < kend) {
            const int pk = ik + 1;
            const bool kin = pk >= 0 && pk < NZn;
            const uint32_t so = (uint32_t)(ik & (KU_RING - 1));
            const int64_t nq = n0 + (int64_t)pk * plane;  // this thread's staged node
            const bool q0 = kin && r0in && ANL_IN_RANGE(nq, plane * NZn);
            const T* src = q0 ? iu : src_base;
            if (MODE == KU_CHEB0) {
                cp_async4(s_D + so * (uint32_t)sizeof(sm.D[0]), q0 ? iD : a.diag, q0);
                if (w == NW - 1) {
                    const bool qn = kin && rNin && ANL_IN_RANGE(nq + NXn, plane * NZn);
                    cp_async4(s_DN + so * (uint32_t)sizeof(sm.D[0]), qn ? iD + NXn : a.diag, qn);
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const uint32_t d = s_u + so * SLOT_U + c * (uint32_t)sizeof(T);
                if (sizeof(T) == 4) cp_async4(d, src + (q0 ? c : 0), q0);
                else cp_async8(d, src + (q0 ? c : 0), q0);
            }
            if (w == NW - 1) {  // node row je + 1 of the last warp
                const bool qn = kin && rNin && ANL_IN_RANGE(nq + NXn, plane * NZn);
                const T* srcn = qn ? iu + 3 * NXn : src_base;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const uint32_t d = s_uN + so * SLOT_U + c * (uint32_t)sizeof(T);
                    if (sizeof(T) == 4) cp_async4(d, srcn + (qn ? c : 0), qn);
                    else cp_async8(d, srcn + (qn ? c : 0), qn);
                }
            }
            const bool qe = ein && ik >= 0 && ik < a.d.nz && ANL_IN_RANGE(e0 + (int64_t)ik * eplane, eplane * a.d.nz);
            cp_async4(s_E + so * SLOT_E, qe ? iE : a.E, qe);
        }
        cp_async_commit();
        ++ik;
        iu += 3 * plane;
        iE += eplane;
        if (MODE == KU_CHEB0) iD += plane;
    }

    __device__ __forceinline__ void node_pair(int slot, V3<T> (&u)[2], V3<T>* raw0 = nullptr,
                                              float* d0 = nullptr) const {
        const T* p = &sm.u[slot][w][lane][0];
        constexpr int ROW = 32 * 3;
        u[0].xy.x = p[0];
        u[0].xy.y = p[1];
        u[0].z = p[2];
        u[1].xy.x = p[ROW];
        u[1].xy.y = p[ROW + 1];
        u[1].z = p[ROW + 2];
        if (MODE == KU_CHEB0) {  // x1 = c2_0 b / diag (b is zero on non-free DOFs)
            if (raw0) *raw0 = u[0];
            if (d0) *d0 = sm.D[slot][w][lane];
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                u[r] = (c2_0 * T(sm.D[slot][w + r][lane])) * u[r];
            }
        }
    }

    // epilogue loads of output node n (plane kk)
    __device__ __forceinline__ void epi_load(int64_t n, bool emit, KuEpi<T>& e) const {
        e.nm = 0;
        if (emit && ANL_IN_RANGE(n, plane * NZn)) {
            e.nm = __ldg(a.nmask + n);
            if (MODE == KU_RESID || MODE == KU_CHEB) {  // CHEB0 has b staged already
#pragma unroll
                for (int c = 0; c < 3; ++c) e.b[c] = ldg_t(a.b + 3 * n + c);
            }
            if (MODE == KU_CHEB) {
                e.dg = __ldg(a.diag + n);
#pragma unroll
                for (int c = 0; c < 3; ++c) e.dv[c] = a.c1_zero ? T(0) : a.dv[c * plane * NZn + n];
            }
        }
    }

    // carry of the node plane staged in `slot` (edge differences only, no forces yet)
    __device__ __forceinline__ void start(int slot, KuCarry<T>& c) const {
        node_pair(slot, c.ub, &c.braw, &c.dg);
        const V3<T> nb0 = shfl_down3(c.ub[0]), nb1 = shfl_down3(c.ub[1]);
        c.dxb[0] = nb0 - c.ub[0];
        c.dxb[1] = nb1 - c.ub[1];
        c.dyb[0] = c.ub[1] - c.ub[0];
        c.dyb[1] = nb1 - nb0;
        c.acc = v3zero<T>();
    }

    // Element layer kk (between node planes kk and kk + 1), staged in ring slot kk % KU_RING;
    // `n` is node (ie, je, kk). Stages layer kk + KU_DEPTH, writes node n when `emit`, and the
    // carry of plane kk + 1 to `o`. `ep` holds node n's epilogue inputs, `epn` receives those
    // of node n + plane.
    __device__ __forceinline__ void step(int kk, int kend, bool emit, int64_t n, int par, const KuCarry<T>& in,
                                         KuCarry<T>& o, const KuEpi<T>& ep, KuEpi<T>& epn, DotAcc<T>& dot) {
        const int slot = kk & (KU_RING - 1);
        issue_next(kend);
        epi_load(n + plane, owner && kk + 1 < kend, epn);
        V3<T> cu[2];
        node_pair(slot, cu, &o.braw, &o.dg);
        const float Ee = sm.E[slot][w][lane];
        // edge differences of the upper plane
        const V3<T> un0 = shfl_down3(cu[0]), un1 = shfl_down3(cu[1]);
        o.dxb[0] = un0 - cu[0];
        o.dxb[1] = un1 - cu[1];
        o.dyb[0] = cu[1] - cu[0];
        o.dyb[1] = un1 - un0;
        V3<T> dz[2][2];
        dz[0][0] = cu[0] - in.ub[0];
        dz[0][1] = cu[1] - in.ub[1];
        dz[1][0] = shfl_down3(dz[0][0]);
        dz[1][1] = shfl_down3(dz[0][1]);
        o.ub[0] = cu[0];
        o.ub[1] = cu[1];

        V3<T> f[2][2][2];
        if (__any_sync(FULL, Ee != 0.f)) {
            modal_element<T>(km, T(Ee), in.dxb, o.dxb, in.dyb, o.dyb, dz, f);
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) (&f[0][0][0])[q] = v3zero<T>();
        }
        // x: corners px = 1 of lane l - 1 are corners px = 0 of lane l
#pragma unroll
        for (int py = 0; py < 2; ++py)
#pragma unroll
            for (int pz = 0; pz < 2; ++pz) f[0][py][pz] = f[0][py][pz] + shfl_up3(f[1][py][pz]);
        // y: corners py = 1 of warp w - 1 are corners py = 0 of warp w
        T* xo = &sm.x[par][w + 1][0][lane];
#pragma unroll
        for (int pz = 0; pz < 2; ++pz) {
            xo[(3 * pz) * 32] = f[0][1][pz].xy.x;
            xo[(3 * pz + 1) * 32] = f[0][1][pz].xy.y;
            xo[(3 * pz + 2) * 32] = f[0][1][pz].z;
        }
        cp_async_wait<KU_DEPTH - 1>();  // this thread's copies of layer kk + 1 have landed
        __syncthreads();                // ... everyone's, and the y hand-over is visible
        const T* xi = &sm.x[par][w][0][lane];
#pragma unroll
        for (int pz = 0; pz < 2; ++pz) {
            V3<T> r;
            r.xy.x = xi[(3 * pz) * 32];
            r.xy.y = xi[(3 * pz + 1) * 32];
            r.z = xi[(3 * pz + 2) * 32];
            f[0][0][pz] = f[0][0][pz] + r;
        }
        o.acc = f[0][0][1];
        if (emit && owner && ANL_IN_RANGE(n, plane * NZn)) {
            const V3<T> yv = in.acc + f[0][0][0];
            const T y[3] = {yv.xy.x, yv.xy.y, yv.z};
            const T u[3] = {in.ub[0].xy.x, in.ub[0].xy.y, in.ub[0].z};
            const T b[3] = {MODE == KU_CHEB0 ? in.braw.xy.x : ep.b[0], MODE == KU_CHEB0 ? in.braw.xy.y : ep.b[1],
                            MODE == KU_CHEB0 ? in.braw.z : ep.b[2]};
            const uint8_t nm = ep.nm;
            if (MODE == KU_APPLY || MODE == KU_APPLY_DOT) {
                T* yp = a.y + 3 * n;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const T v = (nm >> c) & 1 ? y[c] : T(0);
                    yp[c] = v;
                    if (MODE == KU_APPLY_DOT) dot.add(u[c], v);
                }
            } else if (MODE == KU_RESID) {
                if constexpr (std::is_same<T, DF>::value) {  // FP32 residual and ||r||^2
                    float* rp = reinterpret_cast<float*>(a.y) + 3 * n;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const DF rd = b[c] - y[c];
                        const float rf = (nm >> c) & 1 ? rd.hi + rd.lo : 0.f;
                        rp[c] = rf;
                        dot.add_sq(rf);
                    }
                } else {
                    T* yp = a.y + 3 * n;
#pragma unroll
                    for (int c = 0; c < 3; ++c) yp[c] = (nm >> c) & 1 ? b[c] - y[c] : T(0);
                }
            } else if (Smem::CH) {
                // the level's inverse diagonal (0 on nodes without elements): staged with the
                // plane in CHEB0, loaded with the epilogue inputs in CHEB
                const T inv = T(MODE == KU_CHEB0 ? in.dg : ep.dg);
                const T c1 = c1s, c2 = c2s;
                T* dp = a.dv + n;  // component-major: dp[c * N_n]
                T* xp = a.xout + 3 * n;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    T dn = T(0), xn = T(0);
                    if ((nm >> c) & 1) {
                        const T dprev = MODE == KU_CHEB0 ? u[c] : ep.dv[c];  // CHEB0: d_0 = x1
                        dn = c1 * dprev + c2 * (b[c] - y[c]) * inv;
                        xn = u[c] + dn;
                    }
                    if (a.dv_keep) dp[c * plane * NZn] = dn;
                    xp[c] = xn;
                }
            }
        }
    }
};

// Work: the (node column tile, node plane) pairs, column-major, split into equal contiguous
// ranges, one per CTA (a.kz planes each). A CTA walks its range as one or two z-segments of a
// column tile; each segment recomputes the element layer below its first plane.
template <class T, int MODE>
__global__ void __launch_bounds__(KmCfg<T>::NT, KmCfg<T>::MINB) ku_kernel(KuArgs<T> a, KeModal<T> km) {
    constexpr int NT = KmCfg<T>::NT;
    using Tile = KuTile<T, MODE>;
    extern __shared__ __align__(16) unsigned char ku_smem_raw[];
    auto& sm = *reinterpret_cast<typename Tile::Smem*>(ku_smem_raw);
    __shared__ double sred[NT / 32];
    ku_to_slot(a, blockIdx.y);
    if (a.done != nullptr && *a.done) return;

    Tile t(a, km, sm);
    if (threadIdx.y == 0)  // the y hand-over row read by warp 0 stays zero
        for (int q = 0; q < 2 * Tile::Smem::NV; ++q) sm.x[q / Tile::Smem::NV][0][q % Tile::Smem::NV][threadIdx.x] = T(0);
    const int gx = ceil_div_d(t.NXn, KmCfg<T>::OX);
    const int64_t total = (int64_t)gx * ceil_div_d(t.NYn, KmCfg<T>::OY) * t.NZn;
    int64_t idx = (int64_t)blockIdx.x * a.kz;
    const int64_t idx_end = min(total, idx + a.kz);
    DotAcc<T> dot;
    int par = 0;
    while (idx < idx_end) {
        const int64_t col = idx / t.NZn;
        const int k0 = (int)(idx - col * t.NZn);
        const int kend = (int)min((int64_t)t.NZn, (int64_t)k0 + (idx_end - idx));
        idx += kend - k0;
        t.set_column((int)(col % gx), (int)(col / gx), k0);
        // prologue: layers k0-2 (its node plane k0-1 only) .. k0-2+KU_DEPTH in flight, one
        // commit group each; step kk then stages layer kk+KU_DEPTH into the slot of kk-1
#pragma unroll
        for (int q = 0; q <= KU_DEPTH; ++q) t.issue_next(kend);
        cp_async_wait<KU_DEPTH - 1>();  // layers k0-2 and k0-1 have landed
        __syncthreads();
        KuCarry<T> A, B;
        KuEpi<T> EA, EB;
        t.start((k0 - 2) & (KU_RING - 1), A);
        int64_t n = t.n0 + (int64_t)(k0 - 1) * t.plane;  // node (ie, je, kk)
        t.epi_load(n, false, EA);
        __syncthreads();  // slot of layer k0-2 is read before the loop refills it
        if constexpr (std::is_same<T, DF>::value) {
            // one step per trip and the carries copied: the pair arithmetic of a step is long
            // enough that a second inlined copy of it overflows the instruction cache
            for (int kk = k0 - 1; kk < kend; ++kk) {
                t.step(kk, kend, kk >= k0, n, par, A, B, EA, EB, dot);
                par ^= 1;
                n += t.plane;
                A = B;
                EA = EB;
            }
        } else {
            for (int kk = k0 - 1; kk < kend; kk += 2) {
                t.step(kk, kend, kk >= k0, n, par, A, B, EA, EB, dot);
                par ^= 1;
                n += t.plane;
                if (kk + 1 >= kend) break;
                t.step(kk + 1, kend, true, n, par, B, A, EB, EA, dot);
                par ^= 1;
                n += t.plane;
            }
        }
        cp_async_wait<0>();
        __syncthreads();  // the ring is idle before the next segment restages it
    }
    if (MODE == KU_APPLY_DOT || (MODE == KU_RESID && std::is_same<T, DF>::value)) {
        const int tid = threadIdx.y * 32 + threadIdx.x;
        if constexpr (std::is_same<T, double>::value) {
            double v[1] = {dot.value()};
            block_sum<1, NT>(v, sred, tid);
            finish_reduction<1, NT>(v, blockIdx.x, gridDim.x, a.partials, a.counter, a.red_out, tid, sred);
        } else {
            float h[1] = {dot.a.s}, l[1] = {dot.a.c};
            float2* sp = reinterpret_cast<float2*>(sred);
            block_pair_sum<1, NT>(h, l, sp, tid);
            finish_pair_reduction<1, NT>(h, l, blockIdx.x, gridDim.x, a.partials, a.counter, a.red_out, tid, sp);
        }
    }
}

template <class T, int MODE>
static int ku_resident() {
    static int resident = 0;
    if (resident == 0) {
        int dev = 0, sms = 1, occ = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int bytes = (int)sizeof(KuSmem<T, MODE>);
        cudaFuncSetAttribute(ku_kernel<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ku_kernel<T, MODE>, KmCfg<T>::NT, bytes);
        resident = std::max(1, sms * std::max(1, occ));
    }
    return resident;
}

// Evaluates the occupancy of every K u variant once (outside any stream capture).
void ku_prepare() {
    ku_resident<float, KU_APPLY>();
    ku_resident<float, KU_APPLY_DOT>();
    ku_resident<float, KU_RESID>();
    ku_resident<float, KU_CHEB>();
    ku_resident<float, KU_CHEB0>();
    ku_resident<double, KU_APPLY>();
    ku_resident<double, KU_APPLY_DOT>();
    ku_resident<double, KU_RESID>();
    ku_resident<double, KU_CHEB>();
    ku_resident<double, KU_CHEB0>();
    ku_resident<DF, KU_RESID>();
}

template <class T>
int launch_ku(int mode, const KuArgs<T>& args, const KeModal<T>& km, cudaStream_t s) {
    KuArgs<T> a = args;
    const Dims& d = a.d;
    const int NXn = d.nx + 1, NYn = d.ny + 1, NZn = d.nz + 1;
    const int64_t total = (int64_t)ceil_div(NXn, KmCfg<T>::OX) * ceil_div(NYn, KmCfg<T>::OY) * NZn;
    int resident = 1;
    switch (mode) {
        case KU_APPLY: resident = ku_resident<T, KU_APPLY>(); break;
        case KU_APPLY_DOT: resident = ku_resident<T, KU_APPLY_DOT>(); break;
        case KU_RESID: resident = ku_resident<T, KU_RESID>(); break;
        case KU_CHEB: resident = ku_resident<T, KU_CHEB>(); break;
        case KU_CHEB0: resident = ku_resident<T, KU_CHEB0>(); break;
        default: return ANL_ERR_BADARG;
    }
    // one wave of CTAs per right-hand side. A segment costs one extra element layer, but a
    // plane step is a ~1 us latency chain, so small (coarse-level) grids spread over many short
    // segments. Every slot of a batch gets the partition a single solve gets, so its sums (the
    // p.Kp reduction follows the CTAs) and its iterates are those of its own solve.
    const int per_rhs = std::max(1, resident);
    a.kz = (int)std::max<int64_t>(2, (total + per_rhs - 1) / per_rhs);
    const int blocks = (int)((total + a.kz - 1) / a.kz);
    dim3 block(32, KmCfg<T>::NW);
    const dim3 grid(blocks, std::max(1, a.nrhs));
    if (mode == KU_APPLY_DOT && blocks > a.partial_capacity) {
        set_error("K u dot: %d blocks exceed the reduction scratch (%d)", blocks, a.partial_capacity);
        return ANL_ERR_BADARG;
    }
    switch (mode) {
        case KU_APPLY: ku_kernel<T, KU_APPLY><<<grid, block, sizeof(KuSmem<T, KU_APPLY>), s>>>(a, km); break;
        case KU_APPLY_DOT: ku_kernel<T, KU_APPLY_DOT><<<grid, block, sizeof(KuSmem<T, KU_APPLY_DOT>), s>>>(a, km); break;
        case KU_RESID: ku_kernel<T, KU_RESID><<<grid, block, sizeof(KuSmem<T, KU_RESID>), s>>>(a, km); break;
        case KU_CHEB: ku_kernel<T, KU_CHEB><<<grid, block, sizeof(KuSmem<T, KU_CHEB>), s>>>(a, km); break;
        case KU_CHEB0: ku_kernel<T, KU_CHEB0><<<grid, block, sizeof(KuSmem<T, KU_CHEB0>), s>>>(a, km); break;
        default: return ANL_ERR_BADARG;
    }
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

// r = b - K x in double-float arithmetic (the modal form with the FP64 constants): a.u and a.b
// hold x and the right-hand side as (hi, lo) float pairs, a.y receives the FP32 residual (as
// DF*), ||r||^2 goes to a.red_out.
int launch_ku_resid_df(const KuArgs<DF>& args, const KeModal<DF>& km, cudaStream_t s) {
    KuArgs<DF> a = args;
    const Dims& d = a.d;
    const int NXn = d.nx + 1, NYn = d.ny + 1, NZn = d.nz + 1;
    const int64_t total = (int64_t)ceil_div(NXn, KmCfg<DF>::OX) * ceil_div(NYn, KmCfg<DF>::OY) * NZn;
    const int resident = ku_resident<DF, KU_RESID>();
    a.kz = (int)std::max<int64_t>(2, (total + resident - 1) / resident);
    const int blocks = (int)((total + a.kz - 1) / a.kz);
    if (blocks > a.partial_capacity) {
        set_error("accurate residual: %d blocks exceed the reduction scratch (%d)", blocks, a.partial_capacity);
        return ANL_ERR_BADARG;
    }
    ku_kernel<DF, KU_RESID><<<blocks, dim3(32, KmCfg<DF>::NW), sizeof(KuSmem<DF, KU_RESID>), s>>>(a, km);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

// Upper bound of the K u grids (one CTA per SM and resident slot, at most 8 per SM): sizes the
// reduction scratch.
int ku_grid_blocks(const Dims& d) {
    (void)d;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return 8 * sms;
}

template int launch_ku<float>(int, const KuArgs<float>&, const KeModal<float>&, cudaStream_t);
template int launch_ku<double>(int, const KuArgs<double>&, const KeModal<double>&, cudaStream_t);

ANL_DEBUG_UNIT(ku)

}  // namespace anl
