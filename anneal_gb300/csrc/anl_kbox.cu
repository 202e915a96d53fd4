// anl_kbox.cu -- the multigrid smoother passes on small grids: one CTA per 8 x 8 x 8 element box.
//
// The fine-grid K u kernel (anl_ku.cu) marches CTAs up z-columns through a cp.async plane
// ring: at 12.8M DOF it keeps HBM busy, but on the coarse levels of the V-cycle (a few
// thousand to a few hundred thousand nodes) a launch is a chain of latencies (ring prologue,
// one barrier per layer) and costs 6-9 us whatever the level's size. Here every CTA owns a
// box of 7 x 7 x 7 nodes and computes the 8 x 8 x 8 elements around them in one shot:
//
//   1. stage the 9 x 9 x 9 nodes of the box (the iterate; in the fused variants the iterate is
//      formed on the fly) and the 512 element scales in shared memory, and prefetch the owned
//      node's epilogue inputs (mask, inverse diagonal, right-hand side, direction);
//   2. one thread per element: the modal element product (modal_element, anl_common.cuh)
//      writes the 8 corner forces to shared memory;
//   3. one thread per owned node: sums the 8 corner forces that meet there (no atomics, a fixed
//      order) and applies the pass's epilogue.
//
// A node of the box boundary belongs to the neighbouring box, which recomputes the elements
// around it (a (8/7)^3 overlap that costs nothing at these sizes). The passes:
//   KB_RESID  r = b - K x
//   KB_CHEB   d <- c1 d + c2 D^-1 (b - K x), x' = x + d          (one Chebyshev step)
//   KB_CHEB0  the first two Chebyshev steps from x = 0: x1 = c2_0 D^-1 b formed while staging
//   KB_PCHEB  x <- x + P x_c (the coarse-grid correction, trilinear prolongation) formed while
//             staging, then the first Chebyshev step of the post-smoothing sweep
// The arithmetic of a pass is the same as the ku_kernel pass it replaces (FP32, the same modal
// constants), so only the summation order of the corner forces differs.
#include "anl_common.cuh"
#include "anl_kernels.cuh"

namespace anl {

namespace {

constexpr int BE = 8;               // elements per box side
constexpr int BN = BE + 1;          // staged nodes per box side
constexpr int BO = BE - 1;          // owned nodes per box side
constexpr int BT = BE * BE * BE;    // threads per CTA: one element each
constexpr int BNN = BN * BN * BN;   // staged nodes
constexpr int BON = BO * BO * BO;   // owned nodes
constexpr int BC = 6;               // staged coarse nodes per side (fused prolongation)
constexpr int BCN = BC * BC * BC;

// shared memory layout (floats)
constexpr int OFF_U = 0;                          // [BNN][3] staged iterate
constexpr int OFF_E = OFF_U + 3 * BNN + 1;        // [BT] element scales (the +1 keeps 8-byte rows apart)
constexpr int OFF_F = OFF_E + BT;                 // [8 corners][3][BT] corner forces
constexpr int OFF_C = OFF_F + 24 * BT;            // [BCN][3] staged coarse correction (KB_PCHEB)
constexpr int SMEM_FLOATS = OFF_C + 3 * BCN;
constexpr size_t SMEM_BYTES = sizeof(float) * SMEM_FLOATS;

__host__ __device__ constexpr int boxes(int nodes) { return (nodes + BO - 1) / BO; }

template <int MODE>
__global__ void __launch_bounds__(BT) kbox_kernel(KbArgs a, KeModal<float> km) {
    if (blockIdx.y > 0) {  // batch slot r of a multi-right-hand-side launch
        const int r = blockIdx.y;
        a.u = slot_ptr(a.u, r, a.vstride);
        a.b = slot_ptr(a.b, r, a.vstride);
        a.y = slot_ptr(a.y, r, a.vstride);
        a.dv = slot_ptr(a.dv, r, a.vstride);
        a.xout = slot_ptr(a.xout, r, a.vstride);
        a.xc = slot_ptr(a.xc, r, a.cstride);
        a.done = slot_bytes(a.done, r, a.sc_bytes);
    }
    if (a.done != nullptr && *a.done) return;
    extern __shared__ __align__(16) float kb_smem[];
    float* su = kb_smem + OFF_U;
    float* sE = kb_smem + OFF_E;
    float* sF = kb_smem + OFF_F;
    float* sc = kb_smem + OFF_C;
    const int t = threadIdx.x;
    const Dims d = a.d;
    const int NXn = d.nx + 1, NYn = d.ny + 1, NZn = d.nz + 1;
    const int gx = boxes(NXn), gy = boxes(NYn);
    const int bx = blockIdx.x % gx, by = (blockIdx.x / gx) % gy, bz = blockIdx.x / (gx * gy);
    const int ox = BO * bx - 1, oy = BO * by - 1, oz = BO * bz - 1;  // box origin (nodes and elements)

    // ---- epilogue inputs of the owned node (prefetched; they are not needed until step 3)
    const bool owner = t < BON;
    const int ax = 1 + t % BO, ay = 1 + (t / BO) % BO, az = 1 + t / (BO * BO);
    const int gi = ox + ax, gj = oy + ay, gk = oz + az;
    const bool emit = owner && gi < NXn && gj < NYn && gk < NZn && ANL_IN_RANGE(d.node(gi, gj, gk), d.nn());
    const int64_t on = emit ? d.node(gi, gj, gk) : 0;
    uint8_t nm = 0;
    float inv = 0.f, bo[3] = {0.f, 0.f, 0.f}, dprev[3] = {0.f, 0.f, 0.f};
    if (emit) {
        nm = __ldg(a.nmask + on);
#pragma unroll
        for (int c = 0; c < 3; ++c) bo[c] = a.b[3 * on + c];
        if (MODE != KB_RESID) inv = a.diag[on];
        if (MODE == KB_CHEB && !a.c1_zero) {
#pragma unroll
            for (int c = 0; c < 3; ++c) dprev[c] = a.dv[3 * on + c];
        }
    }

    // ---- the coarse-grid correction's nodes (KB_PCHEB)
    const int cox = (ox > 0 ? ox : 0) >> 1, coy = (oy > 0 ? oy : 0) >> 1, coz = (oz > 0 ? oz : 0) >> 1;
    if (MODE == KB_PCHEB) {
        const Dims dc = a.dc;
        for (int q = t; q < BCN; q += BT) {
            const int I = cox + q % BC, J = coy + (q / BC) % BC, K = coz + q / (BC * BC);
            float v0 = 0.f, v1 = 0.f, v2 = 0.f;
            if (I <= dc.nx && J <= dc.ny && K <= dc.nz && ANL_IN_RANGE(dc.node(I, J, K), dc.nn())) {
                const float* p = a.xc + 3 * dc.node(I, J, K);
                v0 = p[0];
                v1 = p[1];
                v2 = p[2];
            }
            sc[3 * q] = v0;
            sc[3 * q + 1] = v1;
            sc[3 * q + 2] = v2;
        }
        __syncthreads();
    }

    // ---- stage the box's nodes and element scales
    const float c20 = MODE == KB_CHEB0 ? (float)a.cheb0[1] : 0.f;
    for (int q = t; q < BNN; q += BT) {
        const int lx = q % BN, ly = (q / BN) % BN, lz = q / (BN * BN);
        const int i = ox + lx, j = oy + ly, k = oz + lz;
        float v[3] = {0.f, 0.f, 0.f};
        if (i >= 0 && j >= 0 && k >= 0 && i < NXn && j < NYn && k < NZn && ANL_IN_RANGE(d.node(i, j, k), d.nn())) {
            const int64_t n = d.node(i, j, k);
            if (MODE == KB_CHEB0) {  // x1 = c2_0 D^-1 b (b is zero on non-free DOFs)
                const float s = c20 * __ldg(a.diag + n);
#pragma unroll
                for (int c = 0; c < 3; ++c) v[c] = s * a.b[3 * n + c];
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c) v[c] = a.u[3 * n + c];
            }
            if (MODE == KB_PCHEB) {  // x += P x_c on free DOFs: the mean of the coarse nodes around
                const uint8_t m = __ldg(a.nmask + n);
                if (m & 7) {
                    const int I0 = (i >> 1) - cox, J0 = (j >> 1) - coy, K0 = (k >> 1) - coz;
                    const int di = i & 1, dj = j & 1, dk = k & 1;
                    const float w = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f) * (dk ? 0.5f : 1.f);
                    float acc[3] = {0.f, 0.f, 0.f};
                    for (int g = 0; g <= dk; ++g)
                        for (int bb = 0; bb <= dj; ++bb)
                            for (int aa = 0; aa <= di; ++aa) {
                                const float* p = sc + 3 * ((I0 + aa) + BC * ((J0 + bb) + BC * (K0 + g)));
                                acc[0] += p[0];
                                acc[1] += p[1];
                                acc[2] += p[2];
                            }
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        if ((m >> c) & 1) v[c] += w * acc[c];
                }
            }
        }
        su[3 * q] = v[0];
        su[3 * q + 1] = v[1];
        su[3 * q + 2] = v[2];
    }
    const int tx = t & (BE - 1), ty = (t / BE) & (BE - 1), tz = t / (BE * BE);
    {
        const int i = ox + tx, j = oy + ty, k = oz + tz;
        const bool in = i >= 0 && j >= 0 && k >= 0 && i < d.nx && j < d.ny && k < d.nz &&
                        ANL_IN_RANGE(d.elem(i, j, k), d.ne());
        sE[t] = in ? __ldg(a.E + d.elem(i, j, k)) : 0.f;
    }
    __syncthreads();

    // ---- one element per thread: corner forces to shared memory
    const float Ee = sE[t];
    V3<float> f[2][2][2];
    if (__any_sync(0xffffffffu, Ee != 0.f)) {
        V3<float> u[2][2][2];
#pragma unroll
        for (int pz = 0; pz < 2; ++pz)
#pragma unroll
            for (int py = 0; py < 2; ++py)
#pragma unroll
                for (int px = 0; px < 2; ++px) {
                    const float* p = su + 3 * ((tx + px) + BN * ((ty + py) + BN * (tz + pz)));
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
        modal_element<float>(km, Ee, dxb, dxt, dyb, dyt, dz, f);
    } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) (&f[0][0][0])[q] = v3zero<float>();
    }
#pragma unroll
    for (int px = 0; px < 2; ++px)
#pragma unroll
        for (int py = 0; py < 2; ++py)
#pragma unroll
            for (int pz = 0; pz < 2; ++pz) {
                const int corner = px + 2 * py + 4 * pz;
                sF[(3 * corner) * BT + t] = f[px][py][pz].xy.x;
                sF[(3 * corner + 1) * BT + t] = f[px][py][pz].xy.y;
                sF[(3 * corner + 2) * BT + t] = f[px][py][pz].z;
            }
    __syncthreads();

    // ---- one owned node per thread: sum the corner forces, then the pass's epilogue
    if (!emit) return;
    float y[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int ez = 0; ez < 2; ++ez)
#pragma unroll
        for (int ey = 0; ey < 2; ++ey)
#pragma unroll
            for (int ex = 0; ex < 2; ++ex) {
                // element (ax - 1 + ex, ...) meets the node at its corner (1 - ex, 1 - ey, 1 - ez)
                const int te = (ax - 1 + ex) + BE * ((ay - 1 + ey) + BE * (az - 1 + ez));
                const int corner = (1 - ex) + 2 * (1 - ey) + 4 * (1 - ez);
#pragma unroll
                for (int c = 0; c < 3; ++c) y[c] += sF[(3 * corner + c) * BT + te];
            }
    if (MODE == KB_RESID) {
        float* o = a.y + 3 * on;
#pragma unroll
        for (int c = 0; c < 3; ++c) o[c] = (nm >> c) & 1 ? bo[c] - y[c] : 0.f;
        return;
    }
    const float* uo = su + 3 * (ax + BN * (ay + BN * az));
    const float c1 = (float)a.cheb[0], c2 = (float)a.cheb[1];
    float* dp = a.dv + 3 * on;
    float* xp = a.xout + 3 * on;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float dn = 0.f, xn = 0.f;
        if ((nm >> c) & 1) {
            // the previous direction: d_0 = x1 after the fused first step; none on a sweep's
            // first step (c1 = 0)
            const float dpv = MODE == KB_CHEB0 ? uo[c] : MODE == KB_CHEB ? dprev[c] : 0.f;
            dn = (MODE == KB_PCHEB || (MODE == KB_CHEB && a.c1_zero)) ? c2 * (bo[c] - y[c]) * inv
                                                                      : c1 * dpv + c2 * (bo[c] - y[c]) * inv;
            xn = uo[c] + dn;
        }
        if (a.dv_keep) dp[c] = dn;
        xp[c] = xn;
    }
}

}  // namespace

void kbox_prepare() {
    static bool done = false;
    if (done) return;
    cudaFuncSetAttribute(kbox_kernel<KB_RESID>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    cudaFuncSetAttribute(kbox_kernel<KB_CHEB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    cudaFuncSetAttribute(kbox_kernel<KB_CHEB0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    cudaFuncSetAttribute(kbox_kernel<KB_PCHEB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    done = true;
}

int launch_kbox(int mode, const KbArgs& a, const KeModal<float>& km, cudaStream_t s) {
    const int64_t nb = (int64_t)boxes(a.d.nx + 1) * boxes(a.d.ny + 1) * boxes(a.d.nz + 1);
    if (nb > (1ll << 31) - 1) {
        set_error("box smoother: grid %d x %d x %d too large", a.d.nx, a.d.ny, a.d.nz);
        return ANL_ERR_BADARG;
    }
    const dim3 grid((unsigned)nb, (unsigned)std::max(1, a.nrhs)), block(BT);
    switch (mode) {
        case KB_RESID: kbox_kernel<KB_RESID><<<grid, block, SMEM_BYTES, s>>>(a, km); break;
        case KB_CHEB: kbox_kernel<KB_CHEB><<<grid, block, SMEM_BYTES, s>>>(a, km); break;
        case KB_CHEB0: kbox_kernel<KB_CHEB0><<<grid, block, SMEM_BYTES, s>>>(a, km); break;
        case KB_PCHEB: kbox_kernel<KB_PCHEB><<<grid, block, SMEM_BYTES, s>>>(a, km); break;
        default: return ANL_ERR_BADARG;
    }
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

ANL_DEBUG_UNIT(kbox)

}  // namespace anl
