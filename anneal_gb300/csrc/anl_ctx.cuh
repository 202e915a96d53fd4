// anl_ctx.cuh -- the solver context behind the opaque anl_ctx handle.
#pragma once

#include <vector>

#include "anl_common.cuh"
#include "anl_kernels.cuh"

namespace anl {

// One level of the voxel hierarchy. Level 0 is the user's grid; level l+1 halves every
// element dimension (rounded up). Vectors are in the context's precision T.
struct Level {
    Dims d{};
    float* E = nullptr;       // element scale (times h at level 0; children sum / 4 below)
    uint8_t* eact = nullptr;  // element is (or covers) an active element
    uint8_t* nmask = nullptr; // node mask bits
    float* diag = nullptr;    // inverse diagonal of K per node (the same for its 3 DOFs; 0 if unused)
    void* x = nullptr;        // V-cycle iterate (level 0: z = M r)
    void* xt = nullptr;       // Chebyshev double buffer
    void* b = nullptr;        // right-hand side (level 0: the CG residual r)
    void* r = nullptr;        // residual scratch
    void* dv = nullptr;       // Chebyshev direction
    double lmax = 0.0;        // upper end of the smoothed spectrum of D^-1 K (diagnostics)
    // x, xt, b, r and dv hold one vector per right-hand-side slot, vs values apart (3 nn
    // rounded up to 64 values, so every slot starts on a 256-byte boundary)
    int64_t vs = 0;
};

struct FilterState {
    bool ready = false;
    int R = 0;
    double r = 0.0;
    float* w = nullptr;   // (2R+1)^3 cone weights, device
    float* Hs = nullptr;  // conv(active), zeros replaced by 1
};

constexpr int kMaxFilterR = 5;
constexpr int kChebMax = 32;
constexpr int kChebStride = 1 + 2 * kChebMax;

}  // namespace anl

struct anl_ctx {
    anl::Dims d{};
    double h = 1.0, nu = 0.3;
    int flags = 0;
    bool fp64 = false;
    size_t tsize = 4;  // bytes per vector entry

    double ke[576];                 // Ke(1) row-major (host)
    double* ke_d = nullptr;         // Ke(1) on the device (coarse assembly)
    anl::KeBlocks<double> kbd{};  // the reflection structure of Ke (checked at creation)
    anl::KeModal<double> kmd{};
    anl::KeModal<float> kmf{};
    anl::KeModal<anl::DF> kmdf{};  // kmd as double-floats (the accurate residual)
    double kdiag = 0.0;
    // lambda_max(Ke) / Ke_00 >= lambda_max(D^-1 K) for every field of element scales (the
    // element-by-element bound: x.Kx = sum_e E_e x_e.Ke x_e <= bound sum_e E_e Ke_00 |x_e|^2)
    double lmax_bound = 0.0;

    bool domain_set = false;
    int64_t nfree = 0;
    uint8_t* active = nullptr;      // level-0 active flags (ne)
    std::vector<anl::Level> lev;
#ifndef ANL_MG_DEGREE
#define ANL_MG_DEGREE 2  // Chebyshev steps per pre- and post-smoothing
#endif
    int mg_degree = ANL_MG_DEGREE;
    // Levels 2 and below: their launches cost about the same whatever their size (launch and
    // pipeline-fill latency), so more and deeper smoothing there is nearly free and saves CG
    // iterations. Measured on the 256x128x128 L-bracket (interval low ends fine / coarse,
    // coarse degree: CG iterations per solve, SIMP iterations/s):
    //   0.05 / 0.05, 2: 48.3, 21.4     0.05 / 0.05, 6: 32.6, 25.3    0.03 / 0.01, 6: 28.8, 28.2
    //   0.03 / 0.002, 6: 27.7, 29.2    0.03 / 0.002, 8: 24.1, 30.4   0.03 / 0.0005, 8: 24.5, 30.0
#ifndef ANL_MG_DEGREE_COARSE
#define ANL_MG_DEGREE_COARSE 8
#endif
    int mg_degree_coarse = ANL_MG_DEGREE_COARSE;
    // first level smoothed by the box kernels (anl_kbox.cu; FP32 contexts): on the levels below
    // 128 x 64 x 64 elements a z-marching K u launch is a chain of latencies
    int box_from = 2;
    // the finest level's K u passes on the tensor cores (anl_kutc.cu; FP32 contexts)
    bool use_tc = false;
    // first level of the one-CTA V-cycle tail (anl_vtail.cu; FP32 contexts), -1 for none
    int tail_from = -1;
    // right-hand-side slots (ANL_FLAG_RHS): the solve's per-vector state (the hierarchy's
    // vectors, p, q, the FP64 solution and right-hand side, its float-pair split, the PCG
    // scalars, the restart flags, the reduction scratch) exists once per slot; a batched solve
    // advances rb slots in lockstep, every kernel of its CG chunk taking its slot from the grid
    int rmax = 1;
    int rb = 1;                   // slots of the chunk being enqueued (1 outside a batched solve)
    int slot = 0;                 // the slot the single-vector code paths work on
    std::vector<int> last_status; // each right-hand side's status in the last anl_solve
    int cg_rb = 0;                // slots of the captured CG chunk
    int64_t part_stride = 0;      // doubles of reduction scratch per slot
    int* restart_d = nullptr;     // per-slot restart flags (p = z on the next direction update)
    // slot 0 of the per-slot arrays (the single-vector code paths point at one slot at a time)
    void* b0_base = nullptr;
    double* xbuf_base = nullptr;
    double* bbuf_base = nullptr;
    void* bdf_base = nullptr;
    anl::PcgScalars* sc_base = nullptr;
    anl::DF* sens_df = nullptr;  // the sensitivity's displacements as float pairs (grows)
    size_t sens_df_cap = 0;
    float4* oc_el = nullptr;     // the OC update's lambda-free element data (grows)
    size_t oc_el_cap = 0;
    float2* oc_gw = nullptr;
    size_t oc_gw_cap = 0;
    double* oc_state = nullptr;  // the OC bisection's device state (OcState, anl_design.cu)
    size_t oc_state_cap = 0;
    float* ainv_hi = nullptr;  // the coarsest dense inverse as float pairs (the tail's coarse solve)
    float* ainv_lo = nullptr;
#ifndef ANL_CHEB_LO
#define ANL_CHEB_LO 0.03
#endif
#ifndef ANL_CHEB_LO_COARSE
#define ANL_CHEB_LO_COARSE 0.002
#endif
    // lower ends of the smoothed intervals, as fractions of their upper end (levels 0-1, 2+)
    double cheb_lo = ANL_CHEB_LO, cheb_lo_coarse = ANL_CHEB_LO_COARSE;
    // per level: {lambda_max bound, then (c1, c2) for up to kChebMax steps}, read by the
    // smoothing kernels from device memory
    double* cheb_d = nullptr;

    // coarsest level: dense factor (FP64) or a Chebyshev fallback when too large
    int nc = 0;
    bool dense_coarse = false;
    bool coarse_ready = false;
    double* A = nullptr;     // nc x nc, lower Cholesky factor after setup
    double* Ainv = nullptr;  // nc x nc inverse
    int* flag_d = nullptr;

    // CG vectors (precision T) and FP64 solution / right-hand side
    void* p = nullptr;
    void* q = nullptr;
    void* xhi = nullptr;
    void* xlo = nullptr;
    void* xdf = nullptr;  // FP32 mode: x as (hi, lo) float pairs for the accurate residual
    void* bdf = nullptr;  // FP32 mode: the right-hand side as (hi, lo) float pairs
    void* y1 = nullptr;
    void* y2 = nullptr;
    void* tmp = nullptr;
    double* xbuf = nullptr;
    double* bbuf = nullptr;

    anl::PcgScalars* sc = nullptr;    // device
    anl::PcgScalars* sc_h = nullptr;  // pinned host mirror

    // reduction scratch
    double* partials = nullptr;
    unsigned* counter = nullptr;
    double* red_out = nullptr;  // small device result area
    double* red_h = nullptr;    // pinned host mirror
    int part_cap = 0;

    // the CG iteration chunk as a CUDA graph, captured on an internal stream and replayed on
    // the caller's stream; invalidated whenever the hierarchy's smoother spectra change
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t cg_exec = nullptr;
    bool cg_valid = false;
    int cg_nodes = 0;
    bool use_graph = true;

    anl::FilterState filt;
    float* ftmp = nullptr;   // element-field scratch (ne)
    float* ftmp2 = nullptr;  // element-field scratch (ne)
};
