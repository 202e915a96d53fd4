// anl_kernels.cuh -- launch interfaces shared by the translation units of the library.
#pragma once

#include <type_traits>

#include "anl_common.cuh"

namespace anl {

// ------------------------------------------------------------------ K u family

// u . (K u) accumulators of the APPLY_DOT passes (and ||r||^2 of the accurate residual)
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
template <>
struct DotAcc<DF> {  // the accurate residual: ||r||^2 of its FP32 values, compensated
    Acc2 a;
    __device__ void add(DF x, DF y) { a.add_prod(x.hi + x.lo, y.hi + y.lo); }
    __device__ void add_sq(float v) { a.add_prod(v, v); }
    __device__ double value() const { return a.value(); }
};


// KU_CHEB0: the first two Chebyshev steps from x = 0 in one pass: x1 = c2_0 D^-1 b is formed
// on the fly from the staged b and diagonal, then x2 = x1 + c1_1 x1 + c2_1 D^-1 (b - K x1)
enum { KU_APPLY = 0, KU_APPLY_DOT = 1, KU_RESID = 2, KU_CHEB = 3, KU_CHEB0 = 4 };

template <class T>
struct KuArgs {
    Dims d;
    int kz = 0;                      // z-layers per CTA (set by the launcher)
    const float* E = nullptr;        // element scale (already times h), full grid
    const uint8_t* nmask = nullptr;  // node mask bits (NODE_FREE_*, NODE_USED)
    const T* u = nullptr;            // input vector (masked: zeros on non-free DOFs)
    T* y = nullptr;                  // APPLY*: K u; RESID: b - K u
    const T* b = nullptr;            // RESID, CHEB
    T* dv = nullptr;                 // CHEB: Chebyshev direction, updated in place; component-major
                                     // (dv[c * N_n + n]): private to a sweep, so every warp store
                                     // and load of it covers whole 32-byte sectors
    T* xout = nullptr;               // CHEB: u + new direction
    T c1 = T(0), c2 = T(0);          // CHEB: d <- c1 d + c2 D^-1 (b - K u)
    const double* cheb = nullptr;    // CHEB: {c1, c2} in device memory (overrides c1, c2)
    int c1_zero = 0;                 // CHEB: first step of a sweep (c1 = 0, d is not read)
    int dv_keep = 1;                 // CHEB, CHEB0: 0 on the last step of a sweep (d is not stored)
    const double* cheb0 = nullptr;   // CHEB0: {c1_0, c2_0} of the step from x = 0
    const float* diag = nullptr;     // CHEB, CHEB0: inverse diagonal of K per node (0 where unused)
    T kdiag = T(0);                  // diagonal entry of Ke(1) (all 24 are equal)
    double* partials = nullptr;      // APPLY_DOT reduction scratch
    unsigned* counter = nullptr;
    int partial_capacity = 0;
    double* red_out = nullptr;       // APPLY_DOT: u . K u
    const int* done = nullptr;       // early-exit flag of the CG loop (may be null)
    // batch of right-hand sides (grid.y): slot r reads and writes its nodal vectors at
    // + r * vstride values, its done flag and dot at + r * sc_bytes bytes, its reduction scratch
    // at partials + r * part_stride and counter + r
    int nrhs = 1;
    int64_t vstride = 0;
    int sc_bytes = 0;
    int64_t part_stride = 0;
};

// The slot of a batched launch: offsets a pointer by `r` strides (elements) or bytes.
template <class P>
__host__ __device__ __forceinline__ P* slot_ptr(P* p, int r, int64_t stride) {
    return p ? p + (int64_t)r * stride : p;
}
template <class P>
__host__ __device__ __forceinline__ P* slot_bytes(P* p, int r, int bytes) {
    return p ? reinterpret_cast<P*>(reinterpret_cast<typename std::conditional<std::is_const<P>::value, const char*, char*>::type>(p) +
                                    (int64_t)r * bytes)
             : p;
}
// A K u argument block moved to batch slot r (the element fields and masks are shared).
template <class T>
__host__ __device__ __forceinline__ void ku_to_slot(KuArgs<T>& a, int r) {
    if (r == 0) return;
    a.u = slot_ptr(a.u, r, a.vstride);
    a.y = slot_ptr(a.y, r, a.vstride);
    a.b = slot_ptr(a.b, r, a.vstride);
    a.dv = slot_ptr(a.dv, r, a.vstride);
    a.xout = slot_ptr(a.xout, r, a.vstride);
    a.done = slot_bytes(a.done, r, a.sc_bytes);
    a.red_out = slot_bytes(a.red_out, r, a.sc_bytes);
    a.partials = slot_ptr(a.partials, r, a.part_stride);
    a.counter = slot_ptr(a.counter, r, (int64_t)1);
}

template <class T>
int launch_ku(int mode, const KuArgs<T>& a, const KeModal<T>& km, cudaStream_t s);
int launch_ku_resid_df(const KuArgs<DF>& a, const KeModal<DF>& km, cudaStream_t s);

// ------------------------------------------------------------------ small-grid smoother passes

// The passes of the V-cycle on the coarse levels, one CTA per 8 x 8 x 8 element box
// (anl_kbox.cu), FP32:
//   KB_RESID  y = b - K u
//   KB_CHEB   one Chebyshev step: d <- c1 d + c2 D^-1 (b - K u), xout = u + d
//   KB_CHEB0  the first two steps from x = 0 (x1 = c2_0 D^-1 b formed while staging)
//   KB_PCHEB  u <- u + P xc (the coarse-grid correction) formed while staging, then the first
//             step of a sweep (c1 = 0)
enum { KB_RESID = 0, KB_CHEB = 1, KB_CHEB0 = 2, KB_PCHEB = 3 };

struct KbArgs {
    Dims d;
    const float* E = nullptr;        // element scale (already times h), full grid
    const uint8_t* nmask = nullptr;  // node mask bits
    const float* diag = nullptr;     // inverse diagonal of K per node (0 where unused)
    const float* u = nullptr;        // iterate (KB_RESID, KB_CHEB, KB_PCHEB)
    const float* b = nullptr;        // right-hand side
    float* y = nullptr;              // KB_RESID: the residual
    float* dv = nullptr;             // Chebyshev direction (read by KB_CHEB unless c1_zero; written if dv_keep)
    float* xout = nullptr;           // the new iterate
    const double* cheb = nullptr;    // {c1, c2} of the step (KB_CHEB0: of step 1)
    const double* cheb0 = nullptr;   // KB_CHEB0: {c1_0, c2_0}
    int c1_zero = 0;                 // KB_CHEB: first step of a sweep
    int dv_keep = 1;                 // 0 on the last step of a sweep
    Dims dc{};                       // KB_PCHEB: the coarse level and its correction
    const float* xc = nullptr;
    const int* done = nullptr;       // early-exit flag of the CG loop (may be null)
    // batch of right-hand sides (grid.y), as in KuArgs; cstride: the coarse correction's slot stride
    int nrhs = 1;
    int64_t vstride = 0;
    int64_t cstride = 0;
    int sc_bytes = 0;
};

int launch_kbox(int mode, const KbArgs& a, const KeModal<float>& km, cudaStream_t s);
void kbox_prepare();

// ------------------------------------------------------------------ V-cycle tail in one CTA

// The smallest levels of the V-cycle and the coarsest dense solve in one CTA (anl_vtail.cu):
// level 0 of the tail takes b0 and returns its V-cycle correction in x0. Every level but the
// last is smoothed (`degree` Chebyshev steps before and after); the last is solved with the
// dense inverse as float pairs (ainv_hi + ainv_lo, nc x nc, symmetric).
constexpr int kTailMaxLevels = 6;
constexpr int kTailMaxSmem = 200 * 1024;
struct TailLevel {
    Dims d{};
    const float* E = nullptr;
    const uint8_t* nmask = nullptr;
    const float* diag = nullptr;
    const double* cheb = nullptr;  // (c1, c2) pairs of the level's sweep
};
struct TailArgs {
    int nlev = 0;
    TailLevel lev[kTailMaxLevels];
    int degree = 0;
    const float* b0 = nullptr;
    float* x0 = nullptr;
    const float* ainv_hi = nullptr;
    const float* ainv_lo = nullptr;
    int nc = 0;
    const int* done = nullptr;
    KeModal<float> km{};
    // right-hand-side slots: CTA r works on slot r (b0, x0 and done offset by these strides)
    int nrhs = 1;
    int64_t vstride = 0;  // floats between the slots' vectors of the first tail level
    int sc_bytes = 0;     // bytes between the slots' done flags
};
size_t tail_smem_bytes(const TailLevel* lev, int nlev);
int vtail_prepare();
int launch_vtail(const TailArgs& a, cudaStream_t s);
int launch_ainv_split(const double* ainv, int n, float* hi, float* lo, cudaStream_t s);

// ------------------------------------------------------------------ tensor-core K u (fine grid)

// The FP32 K u passes KU_APPLY, KU_APPLY_DOT, KU_RESID and KU_CHEB on the tensor cores
// (anl_kutc.cu): the edge-difference form of the element product as TF32 MMAs with a
// three-product split. kutc_prepare builds the constant operand from Ke (unit cube) once per
// device; kutc_error_flag reads the flag a kernel sets when one of its waits gave up.
int kutc_prepare(const double* ke);
int launch_kutc(int mode, const KuArgs<float>& a, const KeModal<float>& km, cudaStream_t s);
int kutc_error_flag(int* out_h);

// ------------------------------------------------------------------ debug build

// The out-of-range records of the checked translation units (ANL_IN_RANGE, anl_common.cuh).
#if ANL_DEBUG
int debug_take_ku(unsigned long long* count, long long* first);
int debug_take_kbox(unsigned long long* count, long long* first);
int debug_take_solver(unsigned long long* count, long long* first);
int debug_take_design(unsigned long long* count, long long* first);
int debug_take_vtail(unsigned long long* count, long long* first);
#endif

}  // namespace anl
