/*
 * anneal_gb300.h -- C ABI of the GB300 (sm_103a) voxel SIMP library.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream, returns an int
 * status (ANL_OK = 0) and allocates nothing except inside anl_ctx_create. Arrays:
 *
 *   element fields  N_e = nx*ny*nz values, x fastest (fem.py:87-127), zero on inactive
 *                   elements; float unless stated
 *   nodal vectors   3*N_n values, N_n = (nx+1)(ny+1)(nz+1), DOF = 3*node + c (fem.py:143),
 *                   double unless stated; non-free DOFs read as zero and are written as zero
 *
 * Each declaration names the reference function it replaces (anneal 0.3.0, path:line).
 */
#ifndef ANNEAL_GB300_H
#define ANNEAL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct anl_ctx anl_ctx;
typedef void* anl_stream_t; /* a cudaStream_t; NULL is the legacy default stream */

enum {
    ANL_OK = 0,
    ANL_ERR_MAXITER = 1,   /* CG did not reach rtol in maxiter iterations (fem.py:225-229) */
    ANL_ERR_NONFINITE = 2, /* a non-finite value appeared in the solve (fem.py:225) */
    ANL_ERR_BREAKDOWN = 3, /* p.Kp <= 0: the operator is not positive definite */
    ANL_ERR_BADARG = 4,
    ANL_ERR_CUDA = 5,
    ANL_ERR_SINGULAR = 6, /* reserved (tiny coarse-grid pivots are regularised, not reported) */
    ANL_ERR_NOMEM = 7,
    ANL_ERR_STATE = 8, /* a call that needs anl_set_domain / anl_filter_init came first */
    ANL_ERR_STAGNATION = 9 /* an FP32 solve stopped improving above rtol: finish it in FP64 */
};

enum { ANL_FLAG_FP64 = 1 /* K u, smoothers and CG vectors in FP64 (default: FP32) */ };
/* Right-hand-side slots of an FP32 context (flags bits 8-15, 1..255; default 1): anl_solve
   with 1 < nrhs <= n solves its cases together, see anl_solve. Each slot holds its own CG
   vectors and V-cycle vectors on every level (about 60 bytes per node). */
#define ANL_FLAG_RHS(n) ((int)(n) << 8)

int anl_version(void);
/* Text of the last error in the calling thread ("" if none). */
const char* anl_last_error(void);

/* ---------------------------------------------------------------- context (FEM) */

/* Replaces FEM.__init__ (fem.py:133-196) minus the CSR build: the operator stays matrix-free.
   Allocates the solver workspaces (multigrid hierarchy, CG vectors, reduction scratch). */
int anl_ctx_create(anl_ctx** out, int nx, int ny, int nz, double h, double nu, int flags);
void anl_ctx_destroy(anl_ctx* ctx);

/* Free-DOF rule of fem.py:142-155: a DOF is free when its node is touched by an active
   element and the DOF is not fixed. active: uint8 per element; fixed: uint8 per DOF.
   Writes the number of free DOFs to *nfree_h (host). */
int anl_set_domain(anl_ctx* ctx, const uint8_t* active, const uint8_t* fixed, int64_t* nfree_h,
                   anl_stream_t stream);

/* Free-DOF mask as uint8 per DOF (1 = free): FEM.free (fem.py:150) in full-grid form. */
int anl_free_mask(anl_ctx* ctx, uint8_t* mask, anl_stream_t stream);

/* ---------------------------------------------------------------- operator and solve */

/* y = K u with K = sum_e escale[e] Ke(h): replaces FEM.assemble (fem.py:198-201) followed by
   K @ u. escale is the per-element stiffness scale Ee (optimize.py:118), float. u and y are
   float (default context) or double (ANL_FLAG_FP64). */
int anl_apply_K(anl_ctx* ctx, const float* escale, const void* u, void* y, anl_stream_t stream);

/* Replaces FEM.solve (fem.py:206-232): solves K x = f for nrhs right-hand sides by CG
   preconditioned with a geometric-multigrid V-cycle: one after another, as the reference does,
   or, in an FP32 context created with ANL_FLAG_RHS(R) and 1 < nrhs <= R, together (every kernel
   of an iteration advances all cases, each with its own CG scalars, residual replacements and
   acceptance; a case's iterates are those of its own solve). f and x are nrhs
   consecutive nodal vectors (double); x holds the initial guesses on entry (x0_list).
   rebuild != 0 re-estimates the smoother spectra and refactors the coarse grid (the
   reference's AMG rebuild, fem.py:207-216); otherwise the last ones are kept. iters / relres
   (host arrays of nrhs) receive the CG iterations and final true relative residuals
   ||f - K x|| / ||f|| of the FP64 operator.
   Acceptance: a solve returns ANL_OK when its true residual meets ||f - K x|| <= rtol ||f||.
   The one exception is an FP64 context whose true residual has stopped falling at the
   attainable accuracy of FP64 arithmetic: it also returns ANL_OK once another round of
   iterations has not halved the residual, if relres <= max(100 rtol, 1e-10); relres then
   exceeds rtol. An FP32 context never accepts above rtol: it returns ANL_ERR_STAGNATION
   (x holds its best iterate) so the caller can finish the solve in an FP64 context.
   Returns ANL_ERR_MAXITER, ANL_ERR_NONFINITE or ANL_ERR_BREAKDOWN where the reference raises
   SolverError. */
int anl_solve(anl_ctx* ctx, const float* escale, const double* f, double* x, int nrhs, double rtol,
              int maxiter, int rebuild, int* iters, double* relres, anl_stream_t stream);

/* Status of right-hand side k (0 <= k < nrhs) in the last anl_solve on this context (ANL_OK,
   ANL_ERR_MAXITER, ...); anl_solve itself returns the first non-OK one. No reference
   counterpart: the reference raises on the first failing case (fem.py:225-229). */
int anl_solve_status(const anl_ctx* ctx, int k);

/* sum over DOFs of a[i] * b[i] (double vectors): the compliance f @ u (optimize.py:125). */
int anl_dot(anl_ctx* ctx, const double* a, const double* b, double* out_h, anl_stream_t stream);

/* ---------------------------------------------------------------- sensitivity */

/* ce[e] = u_e^T Ke(h) u_e on active elements: FEM.element_energy (fem.py:239-242). */
int anl_element_energy(anl_ctx* ctx, const double* u, float* ce, anl_stream_t stream);

/* Fused sensitivity (optimize.py:126-141 up to the filter backward):
     dc  = sum_c coef[c] * (-p xphys^(p-1) (1 - emin) E0 phi ce_c),  ce_c = u_c^T Ke u_c
     out = min(dc, 0) * dxp
     dv  = phi * dxp          (the argument of the volume filter backward, optimize.py:142)
   u: nrhs (<= 16) nodal vectors; coef: host array of nrhs combination weights (w for "sum",
   the p-norm coefficients for "worst"). dxp may be NULL (projection off: dxp = 1); dv may
   be NULL. */
int anl_sensitivity(anl_ctx* ctx, const double* u, int nrhs, const double* coef, const float* xphys,
                    const float* dxp, const float* phi, double p, double emin, double E0, float* out,
                    float* dv, anl_stream_t stream);

/* escale[e] = E0 * phi (emin + xphys^p (1 - emin)) on active elements, zero elsewhere: the
   stiffness scale Ee of optimize.py:118 (anl_apply_K / anl_solve apply Ke(h) = h Ke(1)). */
int anl_stiffness_scale(anl_ctx* ctx, const float* xphys, const float* phi, double E0, double emin,
                        double p, float* escale, anl_stream_t stream);

/* ---------------------------------------------------------------- density filter */

/* Filter.__init__ (optimize.py:25-34): cone weights max(0, r - |d|) on a (2R+1)^3 box,
   R = max(ceil(r) - 1, 1) (R <= 5), Hs = conv(active) with zeros set to 1. */
int anl_filter_init(anl_ctx* ctx, double r_vox, anl_stream_t stream);
/* Filter.forward (optimize.py:41-43): out = conv(in * active) / Hs on active elements. */
int anl_filter_fwd(anl_ctx* ctx, const float* in, float* out, anl_stream_t stream);
/* Filter.backward (optimize.py:45-47): out = conv(in / Hs) * active. */
int anl_filter_bwd(anl_ctx* ctx, const float* in, float* out, anl_stream_t stream);

/* physical (optimize.py:81-93): xphys = project(filter(x)), frozen elements set to 1;
   dxp = d project / d xt (NULL to skip). beta <= 0: no projection. */
int anl_physical(anl_ctx* ctx, const float* x, const uint8_t* frozen, double beta, double eta,
                 float* xphys, float* dxp, anl_stream_t stream);

/* ---------------------------------------------------------------- OC update */

/* Optimality-criteria bisection (optimize.py:144-161) on the active elements: lambda is
   bisected geometrically in [1e-8, 1e8] * scale (scale = mean(-dcx)/mean(dvx) over design
   elements), at most 100 steps, until hi/lo < 1 + 1e-9; the volume sum(phi * physical(xn))
   is accumulated in FP64. xnew receives the last evaluated xn (as the reference keeps it).
   steps_h / lambda_h (host, may be NULL) receive the step count and the last lambda. */
int anl_oc_update(anl_ctx* ctx, const float* x, const float* dcx, const float* dvx, const float* phi,
                  const uint8_t* frozen, double move, double beta, double eta, double vtarget,
                  float* xnew, int* steps_h, double* lambda_h, anl_stream_t stream);

/* Per-iteration history values (optimize.py:162-167), all over active elements:
   out_h[0] = max |xnew - xold| over design (non-frozen) elements (change)
   out_h[1] = fraction of design elements with 0.1 < xphys < 0.9 (grey)
   out_h[2] = sum phi * xphys (volume)
   out_h[3] = number of design elements */
int anl_design_stats(anl_ctx* ctx, const float* xold, const float* xnew, const float* xphys,
                     const float* phi, const uint8_t* frozen, double* out_h, anl_stream_t stream);

/* ---------------------------------------------------------------- allocation-free variant */

/* No counterpart in the reference. The compliance dot product of anl_dot (sum of a[i]*b[i],
   FP64, deterministic) for callers that cannot allocate device memory: a memory-pool hook or
   allocator callback, embedders whose framework owns the whole device pool, and loops that
   must not allocate (or synchronise) mid-step. It needs no context: a, b (n doubles) and out
   (one double) are caller-owned device buffers; the result is written to *out on `stream`.
   The reduction scratch is a fixed 33 KB array in the library's device memory, held by every
   GPU that loads the library until the process exits; n may be at most 268,435,456
   (ANL_ERR_BADARG beyond). Every call looks up that array's device address in the current
   context (cudaGetSymbolAddress, which loads the library's module on a device's first call),
   so make the first call on a device before any stream capture. Calls share the array:
   calls that overlap on the GPU (other streams, other threads) race. Allocates nothing,
   frees nothing. */
int anl_dot_static(const double* a, const double* b, int64_t n, double* out, anl_stream_t stream);

/* Replaces FEM.stress / FEM.von_mises (fem.py:244-263): element-centre stress sigma = E D B0 u_e
   (Voigt xx yy zz xy yz zx, engineering shear) and its von Mises value, FP64, on the full
   element grid (zeros on inactive elements). E_material: per element (double, full grid) or
   NULL to use E_scalar. sig (6 per element) or vm (1 per element) may be NULL. */
int anl_element_stress(anl_ctx* ctx, const double* u, const double* E_material, double E_scalar, double* sig,
                       double* vm, anl_stream_t stream);

/* ---------------------------------------------------------------- iso-surface export */

/* An export workspace: device buffers that grow to the largest field seen, the derived
   marching-cubes case table, and the last extracted mesh (float xyz vertices, int32 faces,
   outward-facing, indexed: one vertex per crossed grid edge). Not thread-safe. */
typedef struct anl_mc anl_mc;
int anl_mc_create(anl_mc** out);
void anl_mc_destroy(anl_mc* mc);

/* Replaces export.surface (export.py:121-131): np.pad(f, 1), ndimage.zoom(order=1) by
   `upsample`, measure.marching_cubes(level, spacing) and the shift origin - h/2.
   field: nx*ny*nz element densities on the device (x fastest, grid.to3d order). Writes the
   vertex and face counts (host). Samples (nx+2)(ny+2)(nz+2) upsample^3 must be <= 2^29. */
int anl_mc_extract(anl_mc* mc, const float* field, int nx, int ny, int nz, int upsample, double level, double h,
                   const double* origin_h, int64_t* nverts_h, int64_t* nfaces_h, anl_stream_t stream);

/* Replaces trimesh.smoothing.filter_taubin (export.py:134): `iterations` umbrella steps
   v += w (mean of neighbours - v), w = lamb on even steps and mu on odd ones (Taubin's
   lambda|mu filter; the reference passes lamb 0.5, nu -0.53). */
int anl_mc_smooth(anl_mc* mc, int iterations, double lamb, double mu, anl_stream_t stream);

/* Replaces mesh.split (export.py:135): the connected component of every face, as the smallest
   vertex index of the component (face_label: int32 per face, device). Writes the number of
   hook-and-jump rounds to *rounds_h when it is not NULL. */
int anl_mc_components(anl_mc* mc, int32_t* face_label, int* rounds_h, anl_stream_t stream);

/* Copies the current mesh out: verts 3*nverts floats, faces 3*nfaces int32 (device or
   pinned host pointers). */
int anl_mc_copy(anl_mc* mc, float* verts, int32_t* faces, anl_stream_t stream);

/* The derived case table (no counterpart in the reference, whose table lives in skimage):
   ntri_h[256] triangles per cube case (bit c set when corner c = (x, y, z bits) is above the
   level), tri_h[256*24] their cube edges (edge 4*axis + q, q the other two corner bits). */
int anl_mc_table(uint8_t* ntri_h, int8_t* tri_h);

/* ---------------------------------------------------------------- voxeliser */

/* A voxeliser workspace: device buffers that grow to the largest mesh and grid seen. Not
   thread-safe. */
typedef struct anl_vox anl_vox;
int anl_vox_create(anl_vox** out);
void anl_vox_destroy(anl_vox* vox);

/* Replaces geometry.voxel_fill (geometry.py:89-149): the fill fraction (0..1) of every element
   of the nx*ny*nz grid (spacing h, origin_h[3] on the host) inside the closed mesh tri
   (ntri triangles x 3 vertices x xyz, FP64, device), by ray parity along z at s^3 sample
   points per element (s in 1..16; the reference uses 3). fill: nx*ny*nz FP64 on the device,
   x fastest. Bit-identical to the reference. stats_h (host, may be NULL; then the call does not
   synchronise): [0] (triangle, sample column) pairs tested, [1] crossings counted.
   ANL_ERR_BADARG for an empty mesh (the reference raises ValueError there). */
int anl_voxel_fill(anl_vox* vox, const double* tri, int64_t ntri, int nx, int ny, int nz, double h,
                   const double* origin_h, int s, double* fill, int64_t* stats_h, anl_stream_t stream);

/* ---------------------------------------------------------------- from design to surface */

/* Replaces export.output_field (export.py:8-14): f = min(max(x fill, active ? solid_fill : 0),
   1 - void_fill), then max(f, fill) on frozen elements. All arrays n elements on the device
   (active, frozen: uint8 0/1). Bit-identical to the reference. */
int anl_output_field(const double* x, const double* fill, const uint8_t* active, const double* solid_fill,
                     const double* void_fill, const uint8_t* frozen, int64_t n, double* f, anl_stream_t stream);

/* Replaces the bisection of export.choose_level (export.py:17-28): `steps` halvings of [lo, hi]
   keeping count(f > t) > target on the low side, t = (lo + hi) / 2. f: n FP64 values on the
   device. Eight steps per read of f. state: 2 doubles, hist: 256 uint64 of device scratch.
   Writes the final [lo, hi] to lo_hi_h (host) and synchronises the stream; the reference's
   level is clip((lo + hi) / 2, 0.3, 0.7). */
int anl_choose_level(const double* f, int64_t n, double target, double lo, double hi, int steps, double* state,
                     unsigned long long* hist, double* lo_hi_h, anl_stream_t stream);

/* The connected components of {f > thr} on the nx*ny*nz grid (6-connectivity: the structure
   ndimage.label uses in keep_load_paths, export.py:43-47). labels (int32, device): the
   smallest element index of the element's component, -1 where f <= thr. n < 2^31. */
int anl_label_above(const double* f, int nx, int ny, int nz, double thr, int32_t* labels, anl_stream_t stream);

/* Exact Euclidean distance transform (ndimage.distance_transform_edt, as member_thickness uses
   it, export.py:150-158): for every element the distance to the nearest element with
   solid == 0 (unit spacing), FP64, on an nx*ny*nz grid (x fastest, each side <= 4096); pad the
   grid with a background layer for the reference's np.pad. scratch: device memory of at least
   align16(4 n) + 16 n + 8 max(ny nz, nx nz, nx ny) bytes. Elements with no background on the
   grid get 1e10 (the square root of the internal infinity). */
int anl_edt(const uint8_t* solid, int nx, int ny, int nz, double* dist, void* scratch, size_t scratch_bytes,
            anl_stream_t stream);

/* ---------------------------------------------------------------- warm-start network layers

   No counterpart in the reference: the reference starts each solve from the previous
   iterate (optimize.py:122); these kernels train and run the network that predicts a better
   start. Tensors are one sample, [C][D][H][W] float with W fastest; weights [cout][cin][k^3]. */

/* z = conv3d(x, w) + b (k = 1 or 3, zero padding k/2, stride 1; b may be NULL); a = GELU(z)
   when act != 0. accumulate != 0 adds to z instead of overwriting it. */
int anl_nn_conv3d(const float* x, const float* w, const float* b, float* z, float* a, int cin, int cout, int D,
                  int H, int W, int ksize, int act, int accumulate, anl_stream_t stream);
/* dx = conv3d^T(dz, w) (the gradient with respect to x); wt_work holds cin*cout*k^3 floats. */
int anl_nn_conv3d_bwd_data(const float* dz, const float* w, float* wt_work, float* dx, int cin, int cout, int D,
                           int H, int W, int ksize, int accumulate, anl_stream_t stream);
/* dw, db (gradients with respect to w and b), summed over voxel chunks in a fixed order;
   part_work holds part_floats >= cout*cin*k^3 + cout floats (more allows more chunks). */
int anl_nn_conv3d_bwd_weight(const float* x, const float* dz, float* part_work, int64_t part_floats, float* dw,
                             float* db, int cin, int cout, int D, int H, int W, int ksize, int accumulate,
                             anl_stream_t stream);
/* dz = da * GELU'(z) (erf form). */
int anl_nn_gelu_bwd(const float* z, const float* da, float* dz, int64_t n, anl_stream_t stream);
/* 2x average pooling of C channels of an even D x H x W grid; backward = 1 maps the pooled
   gradient x to the full-size gradient y (added to y when accumulate != 0). */
int anl_nn_pool2(const float* x, float* y, int C, int D, int H, int W, int backward, int accumulate,
                 anl_stream_t stream);
/* 2x nearest upsampling to an even D x H x W grid; backward = 1 sums the full-size gradient x
   into the half-size gradient y. */
int anl_nn_up2(const float* x, float* y, int C, int D, int H, int W, int backward, anl_stream_t stream);
/* Masked mean-squared error over C channels sharing a per-voxel mask: out2[0] = sum m (y-t)^2,
   out2[1] = sum m (device), dy = 2 m (y - t) / max(1, sum m). work: 2*1216 doubles; counter:
   a zeroed unsigned (left zero). */
int anl_nn_mse(const float* y, const float* tgt, const float* mask, float* dy, int C, int64_t vol, double* work,
               unsigned* counter, double* out2, anl_stream_t stream);
/* One Adam step (bias-corrected, step >= 1) on n FP32 parameters. */
int anl_nn_adam(float* p, const float* g, float* m, float* v, int64_t n, double lr, double b1, double b2, double eps,
                int step, anl_stream_t stream);

/* ---------------------------------------------------------------- measurement */

/* Multigrid hierarchy of the context (no counterpart in the reference): *nlev_h levels,
   dims_h[3*l..3*l+2] the element dims of level l, lmax_h[l] the estimated largest
   eigenvalue of D^-1 K used by its Chebyshev smoother (arrays of 16 entries). */
int anl_mg_info(anl_ctx* ctx, int* nlev_h, int* dims_h, double* lmax_h);

/* Number of kernels this library has launched in the process so far (no counterpart in
   the reference; lets a benchmark count the GPU launches inside its timed region). */
int64_t anl_launch_count(void);

/* Debug build only (no counterpart in the reference; the library built with -DANL_DEBUG=1):
   the number of global-memory accesses the kernels' bounds checks caught and skipped since
   the last call, and first_h[0..2] = index, extent and source line of the first; both
   records are cleared. Synchronises the device. The normal build sets *count_h = -1. */
int anl_debug_oob(long long* count_h, long long* first_h);

/* Benchmark hook (no counterpart in the reference): launches the level-0 K u kernel
   `reps` times on `stream` between two CUDA events and writes the mean time per launch in
   milliseconds to *ms_h. The element scales are those of the last anl_apply_K / anl_solve
   on this context; u must be zero on non-free DOFs (context precision). */
int anl_profile_apply(anl_ctx* ctx, const void* u, void* y, int reps, double* ms_h, anl_stream_t stream);

/* Benchmark hook (no counterpart in the reference): times one finest-level pass of the solve,
   `reps` launches between two CUDA events on `stream`, on the context's own work vectors:
   pass 0 K u, 1 K u with the u.Ku reduction (the CG's q = K p), 2 the residual b - K x, 3 the
   last Chebyshev step of a smoothing sweep, 4 the first two Chebyshev steps fused, 5 the first step of a
   sweep that starts from a nonzero iterate (the post-smoothing after the prolongation). The mean
   milliseconds per launch go to *ms_h. FP32 contexts, after at least one anl_solve; it overwrites the V-cycle
   scratch (the next solve starts afresh), so do not call it during a stream capture. */
int anl_profile_pass(anl_ctx* ctx, int pass, int reps, double* ms_h, anl_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* ANNEAL_GB300_H */
