/*
 * omega2d_gb300.h -- C ABI of the GB300 direct Biot-Savart engine (libomega2d_gb300.so).
 *
 * Drop-in for the O(N^2) influence path of Omega2D.  Every entry point names the reference
 * function it replaces (paths are relative to the Omega2D source tree).  Conventions:
 *
 *   - Arrays are structure-of-arrays, FP32 unless the name says otherwise, caller-owned.
 *     "Host" entry points take host pointers, copy in/out and synchronize before returning;
 *     "_dev" entry points take device pointers and run asynchronously on the context's stream.
 *   - Influence sums are UNSCALED and ACCUMULATED (out += sum), like the reference drivers
 *     (src/Influence.h:207-208, 359-360).  OBS_FLAG_FINALIZE additionally applies the
 *     reference's finalize step, out = fs + out/(2 pi) (src/ElementBase.h:215-234).
 *   - Every call returns an int status: OBS_OK (0) or a negative OBS_ERR_* code.  Nothing
 *     aborts the host process; a failed call leaves the caller's outputs unspecified only for
 *     _dev calls (host calls leave them untouched).
 *   - A context is thread-compatible, not re-entrant: one host thread at a time.
 */
#ifndef OMEGA2D_GB300_H
#define OMEGA2D_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes */
#define OBS_OK 0
#define OBS_ERR_ARG (-1)        /* invalid argument (null pointer, negative size, bad enum)  */
#define OBS_ERR_ALLOC (-2)      /* device or host allocation failed                         */
#define OBS_ERR_CUDA (-3)       /* a CUDA runtime call failed                                */
#define OBS_ERR_TIMEOUT (-4)    /* a bounded device-side wait gave up                        */
#define OBS_ERR_NO_DEVICE (-5)  /* no usable CUDA device                                     */
#define OBS_ERR_SINGULAR (-6)   /* dense solve met a zero pivot                              */
#define OBS_ERR_UNSUPPORTED (-7)
#define OBS_ERR_SCRATCH_LIMIT (-8)  /* size exceeds obs_points_affect_points_noalloc's scratch */
#define OBS_ERR_NO_CONVERGENCE (-9) /* an iterative solve stopped above its tolerance           */

/* ---- core functions (src/CoreFunc.h:35-322 selects one at compile time; here at run time) */
#define OBS_CORE_RM 1           /* Rosenhead-Moore, src/CoreFunc.h:42-82                     */
#define OBS_CORE_GAUSSIAN 2     /* "exponential" = Gaussian blob, src/CoreFunc.h:85-181      */
#define OBS_CORE_V2 3           /* Vatistas n=2 (the reference default), :233-275            */
#define OBS_CORE_WL 4           /* Winckelmans-Leonard, :184-230                              */
#define OBS_CORE_V3 5           /* Vatistas n=3, :278-322                                     */
#define OBS_CORE_SINGULAR 6     /* point vortex 1/d^2 (RM with zero radii), self pair = 0   */
#define OBS_CORE_COMPACT_EXP 7  /* (1 - exp(-(d/s)^3))/d^2; not in the reference            */

/* ---- result types: same values as results_t (src/ResultsType.h:26-32) */
#define OBS_VELONLY 1
#define OBS_VELANDGRAD 2        /* extra0..3 = du/dx, dv/dx, du/dy, dv/dy                    */
#define OBS_PSIONLY 3           /* extra0 = streamfunction; velocity untouched               */
#define OBS_VELANDVORT 4        /* extra0 = vorticity                                         */
#define OBS_VELANDSHEAR 5       /* extra0 = shear rate                                        */

/* ---- accumulation modes */
#define OBS_PLAIN_F32 0         /* FP32 accumulators: the plain drop-in                      */
#define OBS_COMPENSATED 1       /* FP32 pair math, two-sum per 32-source block, FP64 reduce  */

/* ---- flags */
#define OBS_FLAG_FINALIZE 1     /* out = fs + (out + sum)/(2 pi); extras *= 1/(2 pi)          */

typedef struct obs_context obs_context;

/* Context: CUDA device binding, one stream, device work buffers that grow on demand. */
int obs_create(obs_context** ctx, int device);
int obs_destroy(obs_context* ctx);
/* Run subsequent work on an external cudaStream_t (passed as void*; NULL is the legacy default
 * stream).  obs_use_own_stream switches back to the context's own non-blocking stream. */
int obs_set_stream(obs_context* ctx, void* cuda_stream);
int obs_use_own_stream(obs_context* ctx);
int obs_synchronize(obs_context* ctx);
/* Enable CUDA-event timing of the main kernel of each subsequent call (default off). */
int obs_enable_timing(obs_context* ctx, int on);
/* Main-kernel and whole-call device time of the most recent timed call, in milliseconds. */
int obs_last_timing(obs_context* ctx, float* main_kernel_ms, float* call_ms);
/* Device-side failure record seen by the last synchronizing call that reported one: DEV_ERR
 * bits (1 = bounded wait timed out, 4 = bounds check), the check code, and two values. */
int obs_last_failure(obs_context* ctx, int* bits, int* code, int* v1, int* v2);
/* Failure-path self-test: runs, on the context's stream, a bounded wait that nothing
 * completes -- which 0: an mbarrier phase with no arrival (the wait of the tile pipelines),
 * which 1: a grid barrier expecting one block more than the grid (the fused GMRES cycle) --
 * which gives up after max_polls polls, records its location (codes 901 / 700) and returns.
 * Returns the status the next synchronizing call reads: OBS_ERR_TIMEOUT when the wait gave up
 * as designed; the context stays usable. */
int obs_selftest_bounded_wait(obs_context* ctx, int which, int max_polls);
/* Kernel variant for particle-on-particle sums.  AUTO uses the packed-FP32 kernels (two
 * targets per f32x2 register pair) where they exist -- velocity for every core, with 4 target
 * pairs per thread (2 for Vatistas n=3, the singular core and sums with fewer than 49,152
 * targets, 98,304 for the compact exponential); velocity gradient, vorticity
 * and shear for the Gaussian core -- and the generic kernels elsewhere.  GENERIC forces the
 * generic kernels (and the one-kernel-per-step GMRES); PACKED2 / PACKED3 / PACKED4 pick 2, 3
 * (Gaussian only; 2 for the other cores) or 4 target pairs per thread for the packed velocity
 * kernels. */
#define OBS_VARIANT_AUTO 0
#define OBS_VARIANT_GENERIC 1
#define OBS_VARIANT_PACKED2 2
#define OBS_VARIANT_PACKED3 3
#define OBS_VARIANT_PACKED4 4
int obs_set_kernel_variant(obs_context* ctx, int variant);
/* Processing order inside a packed Gaussian or compact-exponential velocity sum.  Binning
 * sorts points into a 256 x 256 Morton-ordered grid over their bounding box (a stable sort), so
 * that each warp's targets and each block of 32 sources lie close together; (warp, block) pairs
 * beyond the core's far radius (4 core radii for the Gaussian, 16^(1/3) for the compact
 * exponential) then take the reference's far-field form G/d^2 without the exponential.
 * Results are always written in the caller's order.
 *   INPUT          : caller's order for targets and sources;
 *   BINNED_TARGETS : binned targets; results are bit-identical to INPUT;
 *   BINNED         : binned targets and sources; sources are summed in the binned order, so
 *                    results differ from INPUT by rounding only (and are reproducible);
 *   AUTO           : BINNED when the sum has at least 3e8 pairs and 4096 targets and sources,
 *                    else INPUT. */
#define OBS_ORDER_AUTO 0
#define OBS_ORDER_INPUT 1
#define OBS_ORDER_BINNED 2
#define OBS_ORDER_BINNED_TARGETS 3
int obs_set_target_order(obs_context* ctx, int order);
/* The spatial order used above, as a utility on device arrays: perm[k] (device, n ints) is the
 * index of the k-th point after a stable sort by the Morton key of its cell in a 256 x 256 grid
 * over the points' bounding box (cell = min(255, floor((v - min) * (256 / (max - min))))).
 * Asynchronous on the context's stream. */
int obs_morton_order_dev(obs_context* ctx, int n, const float* x, const float* y, int* perm);
/* Number of engine kernel launches issued by this context since creation. */
long long obs_launch_count(obs_context* ctx);
const char* obs_status_string(int status);
/* Algorithmic flops per interaction the reference attaches to a kernel (src/Kernels.h flops*,
 * src/CoreFunc.h flops_*), or -1 when the reference has none for that combination. */
int obs_flops_per_pair(int core, int result, int thick_targets);

/*
 * points_affect_points -- replaces src/Influence.h:56-416 (x86 and Vc branches).
 * Sources: ns particles (sx, sy, sr = core radius, ss = circulation).
 * Targets: nt points; tr == NULL selects field points (the "0p" kernels, src/Influence.h:114-250),
 *          otherwise thick targets with core radius tr (the "0b" kernels, :255-406).
 * Outputs: tu, tv (+ extra0..3 per result type) accumulated; flops (optional) receives the
 *          reference's flop count for the call (src/Influence.h:362 convention).
 */
int obs_points_affect_points(obs_context* ctx, int core, int result, int accum, int flags,
                             double fsx, double fsy,
                             int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                             int nt, const float* tx, const float* ty, const float* tr,
                             float* tu, float* tv,
                             float* extra0, float* extra1, float* extra2, float* extra3,
                             double* flops);
int obs_points_affect_points_dev(obs_context* ctx, int core, int result, int accum, int flags,
                                 double fsx, double fsy,
                                 int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                                 int nt, const float* tx, const float* ty, const float* tr,
                                 float* tu, float* tv,
                                 float* extra0, float* extra1, float* extra2, float* extra3,
                                 double* flops);

/* points_affect_points_vorticity -- replaces src/InfluenceVort.h:47-126 (the non-Vc branch):
 * Gaussian-blob vorticity at field points, tw += sum 2 G exp(-d^2/s^2) / s^2 with s the source
 * core radius (no cut-off, as in that branch).  OBS_FLAG_FINALIZE scales tw by 1/(2 pi) like
 * finalize_vels does (src/ElementBase.h:215-234). */
int obs_points_affect_points_vorticity(obs_context* ctx, int accum, int flags,
                                       int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                                       int nt, const float* tx, const float* ty, float* tw);
int obs_points_affect_points_vorticity_dev(obs_context* ctx, int accum, int flags,
                                           int ns, const float* sx, const float* sy, const float* sr,
                                           const float* ss, int nt, const float* tx, const float* ty, float* tw);

/*
 * Panels: straight constant-strength panels given as node coordinates (nx, ny; nnodes) and
 * node-index pairs (idx[2*k], idx[2*k+1]) for panel k, like Surfaces (src/Surfaces.h:682-724).
 * The fluid lies to the left walking node0 -> node1.
 *
 * panels_affect_points -- replaces src/Influence.h:422-614: velocity at points due to panels
 * with vortex sheet strength vs and source sheet strength ss (kernelu_1vs_0p,
 * src/Kernels.h:362-405); ss == NULL gives the vortex-only kernelu_1v_0p (:311-354).
 * Accumulates (unscaled) into tu, tv.
 */
int obs_panels_affect_points(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                             int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                             const float* vs, const float* ss,
                             int nt, const float* tx, const float* ty, float* tu, float* tv);
int obs_panels_affect_points_dev(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                                 int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                                 const float* vs, const float* ss,
                                 int nt, const float* tx, const float* ty, float* tu, float* tv);

/* panels_affect_panels -- replaces src/Influence.h:774-795: velocities at the target panels'
 * centres due to the source panels, through the reference's collocation points
 * (Surfaces::represent_as_particles(1e-4, -1), src/Surfaces.h:830-876: 1 + (int)(len_i /
 * (1.2 len_0)) points per panel, 1e-4 off the panel into the fluid; the first tnp point
 * velocities are added to the tnp panels, index by index, as the reference does).
 * Accumulates (unscaled) into pu, pv. */
int obs_panels_affect_panels(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                             int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                             const float* vs, const float* ss,
                             int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                             float* pu, float* pv);
int obs_panels_affect_panels_dev(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                                 int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                                 const float* vs, const float* ss,
                                 int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                                 float* pu, float* pv);

/* points_affect_panels -- replaces src/Influence.h:633-771: mean velocity over each panel due
 * to point vortices of strength ss (the particle core is not used, as in the reference),
 * accumulated into the panel-centre velocities pu, pv. */
/* Reverse mode of obs_panels_affect_points with respect to the panel strengths (no counterpart
 * in the reference): for cotangents (lu, lv) of the finalized velocities at the nt points
 * (tx, ty) -- L depends on u = fs + (panel sum)/(2 pi) -- accumulates gvs[p] += dL/d(vortex
 * strength p) and, when gss is not null, gss[p] += dL/d(source strength p).  Both panel
 * strength sets enter the forward sum linearly, so these are exact gradients. */
int obs_panels_affect_points_vjp(obs_context* ctx, int accum, int nnodes, const float* nx, const float* ny,
                                 int npan, const unsigned* idx, int nt, const float* tx, const float* ty,
                                 const float* lu, const float* lv, float* gvs, float* gss);
int obs_panels_affect_points_vjp_dev(obs_context* ctx, int accum, int nnodes, const float* nx, const float* ny,
                                     int npan, const unsigned* idx, int nt, const float* tx, const float* ty,
                                     const float* lu, const float* lv, float* gvs, float* gss);
int obs_points_affect_panels(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                             int ns, const float* sx, const float* sy, const float* ss,
                             int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                             float* pu, float* pv);
int obs_points_affect_panels_dev(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                                 int ns, const float* sx, const float* sy, const float* ss,
                                 int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                                 float* pu, float* pv);

/* panels_on_panels_coeff -- replaces src/Coefficients.h:155-427 (the non-augmented part):
 * column-major (nunk*ntarg) x (nunk*nsrc) block, targets are rows, scaled by 1/(2 pi);
 * nunk = 2 is the reference's vortex+source system (src/Surfaces.h:69), nunk = 1 vortex only;
 * self_block != 0 when source and target are the same body (diagonal pi/(2 pi)).
 * Either output may be NULL (FP32 as in the reference, or FP64 for the dense solve). */
int obs_panels_on_panels_coeff(obs_context* ctx, int nunk, int self_block,
                               int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                               int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                               float* A32, double* A64);
int obs_panels_on_panels_coeff_dev(obs_context* ctx, int nunk, int self_block,
                                   int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                                   int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                                   float* A32, double* A64);

/* vels_to_rhs_panels -- replaces src/RHS.h:54-115: rhs = -u.t (and -u.n + bcn). */
int obs_vels_to_rhs_panels(obs_context* ctx, int nunk, int nnodes, const float* nx, const float* ny, int npan,
                           const unsigned* idx, const float* pu, const float* pv, const float* bcn,
                           float* rhs32, double* rhs64);
int obs_vels_to_rhs_panels_dev(obs_context* ctx, int nunk, int nnodes, const float* nx, const float* ny, int npan,
                               const unsigned* idx, const float* pu, const float* pv, const float* bcn,
                               float* rhs32, double* rhs64);

/* FP64 dense solve A x = b (A column-major n x n) on the GPU by LU with partial pivoting; the
 * reference uses Eigen GMRES in FP32 on the host (src/BEM.h:169-234).  rel_residual (optional)
 * receives ||A x - b|| / ||b|| like the reference's check (src/BEM.h:223-233). */
int obs_solve_dense_f64(obs_context* ctx, int n, const double* A, const double* b, double* x,
                        double* rel_residual);
int obs_solve_dense_f64_dev(obs_context* ctx, int n, const double* A, const double* b, double* x,
                            double* rel_residual);

/* Restarted GMRES in FP64 on the GPU (the reference's BEM solver method, Eigen GMRES in FP32,
 * src/BEM.h:169-234): right diagonal preconditioning, classical Gram-Schmidt with one
 * reorthogonalisation, Givens rotations on the device; for restart <= 64 each restart cycle is
 * one cooperative launch with grid barriers.  x holds the initial guess on entry and
 * the solution on return; iterations and rel_residual = ||b - A x|| / ||b|| are optional
 * outputs.  OBS_ERR_NO_CONVERGENCE when maxiter iterations end above tol (x then holds the
 * last iterate). */
int obs_solve_gmres_f64(obs_context* ctx, int n, const double* A, const double* b, double* x, double tol,
                        int restart, int maxiter, int* iterations, double* rel_residual);
int obs_solve_gmres_f64_dev(obs_context* ctx, int n, const double* A, const double* b, double* x, double tol,
                            int restart, int maxiter, int* iterations, double* rel_residual);

/* solve_bem for one fixed reactive body -- replaces src/BEMHelper.h:43-260 without rotation
 * augmentation: particles -> panel velocities, finalize with fs, RHS, influence matrix, FP64
 * solve, strengths out (vs_out; ss_out when nunk == 2).  The solve is FP64 GMRES (restart 60,
 * relative residual 1e-13, at most 2n iterations, zero initial guess); OBS_BEM_DIRECT_LU selects
 * the FP64 LU instead.  OBS_BEM_REUSE_MATRIX keeps the previous matrix (and factorisation) of
 * the same order (the reference's is_A_current, src/BEM.h:49-51). */
#define OBS_BEM_REUSE_MATRIX 2
#define OBS_BEM_DIRECT_LU 4      /* solve by the FP64 LU instead of FP64 GMRES */
int obs_solve_bem(obs_context* ctx, int nunk, int accum, int flags, double fsx, double fsy,
                  int ns, const float* sx, const float* sy, const float* ss,
                  int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx, const float* bcn,
                  float* vs_out, float* ss_out, double* rel_residual);

/* clear_inner_layer -- replaces src/Reflect.h:733-760 (clear_inner_panp2, :491-729) for one body
 * and one point set.  The height of a point above the layer at cutoff_mult * ips is measured
 * along the mean normal of its closest panels or nodes; method 0 (particles only) crops a point
 * lower than its core radius (strength scaled, point shifted outward by the reference's cut
 * tables), method 1 pushes a point below the layer onto it.  x, y (and s, method 0) are updated in place;
 * r holds the points' core radii (NULL: field points, whose radius is ips).  circ_removed
 * (optional) receives the circulation removed (the body's add_to_reabsorbed), ncropped the
 * number of modifications.  OBS_ERR_NO_CONVERGENCE when a point was still being modified
 * after 64 tests (the others are cleared).  The _dev form takes device arrays and, unlike the
 * other _dev calls, synchronizes the context's stream: its two results are host values. */
int obs_clear_inner_layer(obs_context* ctx, int method, float cutoff_mult, float ips, int nnodes, const float* nx,
                          const float* ny, int npan, const unsigned* idx, int n, float* x, float* y, float* s,
                          const float* r, double* circ_removed, long long* ncropped);
int obs_clear_inner_layer_dev(obs_context* ctx, int method, float cutoff_mult, float ips, int nnodes,
                              const float* nx, const float* ny, int npan, const unsigned* idx, int n, float* x,
                              float* y, float* s, const float* r, double* circ_removed, long long* ncropped);

/* Rotation augmentation (src/Coefficients.h:429-572, src/BEMHelper.h:114-135, 197-205): the self
 * block of one body gains a bottom row of panel lengths (under the vortex unknowns), a right
 * column of the unit-rotation velocity along each panel (Surfaces::add_unit_rot_strengths about
 * the body's centroid, their panels_affect_panels velocity, finalized) and the corner 2 * area
 * (Surfaces::set_geom_center).  obs_panels_on_panels_coeff_augmented returns that
 * (nunk*npan+1)^2 column-major block in FP64 and geom = (area, centroid x, centroid y);
 * obs_solve_bem_augmented solves it with circ_rhs as the extra right-hand side (the
 * reference's self + re-absorbed circulation + previous error) and returns the body's rotation
 * rate in omega_out. */
int obs_panels_on_panels_coeff_augmented(obs_context* ctx, int nunk, int accum, int nnodes, const float* nx,
                                         const float* ny, int npan, const unsigned* idx, double* A64,
                                         double* geom);
int obs_solve_bem_augmented(obs_context* ctx, int nunk, int accum, int flags, double fsx, double fsy,
                            int ns, const float* sx, const float* sy, const float* ss,
                            int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                            const float* bcn, double circ_rhs, float* vs_out, float* ss_out, double* omega_out,
                            double* rel_residual);

/* Several bodies in one BEM system (src/BEMHelper.h:147-221 assembles it block by block;
 * src/Coefficients.h:429-572 augments each rotating body): the bodies' nodes and panels are
 * joined in one set (node indices global, body k owns panels [panel_off[k], panel_off[k+1])),
 * the panel unknowns come first in panel order, then one rotation unknown per body with
 * augmented[k] != 0, in body order.  Rotating body a adds a row (its panel lengths under its
 * vortex unknowns, 0 under every other panel, 2 * its area on the diagonal, 0 under the other
 * rotation unknowns) and a column (the velocity of its unit-rotation sheet at every panel of the
 * set, finalized, along each panel's tangent and normal).  The reference orders each body's
 * rotation unknown after that body's panels; this is the same system with its rows and
 * columns permuted.  obs_panels_on_panels_coeff_bodies returns the FP64 matrix (column-major)
 * and geom = (area, centroid x, centroid y) per body; obs_solve_bem_bodies solves it with
 * circ_rhs[k] as body k's rotation right-hand side and writes its rotation rate to
 * omega_out[k] (augmented bodies only).  At most 64 rotating bodies (OBS_ERR_UNSUPPORTED). */
int obs_panels_on_panels_coeff_bodies(obs_context* ctx, int nunk, int accum, int nnodes, const float* nx,
                                      const float* ny, int npan, const unsigned* idx, int nbodies,
                                      const int* panel_off, const int* augmented, double* A64, double* geom);
int obs_solve_bem_bodies(obs_context* ctx, int nunk, int accum, int flags, double fsx, double fsy,
                         int ns, const float* sx, const float* sy, const float* ss,
                         int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                         const float* bcn, int nbodies, const int* panel_off, const int* augmented,
                         const double* circ_rhs, float* vs_out, float* ss_out, double* omega_out,
                         double* rel_residual);

/*
 * Reverse mode (no counterpart in the reference, which has no adjoint).  Cotangents lu, lv are
 * on the FINALIZED velocities u = fs + (1/2 pi) sum (OBS_FLAG_FINALIZE); gradient outputs are
 * ACCUMULATED (+=); any output pointer may be NULL.
 *
 * obs_points_affect_points_vjp: backward of points_affect_points for a separate target set
 * (field points when tr == NULL, thick targets otherwise): dL/d(source x, y, strength) by a
 * source-outer gather over the targets, and dL/d(target x, y) = (1/2 pi) (grad u)^T lam from
 * the velocity-gradient kernel.
 */
int obs_points_affect_points_vjp(obs_context* ctx, int core, int accum,
                                 int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                                 int nt, const float* tx, const float* ty, const float* tr,
                                 const float* lu, const float* lv,
                                 float* gsx, float* gsy, float* gss, float* gtx, float* gty);
int obs_points_affect_points_vjp_dev(obs_context* ctx, int core, int accum,
                                     int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                                     int nt, const float* tx, const float* ty, const float* tr,
                                     const float* lu, const float* lv,
                                     float* gsx, float* gsy, float* gss, float* gtx, float* gty);

/* Backward of the self-interaction (targets are the particles, thick cores): one fused gather
 * per particle gives dL/dx, dL/dy (both source and target roles) and dL/ds. */
int obs_points_affect_points_vjp_self(obs_context* ctx, int core, int accum, int n, const float* x, const float* y,
                                      const float* r, const float* s, const float* lu, const float* lv,
                                      float* gx, float* gy, float* gs);
int obs_points_affect_points_vjp_self_dev(obs_context* ctx, int core, int accum, int n, const float* x,
                                          const float* y, const float* r, const float* s, const float* lu,
                                          const float* lv, float* gx, float* gy, float* gs);

/* Forward op: nsteps of convection of the particles by their own velocity plus freestream, in
 * place, without bodies -- Convection::advect_1st (order 1), advect_2nd_ralston (order 2, the
 * reference's second order), advect_3rd (order 3) and advect_2nd_heun (order 4)
 * (src/Convection.h:274-598). */
#define OBS_ADVECT_EULER 1
#define OBS_ADVECT_RK2_RALSTON 2
#define OBS_ADVECT_RK3 3
#define OBS_ADVECT_RK2_HEUN 4
int obs_advect(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y, const float* r,
               const float* s, double fsx, double fsy, double dt, int nsteps);
int obs_advect_dev(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y, const float* r,
                   const float* s, double fsx, double fsy, double dt, int nsteps);

/* Backward op of obs_advect from the initial positions (x0, y0): given dL/d(final x, y) in
 * (lx, ly), accumulate dL/ds into gs and dL/d(initial x, y) into gx0, gy0.  The trajectory is
 * recomputed per segment from checkpoints every checkpoint_every steps (0: ceil(sqrt(nsteps))).
 * peak_bytes (optional) receives the engine's device-memory footprint (all its buffers). */
/* Forward op that also records the checkpoints (every checkpoint_every steps; 0: ceil(sqrt
 * (nsteps))) and copies of r and s in the context, so that obs_advect_vjp_tape_dev can run the
 * backward without repeating the forward sweep.  One recording per context; the next
 * recording (or obs_advect_vjp) replaces it.
 * checkpoint_every = OBS_TAPE_ALL keeps every step's positions and stage positions on the
 * device (nsteps * stages * 2n floats; RK2: 2 GB for 2M particles over 64 steps): the backward
 * then evaluates no velocity sum, only the VJP gathers.  Gradients are bit-identical to the
 * checkpointed ones. */
#define OBS_TAPE_ALL (-1)
int obs_advect_record_dev(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y,
                          const float* r, const float* s, double fsx, double fsy, double dt, int nsteps,
                          int checkpoint_every);
/* Backward op of the recorded forward: dL/d(final x, y) in (lx, ly); accumulates dL/ds into gs
 * and dL/d(initial x, y) into gx0, gy0 (device arrays; any output may be NULL).  Returns
 * OBS_ERR_ARG when nothing is recorded. */
int obs_advect_vjp_tape_dev(obs_context* ctx, const float* lx, const float* ly, float* gs, float* gx0, float* gy0,
                            long long* peak_bytes);
int obs_advect_vjp(obs_context* ctx, int core, int accum, int order, int n, const float* x0, const float* y0,
                   const float* r, const float* s, double fsx, double fsy, double dt, int nsteps,
                   int checkpoint_every, const float* lx, const float* ly, float* gs, float* gx0, float* gy0,
                   long long* peak_bytes);
int obs_advect_vjp_dev(obs_context* ctx, int core, int accum, int order, int n, const float* x0, const float* y0,
                       const float* r, const float* s, double fsx, double fsy, double dt, int nsteps,
                       int checkpoint_every, const float* lx, const float* ly, float* gs, float* gx0, float* gy0,
                       long long* peak_bytes);

/*
 * points_affect_points for callers that cannot allocate device memory.  No counterpart in the
 * reference.  It is meant for code whose host framework owns every device allocation (pool
 * allocators, memory budgets), for FFI callers that only hand over finished device buffers,
 * and for callers that must avoid the implicit synchronization an allocation can cause.  It
 * calls no cudaMalloc, cudaFree or allocating library routine: its scratch is one fixed
 * device array of 16 MiB + 256 B in the library, reserved on every GPU that loads the
 * library until the process exits.
 *   - Arguments and results as obs_points_affect_points_dev (device pointers, accumulate),
 *     on the given cudaStream_t (NULL = legacy default stream); returns after that stream has
 *     finished the call, so device-side failures are reported by this call's status.
 *   - At most OBS_NOALLOC_MAX_SOURCES sources; more returns OBS_ERR_SCRATCH_LIMIT.  Targets are
 *     unlimited (fewer source splits are used when the partial sums would not fit).
 *   - The first call on each device looks up the scratch's device address (once per device,
 *     with that device current).
 *   - Every call ends by synchronizing its stream, so it cannot be recorded into a CUDA graph:
 *     called while its stream is being captured it does nothing and returns
 *     OBS_ERR_UNSUPPORTED.
 *   - Every call shares the one scratch array: calls that overlap on the GPU (other streams,
 *     other host threads) race and corrupt each other's results.
 */
#define OBS_NOALLOC_MAX_SOURCES 262144
int obs_points_affect_points_noalloc(void* cuda_stream, int core, int result, int accum, int flags,
                                     double fsx, double fsy,
                                     int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                                     int nt, const float* tx, const float* ty, const float* tr,
                                     float* tu, float* tv,
                                     float* extra0, float* extra1, float* extra2, float* extra3);

/*
 * points_affect_points by treecode -- the reference's Barnes-Hut summation slot
 * (summation_t barneshut, src/ExecEnv.h:26-31), which the reference itself reaches only through
 * the external solver hook (onbody's treecode, src/Influence.h:31-38, 74-98).  Velocity only
 * (results_t velonly), every core, thick (tr) or field-point (tr == NULL) targets; outputs
 * accumulated like obs_points_affect_points (OBS_FLAG_FINALIZE applies finalize_vels).
 * Sources in Morton order form a tree of 32-source leaves and 4-way nodes carrying `order`
 * multipole coefficients; a node acts on a warp of 32 targets through its expansion when its
 * radius is at most theta times the distance from its centre to the targets' box and every
 * pair lies where the core equals 1/d^2 (exactly for the Gaussian and compact exponential cut-
 * offs and the singular core; within 2^-24 for the others), else it opens, down to direct
 * sums over leaves with the core.  Truncation per node is below theta^order/(1 - theta) of
 * its summed |strength|/distance.  theta in (0, 1) (0 selects the default), order 1..32 (0:
 * default).  Compensated accumulation; flops (optional) receives the direct-sum count of the
 * same call.  _dev: device arrays, asynchronous on the context's stream.
 */
#define OBS_TREE_THETA_DEFAULT 0.5
#define OBS_TREE_ORDER_DEFAULT 24
#define OBS_TREE_ORDER_MAX 32
int obs_points_affect_points_tree(obs_context* ctx, int core, int flags, double fsx, double fsy, double theta,
                                  int order, int ns, const float* sx, const float* sy, const float* sr,
                                  const float* ss, int nt, const float* tx, const float* ty, const float* tr,
                                  float* tu, float* tv, double* flops);
int obs_points_affect_points_tree_dev(obs_context* ctx, int core, int flags, double fsx, double fsy, double theta,
                                      int order, int ns, const float* sx, const float* sy, const float* sr,
                                      const float* ss, int nt, const float* tx, const float* ty, const float* tr,
                                      float* tu, float* tv, double* flops);

/*
 * Source-compatible replacements for the reference's external direct-solver hook
 * (src/Influence.h:31-38, called at :74-98 when built with -DEXTERNAL_VEL_SOLVE).
 * Same argument order (note ss before sr), counts by pointer, velocities ACCUMULATED and
 * unscaled; the return value is the flop count, or a negative value on error (outputs are
 * then untouched).  They use a process-wide context on device 0 with the core and mode set by
 * obs_external_configure (default: Vatistas n=2, compensated).
 */
float external_vel_solver_f_(int* ns, const float* sx, const float* sy, const float* ss, const float* sr,
                             int* nt, const float* tx, const float* ty, float* tu, float* tv);
float external_vel_solver_tr_f_(int* ns, const float* sx, const float* sy, const float* ss, const float* sr,
                                int* nt, const float* tx, const float* ty, const float* tr,
                                float* tu, float* tv);
float external_vel_solver_d_(int* ns, const double* sx, const double* sy, const double* ss, const double* sr,
                             int* nt, const double* tx, const double* ty, double* tu, double* tv);
int obs_external_configure(int core, int accum);
/* Summation behind the external hook: OBS_SUMMATION_DIRECT (default) or OBS_SUMMATION_TREE
 * (obs_points_affect_points_tree with theta and order; 0 selects their defaults) -- the values
 * of summation_t direct and barneshut (src/ExecEnv.h:26-31).  external_vel_solver_d_ always
 * sums directly in FP64. */
#define OBS_SUMMATION_DIRECT 1
#define OBS_SUMMATION_TREE 2
int obs_external_configure_summation(int summation, double theta, int order);

#ifdef __cplusplus
}
#endif

#endif /* OMEGA2D_GB300_H */
