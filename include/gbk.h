/*
 * gbk.h -- C ABI of the GB300 Gaussian kernel-sum library (libgbkernel.so).
 *
 * This is the drop-in boundary for Deformetrica's Gaussian kernel sums. Each entry point
 * replaces one method of the reference's kernel interface
 *   src/support/kernels/AbstractKernel.h:34-187   (virtual Convolve / ConvolveGradient /
 *                                                   ConvolveHessian / ConvolveSpecialHessian)
 *   src/support/kernels/ExactKernel.cxx             (the FP64 CPU implementation)
 *   src/support/kernels/CUDAExactKernel.cxx:41-320  (the legacy CUDA forwarding)
 *   lib/cuda_convolutions/GpuConv1D.h               (GaussGpu*Conv1D host functions)
 * and is what a new KernelFactory kernel type calls.
 *
 * Conventions (all entry points):
 *  - Matrices are row-major double arrays: n rows x c columns, element (i, k) at p[i * c + k],
 *    exactly the buffers the reference builds with vectorise_row_wise()
 *    (src/support/linear_algebra/ArmadilloMatrixWrapper.h:241).
 *    x: targets (nx x d); y: sources (ny x d); w: weights (ny x dv); sigma: kernel width.
 *    K(x, y) = exp(-|x - y|^2 / sigma^2) (ExactKernel.h:78-86).
 *  - Pointers may be device memory or host memory. Device pointers are used in place and the call
 *    is asynchronous on the context's stream. When any pointer is host memory, the library copies
 *    through context-owned device buffers and the call returns after the results are in host
 *    memory (the synchronous behaviour of the reference's GaussGpu*Conv1D).
 *  - Return value: GBK_OK (0) or a GBK_ERR_* code; gbk_last_error(ctx) describes the failure.
 *    Shape errors are the ones the reference throws std::runtime_error for.
 *  - d is 2 or 3. dv may be any positive count; the kernels are compiled for dv in {1,2,3,4} (d=2)
 *    and {1,2,3,6} (d=3) and other counts run as column chunks.
 *  - Precision (gbk_set_mode): GBK_MODE_F32C (default) evaluates pairs in FP32 with per-row
 *    compensated accumulation and per-tile centred coordinates; GBK_MODE_F64 evaluates in FP64.
 *  - A context is not thread-safe; use one context per host thread (the reference clones one
 *    kernel object per subject thread, AbstractAtlas.cxx:218).
 */
#ifndef GBK_H
#define GBK_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbk_ctx gbk_ctx;

enum {
  GBK_OK = 0,
  GBK_ERR_ARG = 1,         /* bad shape / index / pointer (reference: std::runtime_error) */
  GBK_ERR_UNSUPPORTED = 2, /* dimension or dv combination not supported */
  GBK_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  GBK_ERR_ALLOC = 4,       /* device memory allocation failed */
  GBK_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up (reported by gbk_synchronize) */
  GBK_ERR_STATE = 6,       /* call not allowed in the current state (e.g. during capture) */
  GBK_ERR_BOUNDS = 7       /* an index check of a bounds-checked build failed (reported by gbk_synchronize) */
};

enum { GBK_MODE_F32C = 0, GBK_MODE_F64 = 1 };

/* Order in which the kernel sums visit targets and sources (gbk_set_order).
 *  AUTO: SPATIAL for calls with nx, ny >= 4096 and nx * ny >= 2^30. Below that, in GBK_MODE_F32C,
 *    Convolve, the alpha-gradient and their fusion run as TWO_FLOAT; other ops of 2^22 pairs or more
 *    measure the largest extent of the union of the two point sets and run SPATIAL when it is wider
 *    than 16 sigma / sqrt(log2 e) = 13.3 sigma (where one-float caller order loses accuracy), else
 *    OFF (the extent costs one small launch and one wait for the stream, and is skipped while the
 *    stream is being captured). Smaller calls and GBK_MODE_F64 calls below the size rule are OFF.
 *  OFF: rows in caller order, every (target, source) pair evaluated.
 *  SPATIAL: targets and sources sorted along a Morton curve on the device before the sum; each CTA
 *    takes a compact tile of targets (smaller FP32 coordinate rounding after centring) and skips
 *    source chunks too far away to contribute anything but exact zeros in the precision mode.
 *    Outputs are still written in caller row order.
 *  SPATIAL_NOPRUNE: the same order with every pair evaluated (gives the same bits as SPATIAL).
 *  TWO_FLOAT: caller order; in GBK_MODE_F32C, Convolve, the alpha-gradient and their fusion keep
 *    the centred coordinates of every CTA whose targets spread wider than 16 units of the FP32
 *    coordinate scale (13.3 sigma) as two floats (hi + lo), so a pair's difference is accurate to
 *    ~2u of itself however far the points spread (about 20 % more time in such CTAs; the others
 *    run as OFF; other ops as OFF).
 * The reference has no counterpart: ExactKernel always visits every pair in row order. */
enum {
  GBK_ORDER_AUTO = 0,
  GBK_ORDER_OFF = 1,
  GBK_ORDER_SPATIAL = 2,
  GBK_ORDER_SPATIAL_NOPRUNE = 3,
  GBK_ORDER_TWO_FLOAT = 4
};

/* Gradient formula of the point-cloud and volume-mesh data terms (gbk_set_gradient_mode).
 *  REFERENCE: the reference's formulas. PointCloud::ComputeMatchGradient (PointCloud.cxx:150-198)
 *    returns 2 (G_S + G_T), adding the target term the match subtracts; OrientedVolumeMesh
 *    (OrientedVolumeMesh.cxx:159-280) differentiates the signed volume although the match uses its
 *    absolute value, which agrees with EXACT on positively oriented cells only.
 *  EXACT: the derivative of the match: 2 (G_S - G_T) for point clouds, the determinant's sign
 *    applied per cell for volume meshes. */
enum { GBK_GRADIENT_REFERENCE = 0, GBK_GRADIENT_EXACT = 1 };

/* Estimator of the *_optimize calls (gbk_set_estimator): the reference's FastGradientAscent
 * (FastGradientAscent.cxx:48-300, its default) or GradientAscent (GradientAscent.cxx:48-240:
 * no extrapolation, no sufficient-increase term, every step expanded after an accepted step). */
enum { GBK_ESTIMATOR_FAST_GRADIENT_ASCENT = 0, GBK_ESTIMATOR_GRADIENT_ASCENT = 1 };

/* Operation identifiers (for gbk_autotune). */
enum {
  GBK_OP_CONVOLVE = 0,
  GBK_OP_CONVOLVE_GRADIENT_ALPHA_FUSED = 1,
  GBK_OP_GRADIENT_ALPHA = 2,
  GBK_OP_GRADIENT_VARLIN = 3,
  GBK_OP_GRADIENT_DIM = 4,
  GBK_OP_HESSIAN = 5,
  GBK_OP_HESSIAN_ROWCOL = 6,
  GBK_OP_SPECIAL_HESSIAN = 7
};

/* ---- context --------------------------------------------------------------------------- */

/* Library version (major * 10000 + minor * 100 + patch). */
int gbk_version(void);

/* Creates a context on CUDA device `device` with its own non-blocking stream. Replaces the
 * per-call cudaMalloc/cudaFree of GpuConv1D.cu:97-130 with buffers that grow monotonically. */
int gbk_create(int device, gbk_ctx **out);
void gbk_destroy(gbk_ctx *ctx);
/* Message of the last failed call on this context ("" if none). */
const char *gbk_last_error(const gbk_ctx *ctx);
/* Uses `stream` (a cudaStream_t) for all later calls; NULL restores the context's own stream
 * (pass cudaStreamLegacy, i.e. (void *)0x1, to queue on the legacy default stream). */
int gbk_set_stream(gbk_ctx *ctx, void *stream);
void *gbk_get_stream(const gbk_ctx *ctx);
int gbk_set_mode(gbk_ctx *ctx, int mode);
int gbk_get_mode(const gbk_ctx *ctx);

/* How the spatial order's Convolve-like kernel sums stage each chunk of TJ sorted sources into shared
 * memory (gbk_set_staging; no counterpart in the reference, whose legacy CUDA kernel loads each
 * source tile with every thread, GpuConv1D.cu:35-84):
 *  AUTO: BULK (measured on GB300 at N = M = 1e6, d = 3: 3 % faster at sigma = 0.1, 4 % at 0.02);
 *  LOADS: every thread loads and converts its records with ordinary global loads;
 *  BULK: one thread fetches the next visited chunk's coordinates and weights with cp.async.bulk into
 *    the other half of a double buffer (completion on an mbarrier) while the CTA computes the
 *    current one, then every thread converts from shared memory. Same results, bit for bit. A wait
 *    that does not complete within about a second stops the CTA and is reported by gbk_synchronize
 *    as GBK_ERR_TIMEOUT. */
enum { GBK_STAGING_AUTO = 0, GBK_STAGING_LOADS = 1, GBK_STAGING_BULK = 2 };
int gbk_set_staging(gbk_ctx *ctx, int staging);
int gbk_get_staging(const gbk_ctx *ctx);
/* The compiled variant (launch shape) and source-split count of the context's last kernel-sum launch
 * (-1, 0 before any); for reports and the autotuner's tests. */
int gbk_last_launch(const gbk_ctx *ctx, int *variant, int *nsplit);
/* Sets the GBK_ORDER_* policy of later kernel-sum calls (default GBK_ORDER_AUTO). The
 * registration, atlas and regression steps always use GBK_ORDER_TWO_FLOAT (no sort inside their graphs;
 * the adaptive two-float variant keeps their accuracy on points spread wide relative to sigma). No
 * counterpart in the reference. */
int gbk_set_order(gbk_ctx *ctx, int order);
int gbk_get_order(const gbk_ctx *ctx);
/* Sets the GBK_GRADIENT_* formula of later point-cloud and volume-mesh data terms (default
 * GBK_GRADIENT_REFERENCE; a registration takes the mode current at its creation). */
int gbk_set_gradient_mode(gbk_ctx *ctx, int mode);
int gbk_get_gradient_mode(const gbk_ctx *ctx);
/* Sets the GBK_ESTIMATOR_* of later *_optimize calls (default FastGradientAscent). With
 * GradientAscent the optimisers' tau, freeze-counter and aux outputs are not set. */
int gbk_set_estimator(gbk_ctx *ctx, int estimator);
int gbk_get_estimator(const gbk_ctx *ctx);
/* Waits for all work queued on the context's stream. Returns GBK_ERR_TIMEOUT (and clears the report)
 * when a kernel sum's bounded device-side wait gave up since the last call (see GBK_STAGING_BULK), and
 * GBK_ERR_BOUNDS when, in a library built with bounds checks (GBK_BOUNDS_CHECK=1: build.py
 * build(bounds_check=True), libgbkernel_checked.so), a kernel sum met a target or source index
 * outside its arrays (the index was clamped and the outputs are not valid). */
int gbk_synchronize(gbk_ctx *ctx);
/* Number of the library's own kernels launched on this context so far. */
long long gbk_launch_count(const gbk_ctx *ctx);
/* (target, source) pairs the kernel sums of this context have evaluated so far (pairs in source
 * chunks skipped by GBK_ORDER_SPATIAL are not counted; the registration, atlas and regression steps
 * on this context are, graph replays included). Waits for the context's stream; -1 on error. No
 * counterpart in the reference. */
long long gbk_evaluated_pairs(gbk_ctx *ctx);
/* The same per operation: counts[op] for op = 0 .. n-1 (GBK_OP_* order; 9 operations, the last the
 * fused control-point adjoint update), including the batched atlas launches. Waits for the stream. */
int gbk_evaluated_pairs_by_op(gbk_ctx *ctx, long long *counts, int n);

/* ---- kernel sums (AbstractKernel surface) ------------------------------------------------ */

/* ExactKernel::Convolve, ExactKernel.cxx:51-74; CUDAExactKernel::Convolve, CUDAExactKernel.cxx:41-90;
 * GaussGpuEvalConv1D, GpuConv1D.cu:148-155.  out[i, k] = sum_j K(x_i, y_j) w[j, k]   (nx x dv) */
int gbk_convolve(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y,
                 const double *w, long ny, double sigma, double *out);

/* ExactKernel::ConvolveGradient(X, alpha), ExactKernel.cxx:264-275; CUDAExactKernel.cxx:165-194;
 * GaussGpuGrad1Conv1D, GpuConv1D.cu:282-288.
 * out[i, :] = sum_j (alpha_i . w_j) (-2 K_ij / sigma^2)(x_i - y_j)   (nx x d; alpha is nx x dv) */
int gbk_convolve_gradient_alpha(gbk_ctx *ctx, int d, int dv, const double *x, long nx,
                                const double *y, const double *w, long ny, double sigma,
                                const double *alpha, double *out);

/* Convolve and ConvolveGradient(X, alpha) of the same (x, y, w) in ONE pass over the pairs
 * (distance and exp evaluated once per pair). out_v: nx x dv, out_g: nx x d. */
int gbk_convolve_and_gradient_alpha(gbk_ctx *ctx, int d, int dv, const double *x, long nx,
                                    const double *y, const double *w, long ny, double sigma,
                                    const double *alpha, double *out_v, double *out_g);

/* ExactKernel::ConvolveGradient(X) ("varlin"), ExactKernel.cxx:166-202; CUDAExactKernel.cxx:261-320;
 * GpuGradConv_varlin_1D, GpuConv1D.cu:475-521.
 * out[i, k, l] = sum_j w[j, k] dK(x_i, y_j)/dx_l      (nx x dv x d; the reference's
 * std::vector<MatrixType> of dv x d matrices, one per target) */
int gbk_convolve_gradient(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y,
                          const double *w, long ny, double sigma, double *out);

/* ExactKernel::ConvolveGradient(X, dim), ExactKernel.cxx:294-323 (general sources; the legacy CUDA
 * GpuGradConv1D, GpuConv1D.cu:350-392, assumed X == sources).
 * out[i, k] = sum_j dK(x_i, y_j)/dx_dim w[j, k]       (nx x dv) */
int gbk_convolve_gradient_dim(gbk_ctx *ctx, int d, int dv, const double *x, long nx,
                              const double *y, const double *w, long ny, double sigma, int dim,
                              double *out);

/* ExactKernel::ConvolveGradient(X, k, dp), ExactKernel.cxx:325-363, including its quirk: the
 * result has ny entries (one per SOURCE) and reads the first ny rows of x, so nx >= ny.
 * out[i] = sum_j w[j, k] dK(x_i, y_j)/dx_dp, i < ny */
int gbk_convolve_gradient_kdp(gbk_ctx *ctx, int d, int dv, const double *x, long nx,
                              const double *y, const double *w, long ny, double sigma, int k,
                              int dp, double *out);

/* ExactKernel::ConvolveHessian(X), ExactKernel.cxx:365-397.
 * out[i, k, a, b] = sum_j w[j, k] H_ab(x_i, y_j), H = K (4 (x-y)(x-y)^T / s^4 - 2 I / s^2)
 * (nx x dv x d x d) */
int gbk_convolve_hessian(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y,
                         const double *w, long ny, double sigma, double *out);

/* ExactKernel::ConvolveHessian(X, row, col), ExactKernel.cxx:399-428.  out: nx x dv */
int gbk_convolve_hessian_rowcol(gbk_ctx *ctx, int d, int dv, const double *x, long nx,
                                const double *y, const double *w, long ny, double sigma, int row,
                                int col, double *out);

/* ExactKernel::ConvolveHessian(X, k, dp, dq), ExactKernel.cxx:430-470.  out: nx */
int gbk_convolve_hessian_kdpdq(gbk_ctx *ctx, int d, int dv, const double *x, long nx,
                               const double *y, const double *w, long ny, double sigma, int k,
                               int dp, int dq, double *out);

/* AbstractKernel::ConvolveSpecialHessian(xi), AbstractKernel.cxx:22-88;
 * CUDAExactKernel::ConvolveSpecialHessian, CUDAExactKernel.cxx:196-226 (GradDiff x -1/2).
 * Sources y (n x d) with weights beta = w (n x d), xi (n x d):
 * out[i, :] = sum_j (beta_i . beta_j) H(y_i, y_j) (xi_j - xi_i)   (n x d) */
int gbk_convolve_special_hessian(gbk_ctx *ctx, int d, const double *y, const double *w, long n,
                                 double sigma, const double *xi, double *out);

/* Forward + adjoint of L = sum_i alpha_i . (K w)_i in two fused passes (distance and exp are
 * recomputed, never stored): v = Convolve (nx x dv), gx = dL/dx (nx x d, equal to
 * ConvolveGradient(X, alpha)), gy = dL/dy (ny x d), gw = dL/dw (ny x dv). Any output may be NULL.
 * The source side has no single reference method; it equals ConvolveGradient(Y, w) and
 * Convolve(Y) with sources X and weights alpha (K is symmetric). */
int gbk_forward_adjoint(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y,
                        const double *w, long ny, double sigma, const double *alpha, double *v,
                        double *gx, double *gy, double *gw);

/* <w, K w> = sum_ij w_i . K(y_i, y_j) w_j, summed in FP64 on the device (the RKHS regularity
 * term, DeterministicAtlas.cxx:126-141). `out` is one double (host or device). */
int gbk_kernel_norm(gbk_ctx *ctx, int d, int dv, const double *y, const double *w, long n,
                    double sigma, double *out);

/* ---- deformation (trajectories are T x n x d row-major blocks; dt = 1 / (T - 1)) --------- */

/* Diffeos::Shoot, Diffeos.cxx:589-660: explicit Euler on x' = K(x,x) p, p' = -G(x)^T p, one
 * fused Convolve + alpha-gradient pass per step. Nearly zero momenta (|p0|_F < 1e-20) give the
 * reference's constant trajectory (:611-613). */
int gbk_shoot(gbk_ctx *ctx, int d, long ncp, const double *cp0, const double *mom0, int T,
              double sigma, double *pos_traj, double *mom_traj);

/* Diffeos::FlowLandmarkPointsTrajectory, Diffeos.cxx:661-712: y' = K(y, x_t) p_t with Heun's
 * scheme when heun != 0 (the reference's ImprovedEuler default, Diffeos.cxx:27). */
int gbk_flow_landmarks(gbk_ctx *ctx, int d, long ncp, const double *pos_traj,
                       const double *mom_traj, int T, double sigma, long nlm, const double *lm0,
                       int heun, double *lm_traj);

/* AdjointEquationsIntegrator::IntegrateAdjointOfLandmarkPointsEquations,
 * AdjointEquationsIntegrator.cxx:59-136 (no jumps): theta backward from theta_final. */
int gbk_adjoint_landmarks(gbk_ctx *ctx, int d, long ncp, const double *pos_traj,
                          const double *mom_traj, int T, double sigma, long nlm,
                          const double *lm_traj, const double *theta_final, int heun,
                          double *theta_traj);

/* AdjointEquationsIntegrator::ComputeUpdateAt, AdjointEquationsIntegrator.cxx:476-570 (landmark
 * points): dpos = dXi1 + dXi3 + dXi4, dmom = dXi2 + dXi5 + dXi6, in one fused CP x CP pass and
 * one fused CP x landmark pass (nlm may be 0). */
int gbk_compute_update_at(gbk_ctx *ctx, int d, long ncp, const double *pos, const double *mom,
                          const double *xi_pos, const double *xi_mom, long nlm, const double *lm,
                          const double *theta, double sigma, double *dpos, double *dmom);

/* AdjointEquationsIntegrator::IntegrateAdjointOfDiffeoParametersEquations, :414-470. */
int gbk_adjoint_diffeo(gbk_ctx *ctx, int d, long ncp, const double *pos_traj,
                       const double *mom_traj, int T, double sigma, long nlm,
                       const double *lm_traj, const double *theta_traj, int heun,
                       double *xipos_traj, double *ximom_traj);

/* ---- surface data terms (d = 3; triangles are int triplets, host or device) -------------- */

/* OrientedSurfaceMesh::ComputeMatch / ComputeMatchGradient, OrientedSurfaceMesh.cxx:124-241
 * (currents): *match = |T|^2 + |S|^2 - 2 <S,T>; grad (nv x 3, may be NULL) = d match / d pts.
 * Reductions are FP64; `match` is one double. */
int gbk_currents_match(gbk_ctx *ctx, long nv, const double *pts, long nf, const int *tris,
                       long nv_t, const double *pts_t, long nf_t, const int *tris_t, double sigma,
                       double *match, double *grad);

/* NonOrientedSurfaceMesh::ComputeMatch / ComputeMatchGradient, NonOrientedSurfaceMesh.cxx:124-265
 * (varifolds). */
int gbk_varifold_match(gbk_ctx *ctx, long nv, const double *pts, long nf, const int *tris,
                       long nv_t, const double *pts_t, long nf_t, const int *tris_t, double sigma,
                       double *match, double *grad);
/* OrientedPolyLine::ComputeMatch / ComputeMatchGradient (curve currents: segment centres and
 * tangents p1 - p0) between two polylines of nseg 2-point segments in d = 2 or 3 dimensions. */
int gbk_curve_currents_match(gbk_ctx *ctx, int d, long nv, const double *pts, long nseg, const int *segs,
                             long nv_t, const double *pts_t, long nseg_t, const int *segs_t, double sigma,
                             double *match, double *grad);
/* NonOrientedPolyLine::ComputeMatch / ComputeMatchGradient (NonOrientedPolyLine.cxx:125-256:
 * curve varifold, tangents t / sqrt(|t|) and their tensors). */
int gbk_curve_varifold_match(gbk_ctx *ctx, int d, long nv, const double *pts, long nseg, const int *segs,
                             long nv_t, const double *pts_t, long nseg_t, const int *segs_t, double sigma,
                             double *match, double *grad);
/* PointCloud::ComputeMatch / ComputeMatchGradient (PointCloud.cxx:104-198): weighted points
 * (w, w_t: one weight per point, NULL = unit weights as UpdatePointWeights, :204-225),
 * match = |T|^2 + |S|^2 - 2 sum_i (K_S w_S)(t_i) w_T,i, gradient per gbk_set_gradient_mode. */
int gbk_pointcloud_match(gbk_ctx *ctx, int d, long n, const double *pts, const double *w, long n_t,
                         const double *pts_t, const double *w_t, double sigma, double *match, double *grad);
/* OrientedVolumeMesh::ComputeMatch / ComputeMatchGradient (OrientedVolumeMesh.cxx:115-280):
 * cells of d + 1 vertices (tetrahedra in 3-D, triangles in 2-D) carry their centres and volumes
 * |det(p_1 - p_0, ..., p_d - p_0)| / d!; gradient per gbk_set_gradient_mode. */
int gbk_volume_match(gbk_ctx *ctx, int d, long nv, const double *pts, long ncell, const int *cells, long nv_t,
                     const double *pts_t, long ncell_t, const int *cells_t, double sigma, double *match,
                     double *grad);
/* Landmark::ComputeMatch / ComputeMatchGradient (Landmark.cxx:288-322): |S - T|_F^2 and 2 (S - T)
 * over n corresponding points. */
int gbk_landmark_match(gbk_ctx *ctx, int d, long n, const double *pts, const double *pts_t, double *match,
                       double *grad);

/* ---- registration iteration (shooting + flow + data term + adjoint), CUDA-graph replay ---- */

typedef struct gbk_registration gbk_registration;

/* One subject of DeterministicAtlas with a frozen template (DeterministicAtlas.cxx:99-154,
 * AbstractAtlas.cxx:559-613): template (nv points, nf cells) deformed by ncp control points over T
 * time points, matched to the target with data_kind 0 = surface currents, 1 = surface varifold
 * (triangles, d = 3), 2 = curve currents, 3 = curve varifold (2-point segments, d = 2 or 3),
 * 4 = point cloud (nf = nv, nf_t = nv_t, the cell arrays are ignored and may be NULL; unit weights
 * until gbk_registration_set_point_weights), 5 = volume mesh (cells of d + 1 vertices), 6 =
 * landmarks (nv_t = nv, cells ignored). All device memory is allocated here, except that the first
 * step creates two helper contexts (streams and small buffers, destroyed with the registration) so
 * that the iteration runs on three streams, one step apart; GBK_PIPELINE=0 in the environment at
 * creation keeps one stream (same results bit for bit). */
int gbk_registration_create(gbk_ctx *ctx, int d, long ncp, long nv, const double *tmpl_pts,
                            long nf, const int *tmpl_tris, long nv_t, const double *tgt_pts,
                            long nf_t, const int *tgt_tris, int T, double sigma_def,
                            double sigma_data, double data_sigma2, int data_kind, int heun,
                            gbk_registration **out);
/* A registration whose template has nobj objects (DeformableMultiObject): object k has data_kinds[k]
 * (as data_kind above), nv[k] template points and ncell[k] cells (points and cells concatenated
 * over the objects in tmpl_pts / tmpl_cells, cell indices local to their object), its target's
 * nv_t[k] points and ncell_t[k] cells likewise, data kernel width sigma_data[k] and data sigma^2
 * data_sigma2[k] (the per-object arrays on the host). All template points flow together;
 * L_data = -0.5 sum_k match_k / data_sigma2_k (DeterministicAtlas.cxx:121-125) and loglik[3] is the
 * sum of the matches. */
int gbk_registration_create_multi(gbk_ctx *ctx, int d, long ncp, int nobj, const int *data_kinds, const long *nv,
                                  const double *tmpl_pts, const long *ncell, const int *tmpl_cells, const long *nv_t,
                                  const double *tgt_pts, const long *ncell_t, const int *tgt_cells,
                                  const double *sigma_data, const double *data_sigma2, int T, double sigma_def,
                                  int heun, gbk_registration **out);
/* Replaces the template points (all objects, nv x d, host or device); a captured iteration graph
 * reads the new points. */
int gbk_registration_set_template(gbk_registration *reg, const double *pts);
/* Log-likelihood and gradient at (cp, mom): loglik[5] = {L, L_data, L_reg, match, <K p, p>},
 * grad_cp / grad_mom = dL/dcp, dL/dp (ncp x d). Any output may be NULL. Returns when the outputs
 * are written. The first call runs the kernels directly, the second captures them into a CUDA
 * graph, later calls replay it. */
int gbk_registration_step(gbk_registration *reg, const double *cp, const double *mom,
                          double *loglik, double *grad_cp, double *grad_mom);
/* Point weights of the point-cloud objects (data_kind 4) of a registration: template weights over
 * all template points (nv, entries of other objects ignored) and target weights over all target
 * points, host or device; either may be NULL to keep the current ones. A captured iteration
 * graph reads the new weights (same device buffers). */
int gbk_registration_set_point_weights(gbk_registration *reg, const double *w_tmpl, const double *w_tgt);
/* 0 disables graph capture (every step launches the kernels directly). */
int gbk_registration_set_graph(gbk_registration *reg, int enable);
/* Copies of the last step's trajectories (T x ncp x d or T x nv x d); any pointer may be NULL. */
int gbk_registration_trajectories(gbk_registration *reg, double *pos, double *mom, double *lm,
                                  double *theta, double *xi_pos, double *xi_mom);
/* Kernels in one captured iteration (0 before the capture). */
long long gbk_registration_graph_launches(const gbk_registration *reg);
/* FastGradientAscent::Update (FastGradientAscent.cxx:48-300) of this registration: Nesterov-
 * accelerated gradient ascent with one step size per parameter group (control points when
 * optimize_cp, then momenta), multivariate line search, step expansion after nb_iter_freeze
 * accepted first trials, stop on |dL| < tolerance |L_0 - L| (reference defaults: 10 line-search
 * iterations, shrink 0.5, expand 1.2, tolerance 1e-4, nb_iter_freeze 3). Parameters, trials and
 * gradients stay on the device; every evaluation replays the iteration graph. cp and mom (ncp x 3,
 * host or device) are the start point and receive the final fixed effects; history receives one
 * [data, regularity] row per accepted iteration (at most max_iterations + 1 rows, *iterations of
 * them); info (8 doubles, optional): final step sizes (control points, momenta), tau, the freeze
 * counter, the two squared gradient norms, the number of evaluations and the stop reason (0 max
 * iterations, 1 line search exhausted, 2 tolerance). aux_cp / aux_mom / grad_cp / grad_mom
 * (optional) receive the extrapolated point and the gradient there, as the reference's state. */
int gbk_registration_optimize(gbk_registration *reg, double *cp, double *mom, int optimize_cp, int max_iterations,
                              double initial_step, int max_line_search, double shrink, double expand,
                              double tolerance, int nb_iter_freeze, double *history, int *iterations,
                              double *info, double *aux_cp, double *aux_mom, double *grad_cp,
                              double *grad_mom);
void gbk_registration_destroy(gbk_registration *reg);

/* The same <w, K w> for callers that cannot allocate device memory when they need it (a loop
 * running inside a memory budget fixed at start-up, a pre-sized pool, a stream whose operations
 * must all be known in advance). No counterpart in the reference. Allocates nothing: its scratch
 * (the K w intermediate and source-split partials) is a 16 MiB __device__ array in the library,
 * held by every GPU that loads it until the process exits. y, w and `out` (one double) must be
 * device pointers of the context's GPU (host memory, another GPU's memory and a NaN kernel width
 * return GBK_ERR_ARG); n * dv above 2^21 (2,097,152) returns GBK_ERR_ARG before any launch;
 * gbk_last_error describes every failure. The first call on a device looks up the array's address:
 * make it before any stream capture (a first call on a capturing stream returns GBK_ERR_STATE).
 * After a cudaDeviceReset, create a new context on that device before calling again: gbk_create
 * refreshes the cached address. All calls share the array, so calls that overlap on the GPU race:
 * serialise them. Queued on the context's stream; counted by gbk_launch_count. */
int gbk_kernel_norm_noalloc(gbk_ctx *ctx, int d, int dv, const double *y, const double *w, long n,
                            double sigma, double *out);

/* ---- particle-mesh approximation (the reference's P3MKernel) -------------------------------- */

/* P3MKernel::Convolve (P3MKernel.cxx:1245-1355): the sources' weights splatted multilinearly onto a
 * grid of spacing spacing_ratio x sigma covering the data domain padded by padding_factor x sigma on
 * each side (sizes rounded up to powers of two, DetermineGrids :371-432), convolved with the
 * sampled Gaussian by FFT (cuFFT), interpolated multilinearly at the targets. domain: 2 d doubles on
 * the host (lo[0..d-1], hi[0..d-1]), or NULL for the bounding box of targets and sources. The
 * reference's defaults are spacing_ratio 0.2 and padding_factor 3 (SparseDiffeoParameters.cxx:25-27).
 * An approximation: a few percent relative error against the exact sums. d = 2 or 3, FP64. */
int gbk_p3m_convolve(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y, const double *w, long ny,
                     double sigma, const double *domain, double spacing_ratio, double padding_factor, double *out);
/* P3MKernel::ConvolveGradient(X) (:1386-1447): out nx x dv x d from the sampled kernel gradient. */
int gbk_p3m_convolve_gradient(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y, const double *w,
                              long ny, double sigma, const double *domain, double spacing_ratio, double padding_factor,
                              double *out);
/* P3MKernel::ConvolveGradient(X, alpha) (:1357-1366): out nx x d, the gradient contracted with alpha. */
int gbk_p3m_convolve_gradient_alpha(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y,
                                    const double *w, long ny, double sigma, const double *alpha, const double *domain,
                                    double spacing_ratio, double padding_factor, double *out);
/* P3MKernel::ConvolveGradient(X, dim) (:1443-1504): out nx x dv from the gradient kernel `dim`. */
int gbk_p3m_convolve_gradient_dim(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y,
                                  const double *w, long ny, double sigma, int dim, const double *domain,
                                  double spacing_ratio, double padding_factor, double *out);
/* P3MKernel::ConvolveHessian(X) (:1549-1620; Hessian kernels :947-1085): out nx x dv x d x d
 * (symmetric), from the d(d+1)/2 sampled Hessian entries of the kernel. */
int gbk_p3m_convolve_hessian(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y, const double *w,
                             long ny, double sigma, const double *domain, double spacing_ratio, double padding_factor,
                             double *out);
/* P3MKernel::ConvolveHessian(X, row, col) (:1622-1687): out nx x dv. */
int gbk_p3m_convolve_hessian_rowcol(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y,
                                    const double *w, long ny, double sigma, int row, int col, const double *domain,
                                    double spacing_ratio, double padding_factor, double *out);
/* P3MKernel::ConvolveGradient(X, k, dp) and ConvolveHessian(X, k, dp, dq) (:1506-1547, :1689-1729):
 * the reference checks the indices and returns nx zeros; so do these (out: nx doubles). */
int gbk_p3m_convolve_gradient_kdp(gbk_ctx *ctx, int d, int dv, long nx, long ny, int k, int dp, double *out);
int gbk_p3m_convolve_hessian_kdpdq(gbk_ctx *ctx, int d, int dv, long nx, long ny, int k, int dp, int dq, double *out);

/* ---- the image grid (ExactKernel::ConvolveImageFast and the Diffeos image maps) ------------ *
 * An image is its geometry on the host: origin[d], spacing[d] and size[d] (pixels per axis,
 * identity direction); its points are listed first index fastest (GridFunctions::ImageToPoints,
 * GridFunctions.cxx:41-60). The windowed sums follow the context's precision: GBK_MODE_F64 is the
 * reference's FP64 arithmetic in its order of additions per pixel, GBK_MODE_F32C FP32 exponentials
 * with compensated per-pixel sums (~1e-7 relative). */

/* The physical points of the pixels: points (prod(size) x d) = origin + spacing * index. */
int gbk_image_points(gbk_ctx *ctx, int d, const double *origin, const double *spacing, const long *size,
                     double *points);
/* ExactKernel::ConvolveImageFast (src/support/kernels/ExactKernel.cxx:76-129): out (nx x d) =
 * sum over control points y_j (ny x d, momenta w ny x d) of w_j K(x_p, y_j) over the pixels p of the
 * window of int(6 sigma) pixels per axis starting at the index of y_j - 3 sigma (rounded half up),
 * cropped to the image. x holds one (deformed) point per pixel: nx = prod(size). A window that
 * misses the image returns GBK_ERR_ARG (the reference's ITK region iterator throws), as does
 * 6 sigma < 1. */
int gbk_convolve_image_fast(gbk_ctx *ctx, int d, const double *x, long nx, const double *y, const double *w, long ny,
                            double sigma, const double *origin, const double *spacing, const long *size,
                            double *out);
/* ExactKernel::ConvolveGradientImageFast(X, image) (src/support/kernels/ExactKernel.cxx:207-257): the
 * same windows; out (nx x dv x d, row p = the dv x d matrix G_p) with G_p(k, l) = sum over the control
 * points y_j whose window holds pixel p of w_jk (x_p - y_j)_l (-2 K(x_p, y_j) / sigma^2)
 * (EvaluateKernelGradient, ExactKernel.h:98-110); w is ny x dv, any dv >= 1. Errors as
 * gbk_convolve_image_fast. The reference's image adjoint calls it (AdjointEquationsIntegrator.cxx:196). */
int gbk_convolve_gradient_image_fast(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y,
                                     const double *w, long ny, double sigma, const double *origin,
                                     const double *spacing, const long *size, double *out);
/* ExactKernel::ConvolveGradientImageFast(X, alpha, image) (ExactKernel.cxx:277-290): out (nx x d),
 * row p = G_p^T alpha_p with G_p as above and alpha nx x dv (AdjointEquationsIntegrator.cxx:389, 401). */
int gbk_convolve_gradient_image_fast_alpha(gbk_ctx *ctx, int d, int dv, const double *x, long nx, const double *y,
                                           const double *w, long ny, double sigma, const double *alpha,
                                           const double *origin, const double *spacing, const long *size,
                                           double *out);
/* The backward integration of the image maps (Diffeos.cxx:725-770, non-regression branch): all T
 * maps (T x prod(size) x d) start as the image points; unless |mom_traj[0]| < 1e-20, from
 * t = T-1 down, maps[t-1] = maps[t] - dt V(maps[t]; pos[t], mom[t]) (Heun: the average of both
 * ends), dt = span / (T-1), V the windowed sum (fast = 1) or the full kernel sum (fast = 0), in the
 * context's precision. bbox (host, d x 2: lo, hi per axis, or NULL) stops the integration after
 * the first step whose map leaves it (Diffeos::CheckBoundingBox); *stopped_at = that time index,
 * or -1. */
int gbk_flow_image_maps(gbk_ctx *ctx, int d, long ncp, const double *pos_traj, const double *mom_traj, int T,
                        double sigma, double span, int heun, int fast, const double *origin, const double *spacing,
                        const long *size, const double *bbox, double *maps_traj, int *stopped_at);

/* ---- geodesic regression (the reference's Regression model), CUDA-graph replay ------------ */

typedef struct gbk_geodesic_regression gbk_geodesic_regression;

/* Regression.cxx: a template of nobj objects (described as for gbk_registration_create_multi) flows
 * along the geodesic of (control points, initial momenta) from t0 to tn over T time points;
 * observation o (nobs of them, time indices time_index[o], not decreasing: the reference's
 * int((age - t0)(T - 1)/(tn - t0) + 0.5f), estimate_geodesic_regression.cxx:229-237) has, per object
 * k, nv_t[o * nobj + k] points and ncell_t[o * nobj + k] cells, concatenated observation by
 * observation, object by object. */
int gbk_geodesic_regression_create(gbk_ctx *ctx, int d, long ncp, int nobj, const int *data_kinds, const long *nv,
                                   const double *tmpl_pts, const long *ncell, const int *tmpl_cells,
                                   const double *sigma_data, const double *data_sigma2, int nobs, const int *time_index,
                                   const long *nv_t, const double *tgt_pts, const long *ncell_t, const int *tgt_cells,
                                   int T, double sigma_def, double t0, double tn, int heun,
                                   gbk_geodesic_regression **out);
/* Template-gradient smoothing width (Regression::ConvolveGradTemplate, Regression.cxx:688-712;
 * the reference uses smoothing-kernel-width-ratio x deformation kernel width); 0 keeps L2. */
int gbk_geodesic_regression_set_template_smoothing(gbk_geodesic_regression *reg, double width);
/* 0 (default): the reference's gradient -- no regularity gradient (AddGradientRegularityTerm,
 * Regression.cxx:676-686, works on copies), observations entering the landmark adjoint as rates
 * times dt, at most one of them inside the explicit-Euler loop, none at time index 0
 * (AdjointEquationsIntegrator.cxx:59-136). 1: the regularity gradients applied and every
 * observation added to the adjoint at its own time index. */
int gbk_geodesic_regression_set_corrected_gradient(gbk_geodesic_regression *reg, int enable);
int gbk_geodesic_regression_set_graph(gbk_geodesic_regression *reg, int enable);
/* loglik[5] = {L, L_data, L_reg, sum of matches, <K p, p>} at (cp, mom: ncp x d; tmpl: nv x d or
 * NULL to keep the current template), and the gradients (the template one smoothed); any output
 * may be NULL. */
int gbk_geodesic_regression_step(gbk_geodesic_regression *reg, const double *cp, const double *mom, const double *tmpl,
                                 double *loglik, double *grad_cp, double *grad_mom, double *grad_tmpl);
/* FastGradientAscent over the reference's groups [ControlPoints] InitialMomenta [TemplateData]
 * (Regression.cxx:279-286). info (10 doubles): final steps (cp, momenta, template), tau, freeze
 * counter, squared norms (cp, momenta, template as <L2, smoothed>), evaluations, stop reason. */
int gbk_geodesic_regression_optimize(gbk_geodesic_regression *reg, double *cp, double *mom, double *tmpl,
                                     int optimize_cp, int optimize_template, int max_iterations, double initial_step,
                                     int max_line_search, double shrink, double expand, double tolerance,
                                     int nb_iter_freeze, double *history, int *iterations, double *info,
                                     double *aux_cp, double *aux_mom, double *aux_tmpl, double *grad_cp,
                                     double *grad_mom, double *grad_tmpl);
void gbk_geodesic_regression_destroy(gbk_geodesic_regression *reg);

/* ---- atlas with a multi-object template, one registration per subject ------------------- */

typedef struct gbk_mo_atlas gbk_mo_atlas;

/* DeterministicAtlas (DeterministicAtlas.cxx:99-280, AbstractAtlas.cxx:492-748) of nsubj subjects
 * with a template of nobj objects, described as for gbk_registration_create_multi: template
 * objects by data_kinds, nv, tmpl_pts, ncell, tmpl_cells, sigma_data, data_sigma2; the subjects'
 * objects by nv_t[s * nobj + k] points and ncell_t[s * nobj + k] cells, their points and cells
 * concatenated subject by subject, object by object, in tgt_pts / tgt_cells. Every subject runs as
 * one replayed iteration graph, subjects in order on the atlas's stream. */
int gbk_mo_atlas_create(gbk_ctx *ctx, int d, long ncp, int nobj, const int *data_kinds, const long *nv,
                        const double *tmpl_pts, const long *ncell, const int *tmpl_cells, const double *sigma_data,
                        const double *data_sigma2, int nsubj, const long *nv_t, const double *tgt_pts,
                        const long *ncell_t, const int *tgt_cells, int T, double sigma_def, int heun,
                        gbk_mo_atlas **out);
/* Template-gradient smoothing width (ConvolveGradTemplate, AbstractAtlas.cxx:724-748), applied
 * object by object over that object's template points; 0 (default) keeps the L2 gradient. */
int gbk_mo_atlas_set_template_smoothing(gbk_mo_atlas *atlas, double width);
/* 1 (default): the optimiser deforms the template of the previous SetFixedEffects call, as the
 * reference's AbstractAtlas::SetFixedEffects (AbstractAtlas.cxx:52-65) does, while the step and the
 * smoothing use the current template; 0: every evaluation deforms its own template. */
int gbk_mo_atlas_set_lagged_template(gbk_mo_atlas *atlas, int enable);
/* loglik[3] = {L, L_data, L_reg} at (cp: ncp x d, tmpl: nv x d, mom: nsubj x ncp x d), host or
 * device; grad_cp, grad_tmpl (smoothed), grad_mom: the gradients (any may be NULL). */
int gbk_mo_atlas_step(gbk_mo_atlas *atlas, const double *cp, const double *tmpl, const double *mom, double *loglik,
                      double *grad_cp, double *grad_tmpl, double *grad_mom);
/* FastGradientAscent (FastGradientAscent.cxx:48-300) over [control points] [template] momenta, as
 * gbk_atlas_optimize (same info layout); aux_* / grad_* (optional) receive the extrapolated point
 * and the gradient there. */
int gbk_mo_atlas_optimize(gbk_mo_atlas *atlas, double *cp, double *tmpl, double *mom, int optimize_cp,
                          int optimize_template, int max_iterations, double initial_step, int max_line_search,
                          double shrink, double expand, double tolerance, int nb_iter_freeze, double *history,
                          int *iterations, double *info, double *aux_cp, double *aux_tmpl, double *aux_mom,
                          double *grad_cp, double *grad_tmpl, double *grad_mom);
void gbk_mo_atlas_destroy(gbk_mo_atlas *atlas);

/* ---- batched atlas iteration (all subjects per launch), CUDA-graph replay ---------------- */

typedef struct gbk_atlas gbk_atlas;

/* A DeterministicAtlas iteration with a shared template mesh (nv vertices, nf faces) and shared
 * control points cp (ncp x 3), nsub subjects each matched to its own target mesh
 * (DeterministicAtlas.cxx:99-280, AbstractAtlas.cxx:138-613). Target meshes are concatenated:
 * tgt_pts holds sum(nv_t) x 3 points, tgt_tris sum(nf_t) x 3 vertex indices local to each subject.
 * data_kind 0 = currents, 1 = varifold. Every stage runs as one launch over all subjects; all
 * device memory is allocated here. */
int gbk_atlas_create(gbk_ctx *ctx, long ncp, const double *cp, long nv, const double *tmpl_pts,
                     long nf, const int *tmpl_tris, int nsub, const long *nv_t,
                     const double *tgt_pts, const long *nf_t, const int *tgt_tris, int T,
                     double sigma_def, double sigma_data, double data_sigma2, int data_kind,
                     int heun, gbk_atlas **out);
/* mom: nsub x ncp x 3. loglik[3 + nsub] = {L, L_data, L_reg, L_0 .. L_{nsub-1}};
 * grad_mom (nsub x ncp x 3) = dL/dp_s; grad_cp (ncp x 3) = sum_s dL_s/dcp; grad_tmpl (nv x 3) =
 * sum_s -theta_s(0), the template vertex gradient. Any output may be NULL. Graph replay from the
 * third call, as gbk_registration_step. */
int gbk_atlas_step(gbk_atlas *atlas, const double *mom, double *loglik, double *grad_mom,
                   double *grad_cp, double *grad_tmpl);
int gbk_atlas_set_graph(gbk_atlas *atlas, int enable);
long long gbk_atlas_graph_launches(const gbk_atlas *atlas);
/* Smooths the template gradient by a Gaussian of this width over the template points
 * (AbstractAtlas::ConvolveGradTemplate, AbstractAtlas.cxx:724-748; the reference uses
 * smoothing-kernel-width-ratio x deformation kernel width, estimate_atlas.cxx:457); 0 (default)
 * returns the L2 gradient. */
int gbk_atlas_set_template_smoothing(gbk_atlas *atlas, double width);
/* 1 (default): gbk_atlas_optimize deforms the template of the previous SetFixedEffects call, as
 * the reference's AbstractAtlas::SetFixedEffects (AbstractAtlas.cxx:52-65) does, while the step and
 * the smoothing use the current template; 0: every evaluation deforms its own template. */
int gbk_atlas_set_lagged_template(gbk_atlas *atlas, int enable);
/* FastGradientAscent (FastGradientAscent.cxx:48-300) of the atlas over its control points
 * (optimize_cp), template points (optimize_template) and all subjects' momenta, on the device.
 * cp (ncp x 3), tmpl (nv x 3), mom (nsub x ncp x 3): start point in, final fixed effects out (host or
 * device). history: one [data, regularity] row per iteration (at most max_iterations + 1,
 * *iterations of them). info (10 doubles, optional): final steps (cp, template, momenta), tau,
 * freeze counter, squared gradient norms (cp, template as <L2, smoothed>, momenta), evaluations,
 * stop reason (0 max iterations, 1 line search, 2 tolerance). */
int gbk_atlas_optimize(gbk_atlas *atlas, double *cp, double *tmpl, double *mom, int optimize_cp,
                       int optimize_template, int max_iterations, double initial_step, int max_line_search,
                       double shrink, double expand, double tolerance, int nb_iter_freeze, double *history,
                       int *iterations, double *info);
void gbk_atlas_destroy(gbk_atlas *atlas);

/* ---- library-owned device arrays ------------------------------------------------------------ *
 * For callers that keep no device memory themselves but call repeatedly with the same inputs: the
 * C++ reference binding uploads a kernel object's sources and weights once and again only after
 * SetSources / SetWeights / SetKernelWidth set the object's m_Modified flag (AbstractKernel.h:85-115,
 * 172-185), where the legacy CUDA path copied them on every call (CUDAExactKernel.cxx:46-48).
 * gbk_buffer_data's device pointer can be passed to every entry point in place of a host array. */
typedef struct gbk_buffer gbk_buffer;
int gbk_buffer_create(gbk_ctx *ctx, gbk_buffer **out);
/* Copies `count` doubles from host memory into the buffer (growing it on the context's GPU) and
 * waits for the copy. Not while the context's stream is being captured. */
int gbk_buffer_upload(gbk_ctx *ctx, gbk_buffer *buf, const double *host, size_t count);
const double *gbk_buffer_data(const gbk_buffer *buf);
/* Number of uploads into the buffer so far (-1 for NULL). */
long long gbk_buffer_uploads(const gbk_buffer *buf);
/* Frees the device array (waits for the buffer's GPU) and the handle. */
void gbk_buffer_destroy(gbk_buffer *buf);

/* ---- tuning ------------------------------------------------------------------------------ */

/* The autotuner (no counterpart in the reference). A kernel-sum launch takes one of three paths --
 * caller order with one-float coordinates, caller order with adaptive two-float coordinates (the
 * automatic order below its size rule), or the spatial order -- and each path has a family of
 * compiled launch shapes with the same arithmetic (default, 2-way unroll, 4 targets per thread,
 * scalar lanes, 128-thread CTAs, the small shape, two-float default / small, bulk staging), so a
 * tuned choice changes the speed, never the accuracy. The tuning table maps (op, precision, d, dv,
 * log2 nx, log2 ny, path) to (shape, source splits); a call whose key is in the table uses it. A
 * context created while the environment variable GBK_TUNE_FILE names a file saved by gbk_tune_save
 * starts with that table. op is a GBK_OP_* up to GBK_OP_HESSIAN_ROWCOL (Convolve, the fused Convolve +
 * alpha-gradient, the alpha-gradient, varlin, ConvolveGradient(X, dim), the Hessians); dv one
 * compiled column width.
 *
 * Times every shape of the path such a call takes (with the context's order and staging policy)
 * with a range of split counts on synthetic uniform inputs of that size, and keeps the fastest. */
int gbk_autotune(gbk_ctx *ctx, int op, int d, int dv, long nx, long ny, double sigma);
/* The same on the caller's own arrays (host or device; alpha nx x dv for the alpha-gradient ops,
 * else may be NULL), through exactly the path the call with these arrays takes (sorts and pruning
 * included). variant, nsplit and ms (optional) receive the choice and its time per launch. */
int gbk_autotune_data(gbk_ctx *ctx, int op, int d, int dv, const double *x, long nx, const double *y,
                      const double *w, long ny, double sigma, const double *alpha, int *variant, int *nsplit,
                      double *ms);
/* Saves / loads the tuned table as JSON lines (entries for shapes this build does not compile are
 * skipped on load). */
int gbk_tune_save(const gbk_ctx *ctx, const char *path);
int gbk_tune_load(gbk_ctx *ctx, const char *path);
/* Forces the number of source splits (0 = automatic) -- for tests and tuning. */
int gbk_set_split(gbk_ctx *ctx, int nsplit);
/* Fault injection for tests: from now on every growth of one of the context's device buffers
 * beyond `bytes` fails with GBK_ERR_ALLOC as if cudaMalloc had failed (0 = no limit). The context
 * stays usable: lift the limit and the same call succeeds. */
int gbk_set_alloc_limit(gbk_ctx *ctx, size_t bytes);
/* Fault injection for tests: from now on every device allocation passed to the context is treated as
 * memory of GPU `device` (-1 = off), so the refusal of another GPU's memory (GBK_ERR_ARG, nothing
 * queued: the kernels cannot read it without peer access) can be exercised on a one-GPU machine. */
int gbk_inject_pointer_device(gbk_ctx *ctx, int device);

#ifdef __cplusplus
}
#endif

#endif /* GBK_H */
