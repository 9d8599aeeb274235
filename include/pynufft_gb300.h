/*
 * pynufft_gb300 — C ABI of the GB300 (sm_103a) min-max NUFFT.
 *
 * This is the drop-in boundary for the reference class `NUFFT`
 * (pynufft 2025.2.1, nufft/__init__.py:496-738).  Every entry point takes
 * plain pointers and sizes, returns an `int` status (NUFFT_OK == 0) and runs
 * asynchronously on the caller's CUDA stream (`stream` is a cudaStream_t
 * passed as void*; NULL means the legacy default stream).
 *
 * Array conventions (all complex data is interleaved float32 pairs,
 * i.e. numpy complex64 / C float _Complex):
 *   om : M x ndim float64, C order, normalised frequencies in radians
 *        (any range; wrapped modulo the oversampled grid).
 *   x  : Nd + (batch,) image, C order, batch (coil) fastest.
 *   k  : Kd + (batch,) oversampled k-space grid, C order, batch fastest.
 *   y  : (M, batch) non-uniform samples, batch fastest.
 *   With ninst > 1 independent instances, x, k and y gain a leading instance
 *   axis for x and k ((ninst,) + Nd + (batch,)) and y is the concatenation of
 *   the instances' samples in instance order.
 * Device pointers must be 16-byte aligned (true of every cudaMalloc/torch
 * allocation).  The plan owns its tables and workspace; inputs are never
 * written; outputs are fully overwritten.  Calls on one plan must be
 * serialised (one stream at a time); distinct plans are independent.
 */
#ifndef PYNUFFT_GB300_H
#define PYNUFFT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the Python layer maps them to the reference's exception
 *      types: TypeError/KeyError for plan arguments, ValueError, RuntimeError) */
#define NUFFT_OK                 0
#define NUFFT_EINVAL             1  /* bad argument, shape or size            */
#define NUFFT_EOM_NONFINITE      2  /* om holds NaN or Inf                    */
#define NUFFT_ENOMEM             3  /* device allocation failed               */
#define NUFFT_ECUDA              4  /* CUDA runtime error                     */
#define NUFFT_ECUFFT             5  /* cuFFT error                            */
#define NUFFT_ENOPOINTS          6  /* nufft_set_points has not been called   */
#define NUFFT_ECG_BREAKDOWN      7  /* CG: p^H A p <= 0 or not finite         */
#define NUFFT_EUNSUPPORTED       8  /* valid request this build does not do   */
#define NUFFT_ETIMEOUT           9  /* a kernel's bounded wait ran out        */

/* ---- plan flags */
#define NUFFT_FLAG_DETERMINISTIC 1  /* bitwise-reproducible gridding (y2k)    */
#define NUFFT_FLAG_OWN_FFT       2  /* the library's own pruned power-of-two
                                       FFT passes instead of cuFFT, where the
                                       plan allows them (see
                                       nufft_plan_transform_kind)             */
#define NUFFT_FLAG_CUFFT         4  /* cuFFT even where the own passes would
                                       be chosen without a flag               */

typedef struct nufft_plan_s* nufft_plan_t;

/* Human-readable text of the last error raised on the calling thread. */
const char* nufft_last_error(void);

/* Library version string, e.g. "pynufft_gb300 0.1.0 (sm_103a)". */
const char* nufft_version(void);

/* Plan-time numerics of one axis, host only (no GPU needed).  Replaces
 * helper.nufft_alpha_kb_fit / nufft_scale1 / nufft_T
 * (src/_helper/helper.py:910-958, 1015-1036, 1060-1083).
 *   alpha_in  : NULL to fit the cosine-series coefficients here, or the L_in+1
 *               coefficients to use (e.g. the reference's own float32 fit)
 *   alpha_out : float[16]  coefficients used (L+1 valid, L <= 14)
 *   L_out     : series order L
 *   sn_out    : double[N]  real scaling factor of this axis
 *   T_out     : double[J*J] pinv(CSSC), row major                     */
int nufft_axis_params(int N, int J, int K, const float* alpha_in, int L_in,
                      float* alpha_out, int* L_out, double* sn_out, double* T_out);

/* Create a plan.  Replaces NUFFT.plan(om, Nd, Kd, Jd[, batch])
 * (nufft/__init__.py:552-596 -> _plan_cpu, nufft/_nufft_class_methods_cpu.py:27-124;
 *  batch semantics of linalg/nufft_hsa.py:152-242).  ndim in 1..3,
 * Jd[d] <= 16, Jd[d] <= Kd[d], Nd[d] <= Kd[d]; batch >= 1; ninst >= 1.
 * Allocates the plan's device workspace on the current device. */
int nufft_plan_create(int ndim, const int* Nd, const int* Kd, const int* Jd,
                      int batch, int ninst, int flags, nufft_plan_t* plan_out);

/* Replace the cosine-series coefficients of one axis (L+1 values, L <= 14)
 * and re-derive its scaling factor and interpolator normal matrix.  Call
 * before nufft_set_points.  The reference fits these coefficients with a
 * complex64 least-squares solve (helper.py:949-958); a caller that has that
 * fit reproduces the reference's interpolator exactly. */
int nufft_plan_set_alpha(nufft_plan_t plan, int axis, const float* alpha, int L);

/* Set the non-uniform points: counts[i] points of instance i, om holding
 * sum(counts) rows of ndim float64 (instances concatenated).  om may be a
 * host or a device pointer (om_on_device).  Builds the bin-sorted per-axis
 * interpolation tables on the device (the GPU counterpart of the CSR build in
 * helper.plan, src/_helper/helper.py:736-786).  Synchronises `stream` once. */
int nufft_set_points(nufft_plan_t plan, const int64_t* counts, const double* om,
                     int om_on_device, void* stream);

int nufft_plan_destroy(nufft_plan_t plan);

/* Per-plan tuning: bin shape (cells per axis) and the largest number of
 * points one thread block takes from a bin.  Takes effect at the next
 * nufft_set_points.  Zero entries keep the default. */
int nufft_plan_set_bins(nufft_plan_t plan, const int* bin_shape, int max_sub_points);

/* Lane mappings of the interpolation (k2y) and gridding (y2k) kernels for
 * plans with fewer than 8 coils (plans with 8 or more always split coils
 * across lanes).  0 keeps the default: k2y gathers from a shared tile with two
 * threads per point when sub-problems average 8 or more points (else one
 * thread per point straight from the grid); y2k uses one thread per point
 * (two for single-coil 2D/3D plans).  Used by the autotuner; results are
 * identical up to float32 rounding order. */
#define NUFFT_K2Y_COIL  0   /* (internal) lanes over coils                    */
#define NUFFT_K2Y_ZTEAM 1   /* J lanes per point along the innermost axis     */
#define NUFFT_K2Y_POINT 2   /* one thread per point                           */
#define NUFFT_K2Y_TILE  3   /* bin footprint staged in shared memory + z-teams */
#define NUFFT_K2Y_TILE_POINT 4  /* bin footprint in shared memory + 1-2 threads
                                   per point                                   */
#define NUFFT_Y2K_COIL  0   /* (internal) lanes over coils                    */
#define NUFFT_Y2K_ZTEAM 1   /* J lanes per point along the innermost axis     */
#define NUFFT_Y2K_POINT 2   /* one thread per point                           */
#define NUFFT_Y2K_GLOBAL 3  /* z-teams adding floats straight into the grid
                               (no shared tile; not in deterministic mode)    */
int nufft_plan_set_methods(nufft_plan_t plan, int k2y_method, int y2k_method);

/* Optional timing of the interpolation (k2y) and gridding (y2k) kernels:
 * with period n > 0, the 1st, (n+1)-th, (2n+1)-th ... k2y and y2k kernel
 * launches of this plan are each bracketed by a pair of CUDA events on their
 * own stream (skipped while the stream is being captured into a graph);
 * period 0 turns timing off, a negative period is NUFFT_EINVAL.
 * nufft_plan_kernel_times waits for the recorded events and returns the
 * summed time (ms) and the number of timed launches of each, then forgets
 * them.  Setting the period also forgets them.  No counterpart in the
 * reference. */
int nufft_plan_kernel_timing(nufft_plan_t plan, int period);
int nufft_plan_kernel_times(nufft_plan_t plan, double* k2y_ms, int* k2y_launches,
                            double* y2k_ms, int* y2k_launches);

/* Device address of page-locked host memory that is mapped into the device
 * address space (cudaHostAlloc / pinned tensors on unified-addressing
 * systems), for passing a host image straight to nufft_forward (read) or
 * nufft_adjoint (written) instead of copying it: the image kernels then access
 * host memory over the host link.  NUFFT_EINVAL if `host` is not such memory.
 * No counterpart in the reference. */
int nufft_mapped_pointer(const void* host, void** dev_out);

/* Self-test of the bounded wait the bulk-copy kernels use: one block waits
 * `polls` polls (1 .. 2^22) on an mbarrier whose bytes never arrive and
 * *timed_out receives 1 if the wait ran out (the expected answer).  Faults and
 * hangs nothing; synchronises the device.  No counterpart in the reference. */
int nufft_selftest_bounded_wait(int polls, int* timed_out);

/* Synchronise `stream` and report whether any kernel of this plan gave up a
 * bounded wait for its asynchronous (bulk-copy) loads since the last check:
 * NUFFT_ETIMEOUT if so (that launch's output is incomplete; the flag is
 * cleared), else NUFFT_OK.  No counterpart in the reference. */
int nufft_plan_check(nufft_plan_t plan, void* stream);

/* Query plan geometry: total points, number of gridding sub-problems and
 * bytes of device memory the plan holds. */
int nufft_plan_info(nufft_plan_t plan, int64_t* M_total, int64_t* n_subproblems,
                    int64_t* device_bytes);

/* Which transform the image <-> spectrum stages of this plan run:
 * NUFFT_FFT_CUFFT (cuFFT over the whole padded grid), NUFFT_FFT_CUFFT_PRUNED
 * (cuFFT on the slabs the padding leaves nonzero), NUFFT_FFT_OWN_PRUNED (the
 * library's pruned power-of-two passes: one coil, one instance, 2D/3D,
 * Nd[0] < Kd[0], every Kd a power of two in 16..4096, and either
 * NUFFT_FLAG_OWN_FFT set or -- without NUFFT_FLAG_CUFFT -- every Kd 256 and
 * every Nd 128 or 256, where the passes' specialised 256-point kernels beat
 * cuFFT), NUFFT_FFT_OWN_COILS (the library's coil-batched passes on the
 * coil-fastest layout, pruned and with the pad / crop / scaling fused: 2D
 * or 3D, a multiple of 8 coils, one instance, every Kd in {128, 160, 192,
 * 256, 320, 384, 512, 640}, unless NUFFT_FLAG_CUFFT is set).  No
 * counterpart in the reference (numpy fftn / ifftn). */
#define NUFFT_FFT_CUFFT        0
#define NUFFT_FFT_CUFFT_PRUNED 1
#define NUFFT_FFT_OWN_PRUNED   2
#define NUFFT_FFT_OWN_COILS    3
int nufft_plan_transform_kind(nufft_plan_t plan, int* kind);

/* ---- the six stages (nufft/__init__.py:658-692) ---------------------------
 * x2xx  (_x2xx_cpu  :224-230)  xx = x * sn                       Nd -> Nd
 * xx2k  (_xx2k_cpu  :232-249)  k  = fftn(zero-pad(xx))           Nd -> Kd
 * k2y   (_k2y_cpu   :273-288)  y  = interpolate(k)               Kd -> M
 * y2k   (_y2k_cpu   :290-314)  k  = grid(y) (adjoint of k2y)     M  -> Kd
 * k2xx  (_k2xx_cpu  :316-329)  xx = crop(ifftn(k)), 1/prod(Kd)   Kd -> Nd
 * xx2x  (_xx2x_cpu  :346-351)  x  = xx * sn                      Nd -> Nd */
int nufft_x2xx(nufft_plan_t plan, const void* x, void* xx, void* stream);
int nufft_xx2k(nufft_plan_t plan, const void* xx, void* k, void* stream);
int nufft_k2y(nufft_plan_t plan, const void* k, void* y, void* stream);
int nufft_y2k(nufft_plan_t plan, const void* y, void* k, void* stream);
int nufft_k2xx(nufft_plan_t plan, const void* k, void* xx, void* stream);
int nufft_xx2x(nufft_plan_t plan, const void* xx, void* x, void* stream);

/* forward (_forward_cpu :168-179): y = k2y(xx2k(x2xx(x))), sn-scale and
 * zero-pad fused into one pass ahead of the FFT. */
int nufft_forward(nufft_plan_t plan, const void* x, void* y, void* stream);
/* adjoint (_adjoint_cpu :181-193): x = xx2x(k2xx(y2k(y))), crop, 1/prod(Kd)
 * and sn-scale fused into one pass after the inverse FFT. */
int nufft_adjoint(nufft_plan_t plan, const void* y, void* x, void* stream);
/* selfadjoint (_selfadjoint_cpu :201-214) = adjoint(forward(x)). */
int nufft_selfadjoint(nufft_plan_t plan, const void* x, void* x_out, void* stream);
/* k2y2k (_k2y2k_cpu :353-362) = y2k(k2y(k)). */
int nufft_k2y2k(nufft_plan_t plan, const void* k, void* k_out, void* stream);

/* solve(y, 'cg', maxiter) (linalg/solve_cpu.py:256-288): conjugate gradients
 * on the k-space normal operator y2k.k2y with x0 = 0 and scipy's stopping
 * rule ||r|| < max(atol, rtol*||b||), then x = k2xx(k) / sn.  maxiter < 0
 * means scipy's default of 10 * prod(Kd).  The set-up and chunks of
 * up to 32 iterations run as captured CUDA graphs with device-side scalars
 * (FP64 dots and norms); a solve longer than one chunk checks convergence on
 * the host between chunks.  Each coil/instance is an independent system.
 * iters_out (host pointer, may be NULL) receives the most iterations any
 * system ran; reading it synchronises `stream`. */
int nufft_solve_cg(nufft_plan_t plan, const void* y, void* x, int maxiter,
                   double rtol, double atol, int* iters_out, void* stream);

/* solve(y, 'L1TVOLS', maxiter, rho) (L1TVOLS, linalg/solve_cpu.py:42-163):
 * L1 total-variation regularised least squares by split Bregman with
 * mu = 1 and lambda = rho, maxiter outer iterations, x0 = 0; k-space
 * preconditioner mu |xx2k(adjoint(1))| - lambda FFT(Laplacian).  Single-coil,
 * single-instance plans.  Allocates its work vectors stream-ordered
 * (cudaMallocAsync) and does not synchronise `stream`. */
int nufft_solve_l1tvols(nufft_plan_t plan, const void* y, void* x, int maxiter, double rho,
                        void* stream);

/* SENSE coil operators of the deprecated reference class
 * (linalg/nufft_cpu.py:163-203).  nufft_set_sense copies coil maps of shape
 * Nd + (batch,) (complex64, coil fastest; host or device pointer; NULL
 * forgets them).  forward_one2many: single-coil image x (Nd) -> y (M, batch)
 * = forward(x * maps), the map multiply fused into the sn/zero-pad pass.
 * adjoint_many2one: y (M, batch) -> x (Nd) = mean over coils of
 * conj(maps) * adjoint(y), fused into the crop pass.  Single-instance plans. */
int nufft_set_sense(nufft_plan_t plan, const void* maps, int maps_on_device, void* stream);
int nufft_forward_one2many(nufft_plan_t plan, const void* x, void* y, void* stream);
int nufft_adjoint_many2one(nufft_plan_t plan, const void* y, void* x, void* stream);

/* Gridding (y2k) with the 64-bit fixed-point accumulation of the
 * deterministic mode, for callers that cannot allocate device memory while
 * they run: applications that hand all GPU memory to their own pool up front
 * (where a stray cudaMalloc can fail or fragment the pool) and
 * latency-critical code that cannot afford cudaMalloc/cudaFree (cudaFree
 * synchronises the whole device).  No counterpart in the reference.
 * It allocates nothing: its accumulators live in a scratch array compiled
 * into the library (NUFFT_STATIC_SCRATCH_CELLS grid cells, 16 MiB, held on
 * every GPU that loads the library until the process exits), and plans whose
 * ninst * prod(Kd) * batch exceeds that size are rejected with NUFFT_EINVAL.
 * The first call on a device looks the scratch address up for that device
 * (the device must be current); make that first call before any stream
 * capture.  All calls share the scratch, which keeps the last call's
 * contents (each call clears it first): calls that overlap on the GPU, on
 * different streams or threads, race.  Works on any plan; the result equals
 * nufft_y2k on a plan created with NUFFT_FLAG_DETERMINISTIC, bit for bit:
 * every contribution summed exactly, or, on plans of 8 or more coils that
 * grid by tile rows, per-row float sums in a fixed order combined exactly
 * (those plans also use their coil-major spectrum buffer, allocated with the
 * plan, before one transpose into k, unless they run the coil-batched FFT
 * passes: then the rows go straight into k). */
#define NUFFT_STATIC_SCRATCH_CELLS (1u << 20)
int nufft_y2k_exact_static(nufft_plan_t plan, const void* y, void* k, void* stream);

/* Trajectory gradient support: dy[m, d] = sum_n x_n (-i (n_d - N_d/2))
 * e^{-i om_m.(n - N/2)}, evaluated with the plan's interpolator as the
 * forward transform of (-i (n_d - N_d/2)) x.  dy is ndim consecutive (M,batch)
 * blocks. */
int nufft_forward_dom(nufft_plan_t plan, const void* x, void* dy, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PYNUFFT_GB300_H */
