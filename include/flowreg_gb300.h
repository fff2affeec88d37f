/*
 * flowreg_gb300.h -- C ABI of the GB300 (sm_103a) backend for pyflowreg's
 * variational optical-flow path.
 *
 * Plain C: device pointers are `float*` to CUDA device memory, streams are
 * passed as `void*` (a cudaStream_t; NULL = legacy default stream).  Arrays
 * use numpy's C order unless stated.  All work is enqueued on the stream;
 * nothing synchronises the host except where a function says so.  Functions
 * return FRG_OK or an error code; frg_last_error() then describes it
 * (thread-local).
 *
 * Reference interfaces (pyflowreg, paths relative to src/pyflowreg/):
 *   frg_plan_create / frg_set_reference / frg_get_displacement
 *       replace get_displacement(fixed, moving, ...)     core/optical_flow.py:773-929
 *       called once per frame by the executors          motion_correction/parallelization/sequential.py:141-145
 *   frg_level_solve  replaces compute_flow via the level_solver_backend seam
 *                                                        core/optical_flow.py:348-411, 584-606
 *                                                        core/level_solver.py:158-369
 *   frg_level_solve_f64 replaces compute_flow / compute_flow_gnc at that seam
 *                    in float64                          core/level_solver.py:158-555
 *   frg_imregister   replaces imregister_wrapper          core/warping.py:160-234
 *   frg_resize       replaces imresize_fused_gauss_cubic  util/resize_util.py:232-254
 *   frg_motion_tensor replaces get_motion_tensor_gc/_gray core/optical_flow.py:73-228
 *   frg_median5      replaces median_filter(size=(5,5), mode="mirror")
 *                                                        core/optical_flow.py:607-609
 */
#ifndef FLOWREG_GB300_H
#define FLOWREG_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FRG_OK 0
#define FRG_EINVAL 1          /* bad argument (shape, pointer, option) */
#define FRG_ENOMEM 2          /* device or host allocation failed */
#define FRG_ECUDA 3           /* a CUDA call failed */
#define FRG_EUNSUPPORTED 4    /* option not implemented by this backend */
#define FRG_ECALLBACK 5       /* a host callback reported failure */

#define FRG_MAX_CHANNELS 8
#define FRG_MAX_GNC_STAGES 16
#define FRG_ABI_VERSION 2

/* Optical-flow options, the subset of OFOptions.to_dict()
 * (motion_correction/OF_options.py:1084-1101) that get_displacement uses. */
typedef struct frg_params {
    double alpha_x, alpha_y;              /* smoothness weights (OFOptions.alpha) */
    double eta;                           /* pyramid factor, 0 < eta <= 1 */
    int levels;                           /* maximum number of pyramid levels */
    int min_level;                        /* finest level computed (effective value, >= 0) */
    int iterations;                       /* SOR iterations per level */
    int update_lag;                       /* iterations between nonlinearity updates */
    double a_smooth;                      /* smoothness Charbonnier exponent (1.0 only) */
    double a_data[FRG_MAX_CHANNELS];      /* data-term exponent per channel */
    int const_assumption;                 /* 0: gradient constancy "gc", 1: gray value "gray", 2: census "cs" */
    double omega;                         /* SOR relaxation factor (reference: 1.95) */
    int precision;                        /* FRG_FP32 (default) or FRG_FP64_REFERENCE */
    /* Graduated non-convexity (get_displacement's gnc_schedule / warping_steps,
     * core/optical_flow.py:620-770, 887-929): gnc_stages = 0 runs the plain
     * pyramid; otherwise gnc_stages (2..FRG_MAX_GNC_STAGES) betas, nondecreasing
     * from 0 to 1, each stage re-running the pyramid from the previous stage's
     * flow with warping_steps warp / relinearise rounds per level. */
    int gnc_stages;
    double gnc_schedule[FRG_MAX_GNC_STAGES];
    int warping_steps;
} frg_params;

/* precision: FRG_FP32 is the fast path (float32 arithmetic, folded SOR
 * coefficients, shared-memory wavefront).  FRG_FP64_REFERENCE computes in
 * the reference's own precision and operation order (float32 images and
 * resize products, float64 accumulators, tensors and solver) with the same
 * exact update order; it is the parity mode.  Its plans are driven with
 * frg_get_displacement_f64. */
#define FRG_FP32 0
#define FRG_FP64_REFERENCE 1

typedef struct frg_plan frg_plan;

int frg_version(void);
const char* frg_last_error(void);

/* Host-only helpers (no GPU needed), exposing the plan's schedule for tests:
 *   frg_schedule: pyramid levels, coarsest first, as _solve_displacement_stage
 *     iterates them (core/optical_flow.py:494-518, 572-577): sizes and the
 *     scaled alpha.  Returns the number of levels (writes at most max_levels),
 *     or a negative error code.
 *   frg_resize_tables: tap indices/weights (out_len, P) of the fused
 *     Gauss-cubic resize (util/resize_util.py:194-229).  Returns P; writes
 *     nothing if P > max_taps.
 *   frg_iteration_passes: how the SOR iterations are cut into wavefront
 *     passes at the nonlinearity ticks ((t+1) % update_lag == 0,
 *     core/level_solver.py:230).  G[i] iterations per pass; fold_mode[i] = -1
 *     when the pass reuses the previous coefficients, else bit 0 = first
 *     pass (du = dv = 0), bit 1 = psi recomputed.  Returns the pass count. */
int frg_schedule(const frg_params* params, int height, int width, int max_levels, int* h, int* w,
                 double* alpha_x, double* alpha_y);
int frg_resize_tables(int in_len, int out_len, double sigma, int max_taps, int* idx, float* wt);
int frg_iteration_passes(int iterations, int update_lag, int max_passes, int* G, int* fold_mode);

/* A plan fixes the frame shape (height x width x channels), the options and
 * the largest batch.  It owns all device memory it needs (tables, the
 * reference pyramid and the per-batch workspace); frg_plan_device_bytes
 * reports the total.  A plan is not thread-safe: use one per stream. */
int frg_plan_create(const frg_params* params, int height, int width, int channels, int max_frames,
                    frg_plan** out);
void frg_plan_destroy(frg_plan* plan);
size_t frg_plan_device_bytes(const frg_plan* plan);
int frg_plan_num_levels(const frg_plan* plan);
/* level 0 is the coarsest level actually solved */
int frg_plan_level_info(const frg_plan* plan, int level, int* h, int* w, double* alpha_x,
                        double* alpha_y);

/* Replaces the resize tap tables of one level (host pointers, copied):
 * kind 0 resizes the full-size frame to the level, kind 1 the previous
 * level's flow (the full-size uv_init at the top level) to the level.
 * ix/wx are (w, taps), iy/wy (h, taps), int32 / float32, as
 * _precompute_fused_gauss_cubic returns them (util/resize_util.py:216-229).
 * The library builds equivalent tables itself; the reference builds them with
 * numpy, whose float32 exp differs in the last bit between CPU builds, and the
 * solver amplifies such differences, so a host that wants the reference's
 * tables bit for bit passes them here.  taps must equal the plan's. */
int frg_plan_set_level_tables(frg_plan* plan, int level, int kind, int taps, const int* ix, const float* wx,
                              const int* iy, const float* wy);

/* Tuning of one level's fused SOR launches (no reference counterpart; the
 * results do not change, only the launch shape): sor_G iterations per
 * wavefront pass (0: the most the shared-memory ring holds, reported as gmax)
 * and sor_threads threads per CTA (0: the level's rows rounded up to 32,
 * reported as rows; else a multiple of 32 in [rows, 1024]).  Levels that do
 * not use the fused kernel report gmax 0 and accept only (0, 0).  Levels of an
 * FP64 plan that run the float64 chained SOR take sor_G = 0 and sor_threads =
 * the rows per CTA strip: 64, 128 or 256 with at most 8 strips, or 0 to choose
 * from each call's batch size (the tallest strips that still give every SM a
 * CTA). */
int frg_plan_set_level_tuning(frg_plan* plan, int level, int sor_G, int sor_threads);
int frg_plan_level_tuning(const frg_plan* plan, int level, int* sor_G, int* sor_threads, int* gmax, int* rows);
/* Which fused SOR kernel a level runs: 0 the diagonal ring in shared memory
 * (any level up to 1024 rows; sor_threads applies), 1 one thread per row with
 * the state in registers (levels up to 512 rows; sor_G applies, sor_threads
 * does not).  Both give the same bits.  n_variants: how many serve the level
 * (0 when it does not use a fused kernel). */
int frg_plan_set_level_variant(frg_plan* plan, int level, int variant);

/* A host level solver that the float64 path calls in place of its own SOR:
 * the `level_solver_backend` of get_displacement (core/optical_flow.py:579-606).
 * It is called once per pyramid level and frame, on the thread inside
 * frg_get_displacement_f64, after the stream has finished the level's motion
 * tensor.  m = h + 2 and n = w + 2 (the padded level); J (6, K, m*n: J11, J22,
 * J33, J12, J13, J23 with a zero ring), W (K, m*n, zero ring), u, v (m*n, edge
 * ring) and du, dv (m*n) are float64 device pointers; alpha_x, alpha_y are the
 * level's smoothness weights and hx, hy its column and row spacings.  The
 * callback writes du, dv (complete on the device when it returns) and returns
 * 0, or nonzero to end the call with FRG_ECALLBACK. */
typedef int (*frg_level_solver_fn)(void* user, int level, int frame, int m, int n, int K, const double* J,
                                   const double* W, const double* u, const double* v, double alpha_x,
                                   double alpha_y, double hx, double hy, double* du, double* dv);
/* Installs (fn non-null) or removes (fn null) the host level solver of a
 * float64 plan without GNC stages; FRG_EUNSUPPORTED for other plans. */
int frg_plan_set_level_solver(frg_plan* plan, frg_level_solver_fn fn, void* user);
int frg_plan_level_variant(const frg_plan* plan, int level, int* variant, int* n_variants);

/* Reference (fixed) frame (height, width, channels) float32 and the per-pixel
 * channel weight (height, width, channels) float32 (NULL: 1/channels), as
 * get_displacement receives them after its input normalisation
 * (core/optical_flow.py:846-879).  Builds the reference and weight pyramids. */
int frg_set_reference(frg_plan* plan, const float* fixed, const float* weight, void* stream);

/* Flow of n_frames moving frames (n_frames, height, width, channels) against
 * the reference: flow_out (n_frames, height, width, 2) with [..., 0] = u
 * (columns) and [..., 1] = v (rows).  uv_init (height, width, 2) or NULL is
 * the initial field shared by all frames (the executors' w_init). */
int frg_get_displacement(frg_plan* plan, int n_frames, const float* moving, const float* uv_init,
                         float* flow_out, void* stream);

/* The same for a plan created with precision = FRG_FP64_REFERENCE; flow_out
 * (n_frames, height, width, 2) is float64 like the reference's return value. */
int frg_get_displacement_f64(frg_plan* plan, int n_frames, const float* moving, const float* uv_init,
                             double* flow_out, void* stream);

/* Measurement hooks (no reference counterpart; pyflowreg has no tracing,
 * only wall-clock prints in compensate_recording.py:770-890):
 *   frg_launch_count: kernels launched by this library in this process.
 *   frg_plan_set_profiling: when enabled, every SOR launch of the plan is
 *     bracketed by CUDA events on its stream (counters reset on each call).
 *   frg_plan_profile: waits for those events and returns the number of SOR
 *     launches, their summed device time (ms) and their algorithmic bytes
 *     (36 B per interior pixel per pipelined iteration). */
long long frg_launch_count(void);
int frg_plan_set_profiling(frg_plan* plan, int enable);
int frg_plan_profile(frg_plan* plan, long long* sor_launches, double* sor_ms, double* sor_bytes);

/* Backward warp of frames (n_frames, height, width, channels) by flow
 * (n_frames, height, width, 2); out-of-bounds pixels take reference
 * (height, width, channels).  cubic = 1 bicubic, 0 bilinear. */
int frg_imregister(int n_frames, int height, int width, int channels, const float* frames,
                   const float* flow, const float* reference, int cubic, float* out, void* stream);

/* One pyramid level of the lagged-nonlinearity SOR in the reference's exact
 * (column-major lexicographic) update order.  J is six arrays (m, n, K) back
 * to back in the order J11, J22, J33, J12, J13, J23; weight (m, n, K); u, v,
 * du, dv (m, n); m, n include the one-pixel ring.  hx scales column
 * differences, hy row differences.  du/dv rings are set to the adjacent
 * interior values.  Allocates its scratch with cudaMallocAsync on `stream`. */
int frg_level_solve(int m, int n, int K, const float* J, const float* weight, const float* u,
                    const float* v, double alpha_x, double alpha_y, int iterations, int update_lag,
                    const double* a_data, double a_smooth, double hx, double hy, double omega,
                    float* du, float* dv, void* stream);

/* frg_level_solve for callers that cannot allocate device memory -- code
 * running while a CUDA graph is being captured (allocation calls are not
 * allowed then), or a host whose device memory is reserved up front by
 * another framework's pool, where a cudaMalloc would fail or would
 * synchronise the device.  It has no counterpart in pyflowreg.
 *
 * Same arguments and results as frg_level_solve; it allocates nothing.  Its
 * scratch is a fixed 8 MiB device array inside the library (every GPU that
 * loads the library holds it until the process exits), so the level must fit
 * in it: (7*K + 9) * (h + w - 1) * ceil32(h) floats, h = m - 2, w = n - 2,
 * ceil32 = rounded up to a multiple of 32 (for K = 2 about 200 x 200 pixels;
 * frg_level_solve_noalloc_capacity() returns the byte size).  Larger levels
 * are rejected with FRG_EINVAL.
 *
 * The first call on each device looks up the array's device address (with
 * that device current); make that first call before any stream capture.
 * All calls share the one array: calls whose work overlaps on the GPU (on
 * different streams, or from different threads) race and corrupt each
 * other's results; serialise them.  Each call writes every scratch element
 * it reads, so no clearing between calls is needed. */
int frg_level_solve_noalloc(int m, int n, int K, const float* J, const float* weight, const float* u,
                            const float* v, double alpha_x, double alpha_y, int iterations,
                            int update_lag, const double* a_data, double a_smooth, double hx, double hy,
                            double omega, float* du, float* dv, void* stream);
size_t frg_level_solve_noalloc_capacity(void);

/* The level solver in the reference's own precision and operation order, for
 * the level_solver_backend seam fed with the reference's float64 arrays
 * (core/optical_flow.py:348-411): compute_flow (core/level_solver.py:158-369)
 * when gnc_beta < 0, compute_flow_gnc (core/level_solver.py:372-555) with
 * that stage weight when gnc_beta is in [0, 1]; any a_smooth > 0.  Layouts as
 * frg_level_solve, all arrays double on the device; du, dv receive the whole
 * (m, n) result, their rings as set_boundary_2d left them at the start of the
 * last iteration.  Allocates its scratch with cudaMallocAsync on `stream`. */
int frg_level_solve_f64(int m, int n, int K, const double* J, const double* weight, const double* u,
                        const double* v, double alpha_x, double alpha_y, int iterations, int update_lag,
                        const double* a_data, double a_smooth, double hx, double hy, double omega,
                        double gnc_beta, double* du, double* dv, void* stream);

/* Fused Gauss-cubic resize of n_planes planes (n_planes, ih, iw) to
 * (n_planes, oh, ow), sigma = 0.6 / min(oh/ih, ow/iw) when that is < 1. */
int frg_resize(int n_planes, int ih, int iw, const float* src, int oh, int ow, float* dst,
               void* stream);

/* Motion tensor of one channel: f1, f2 (h, w); out six planes (h+2, w+2)
 * back to back (J11, J22, J33, J12, J13, J23) with a zero ring.
 * gray = 0: gradient constancy, 1: gray-value constancy. */
int frg_motion_tensor(int h, int w, const float* f1, const float* f2, double hy, double hx, int gray,
                      float* out, void* stream);

/* 5x5 median with mirror boundary of one plane (h, w), h, w >= 3. */
int frg_median5(int h, int w, const float* src, float* dst, void* stream);
/* The same in float64, as the reference filters du and dv (float64 arrays):
 * the selection the float64 level loop uses, exact (ties included). */
int frg_median5_f64(int h, int w, const double* src, double* dst, void* stream);

/* out[i] = x[i]^b (n doubles, device memory) by the power function of the
 * float64 solver's data-term nonlinearity psi = a (E + 1e-5)^(a - 1)
 * (core/level_solver.py:247, `(val + 0.00001) ** (a_data[k] - 1.0)`): for
 * |b| <= 1 a table of 2^(e b) c^b built for b (on the host, per call) with a
 * binomial series, else a table-driven log2 / exp2; within a few ulp of the
 * correctly rounded power for positive normal x, pow's results elsewhere.
 * Exported so that its accuracy can be tested on its own. */
int frg_pow_f64(long long n, const double* x, double b, double* out, void* stream);

/* Page-locks (cudaHostRegister, default flags) or releases host memory that
 * asynchronous device-to-host copies of flows write into: the batch call's
 * output array, so that the last parts of a batch are read back by one copy
 * each instead of through a pinned staging buffer.  Host-side I/O of the batch
 * form (motion_correction/parallelization/base.py:76-110 hands the executor
 * host arrays); it replaces no reference function.  A refused registration
 * returns FRG_ECUDA (frg_last_error says why) and leaves no pending CUDA error
 * behind for later launches. */
int frg_host_register(void* ptr, long long bytes);
int frg_host_unregister(void* ptr);

/* Preprocessing of frames before the flow, as compensate_recording does it
 * (motion_correction/compensate_recording.py:521-561, normalize and
 * apply_gaussian_filter in util/image_processing.py:12-165): out =
 * gaussian(normalise(raw)) with normalise(x) = (x - lo[k]) / den[k] and a
 * separable Gaussian in axis order time, rows, columns, scipy's "reflect"
 * mode and scipy's symmetric correlation order.  raw, out (n_frames, height,
 * width, channels) float32 on the device; lo, den host arrays (channels);
 * rt, ry, rx host arrays of the radius per channel; wt, wy, wx device
 * arrays of taps w[0..r_k] per channel, stored with stride (max_k r_k + 1);
 * f32_norm: normalise in float32 (numpy's result for float32 frames and
 * reference), else float64; f32_storage: keep the normalised values and each
 * pass's output in float32 (joint normalisation of float32 data), else
 * float64 (per-channel normalisation writes into a float64 array); tmp holds
 * n_frames * channels * height * width values of the storage type. */
int frg_preprocess(int n_frames, int height, int width, int channels, const float* raw, const double* lo,
                   const double* den, const double* wt, const int* rt, const double* wy, const int* ry,
                   const double* wx, const int* rx, int f32_norm, int f32_storage, void* tmp, float* out, void* stream);
/* frg_preprocess for float64 frames (the raw reference is held in float64,
 * motion_correction/compensate_recording.py:491-498): numpy then normalises
 * in float64, so there is no f32_norm argument; f32_storage must be 0. */
int frg_preprocess_f64(int n_frames, int height, int width, int channels, const double* raw, const double* lo,
                       const double* den, const double* wt, const int* rt, const double* wy, const int* ry,
                       const double* wx, const int* rx, int f32_storage, void* tmp, float* out, void* stream);

/* Post-registration pass over flows (n_frames, height, width, 2) float32:
 * valid (n_frames, height, width) uint8 0/255 masks of the backward warp
 * (core/warping.py:14-60, compute_batch_valid_masks; may be NULL) and stats
 * (n_frames, 4) float64 on the device: mean |w|, max |w|, mean divergence
 * (np.gradient), |mean w| (motion_correction/compensate_recording.py:808-821).
 * workspace: frg_flow_post_workspace bytes of device memory. */
size_t frg_flow_post_workspace(int n_frames, int height, int width);
int frg_flow_post(int n_frames, int height, int width, const float* flow, unsigned char* valid, void* workspace,
                  double* stats, void* stream);

/* ---------------------------------------------------------------------------
 * Differentiable mode.
 *
 * pyflowreg's flow path with the level solver of its torch backend
 * ("flowreg_torch": torch/core/level_solver.py:11-199, registered at
 * core/__init__.py:140-197; red-black order, eps = 1e-6, psi tick when
 * it % update_lag == 0; within-pixel order selectable, below) and a continuous warp (the map is not rounded to
 * 1/32 px as cv2.remap does in core/warping.py:160-234; Keys cubic,
 * replicated borders, out-of-bounds pixels from the reference frame).  The
 * reference runs that backend under torch.no_grad(); these entry points add
 * what it has no counterpart for: the gradient of the flow with respect to
 * both frames and alpha.  frg_diff_forward stores per-level checkpoints (the
 * resized frames, the level's input flow and the solver state at every psi
 * tick); frg_diff_backward recomputes each level from them and runs the
 * adjoint sweeps.  Supported: gradient constancy, a_smooth = 1, min_level 0.
 *
 * Arrays are device memory, planar: frames (F, K, H, W), flows (F, 2, H, W)
 * with plane 0 = u (columns) and plane 1 = v (rows).  The element type is
 * float for a plan created with precision FRG_FP32 and double for
 * FRG_FP64_REFERENCE (the pointers below are void* for that reason).
 * ------------------------------------------------------------------------- */
typedef struct frg_diff_plan frg_diff_plan;

/* Plan flags.
 * FRG_DIFF_TORCH_ORDER: the torch backend's within-pixel order, du and dv of
 *   a moving pixel both from the old values: a Jacobi step on the 2x2 pixel
 *   block, which diverges with omega = 1.95 wherever |A12| / sqrt(A11 A22)
 *   > 2 / omega - 1 (most data-dominated pixels of a gradient-constancy
 *   tensor).  Without it (default) dv is taken from the new du, the numba
 *   solver's order (core/level_solver.py:355-364): the sweep is then SOR on a
 *   symmetric positive definite system and converges for omega < 2.
 * FRG_DIFF_STORE_SWEEPS: the forward keeps the pixels moved by every
 *   half-sweep (2 * iterations * F * h * ceil(w / 2) * 2 elements per level)
 *   and the backward reads them; without it the forward keeps the state at
 *   each psi tick only and the backward recomputes each window. */
#define FRG_DIFF_TORCH_ORDER 1
#define FRG_DIFF_STORE_SWEEPS 2
/* Backward flag FRG_DIFF_LAGGED_PSI: hold psi fixed at each tick (the adjoint
 * of the lagged-nonlinearity system); without it the gradient also runs
 * through psi = a (E + 1e-6)^(a - 1), whose slope near E = 0 (~1e9) makes it
 * exact but stiff. */
#define FRG_DIFF_LAGGED_PSI 1
/* Backward flag FRG_DIFF_IMPLICIT: per level, hold psi at its last tick and
 * differentiate the fixed point of the level system M x = b (M symmetric
 * positive definite, the operator the sweeps iterate) instead of the
 * unrolled iterations: lam = M^-1 dL/dx by one red-black SOR solve of
 * `iterations` sweeps on the same operator, then dL/db = lam and
 * dL/dM = -lam x^T with x the level's final state.  Exact for a converged
 * forward; an approximation of the unrolled gradient otherwise. */
#define FRG_DIFF_IMPLICIT 2
/* Backward flag FRG_DIFF_STEPWISE_ADJOINT: run the unrolled adjoint one
 * launch per half-sweep.  By default each tick window's half-sweeps run in
 * one launch over tiles with halos held in shared memory (the same
 * per-pixel arithmetic, so the flow's gradients agree to rounding in the
 * alpha sums); windows too large for shared memory run stepwise anyway. */
#define FRG_DIFF_STEPWISE_ADJOINT 4

int frg_diff_plan_create(const frg_params* params, int height, int width, int channels, int max_frames, int flags,
                         frg_diff_plan** out);
void frg_diff_plan_destroy(frg_diff_plan* plan);
size_t frg_diff_plan_device_bytes(const frg_diff_plan* plan);
int frg_diff_plan_num_levels(const frg_diff_plan* plan);
/* Replaces the tap tables of one level (same layout as frg_plan_set_level_tables). */
int frg_diff_set_level_tables(frg_diff_plan* plan, int level, int kind, int taps, const int* ix, const float* wx,
                              const int* iy, const float* wy);
/* weight: (K, H, W) device array of the plan's element type. */
int frg_diff_set_weight(frg_diff_plan* plan, const void* weight, void* stream);
/* flow_out (F, 2, H, W); uv_init (F, 2, H, W) or NULL for zero.  alpha_x,
 * alpha_y override the plan's (the values the backward differentiates at). */
int frg_diff_forward(frg_diff_plan* plan, int n_frames, double alpha_x, double alpha_y, const void* fixed,
                     const void* moving, const void* uv_init, void* flow_out, void* stream);
/* Gradient of a loss L given g_flow = dL/dflow (F, 2, H, W) for the last
 * frg_diff_forward: g_fixed, g_moving (F, K, H, W) are overwritten;
 * g_alpha (F, 2) device doubles are overwritten with dL/d(alpha_x, alpha_y)
 * per frame.  Any of the outputs may be NULL. */
int frg_diff_backward(frg_diff_plan* plan, const void* g_flow, void* g_fixed, void* g_moving, double* g_alpha,
                      int flags, void* stream);
/* Continuous compensation warp out = src(x + flow) with out-of-bounds pixels
 * from fill (motion_correction/parallelization/sequential.py:148-154), and its
 * adjoint (g_src, g_fill, g_flow overwritten; any may be NULL except g_src).
 * precision selects float (FRG_FP32) or double (FRG_FP64_REFERENCE). */
int frg_diff_warp(int precision, int n_frames, int channels, int height, int width, const void* src,
                  const void* flow, const void* fill, void* out, void* stream);
int frg_diff_warp_backward(int precision, int n_frames, int channels, int height, int width, const void* src,
                           const void* flow, const void* g_out, void* g_src, void* g_fill, void* g_flow,
                           void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FLOWREG_GB300_H */
