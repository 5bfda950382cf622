/*
 * gbode.h -- C ABI of libgbode.so, the GB300 (sm_103a) implementation of the
 * adaptive embedded Runge-Kutta N-body hot path of noether17/ode_prototyping.
 *
 * Conventions
 *  - Every entry point returns an int status: GB_OK (0), a negative gb_status
 *    on an argument, CUDA or numerical failure.  Nothing aborts; the last CUDA
 *    error is kept for gb_last_cuda_error().  (The reference prints CUDA errors
 *    and continues, src/cuda_util/CudaErrorCheck.cuh:8-16; here the caller
 *    decides.)
 *  - Pointers named *_dev are device pointers; *_host are host pointers.
 *  - State vectors use the reference layout (src/ode/NBodyODE.hpp:12-13):
 *    x = [x0 y0 z0 x1 ... z_{N-1} | vx0 vy0 vz0 ... vz_{N-1}], n_var = 6N FP64.
 *  - Work is enqueued on `stream` (a cudaStream_t; NULL = legacy default
 *    stream).  Entry points that return a host scalar synchronise the stream.
 *  - No entry point uses torch or any C++ type.
 */
#ifndef GBODE_H_
#define GBODE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* gb_stream_t; /* == cudaStream_t */

typedef enum {
  GB_OK = 0,
  GB_ERR_INVALID_ARGUMENT = -1,
  GB_ERR_CUDA = -2,
  GB_ERR_UNSUPPORTED = -3,
  GB_ERR_NOT_FINITE = -4,    /* error estimate or state became NaN/Inf */
  GB_ERR_BUDGET = -5,        /* attempt budget exhausted before tf */
  GB_ERR_TIMEOUT = -6,       /* a bounded host or device wait ran out */
  GB_ERR_CAPACITY = -7,      /* caller-provided workspace too small */
  GB_ERR_STEP_UNDERFLOW = -8 /* step size fell below the floor at t < tf */
} gb_status;

const char* gb_status_string(int status);
/* Last cudaError_t value observed by the library (0 if none). */
int gb_last_cuda_error(void);
/* Library version as major*10000 + minor*100 + patch. */
int gb_version(void);

/* ---------------------------------------------------------------------- */
/* Butcher tableaus                                                         */
/* Replaces: the tableau template parameter of RKEmbeddedParallel          */
/* (src/integrator/RKEmbeddedParallel/RKEmbeddedParallel.hpp:11) and the   */
/* structs of butcher_tableaus/BT*.hpp (a, b, bt, p, pt, n_stages).        */
/* a[s-1][j] is the coefficient of k_j in stage s (j < s); there is no c   */
/* vector because the ODE interface is autonomous.                         */
/* ---------------------------------------------------------------------- */
#define GB_MAX_STAGES 16

typedef struct {
  int32_t n_stages;
  int32_t p;  /* order of the propagated solution (b) */
  int32_t pt; /* order of the embedded solution (bt) */
  double a[GB_MAX_STAGES][GB_MAX_STAGES];
  double b[GB_MAX_STAGES];
  double bt[GB_MAX_STAGES];
} gb_tableau;

enum { GB_HE21 = 0, GB_RKF45 = 1, GB_DOPRI5 = 2, GB_DVERK = 3, GB_RKF78 = 4 };

/* Fills `out` with one of the built-in tableaus (BTHE21.hpp:5-12,
 * BTRKF45.hpp:5-21, BTDOPRI5.hpp:5-26, BTDVERK.hpp:5-27, BTRKF78.hpp:5-45). */
int gb_tableau_builtin(int32_t id, gb_tableau* out);

/* ---------------------------------------------------------------------- */
/* Device memory helpers, so that host code using only this header (no     */
/* CUDA headers) can own device states.                                    */
/* Replaces: CudaState's cudaMalloc/cudaMemcpy/cudaFree                    */
/* (src/state/CudaState.cuh:15-50).                                        */
/* ---------------------------------------------------------------------- */
int gb_device_alloc(void** ptr_dev, size_t bytes);
int gb_device_free(void* ptr_dev);
/* kind: 0 host->device, 1 device->host, 2 device->device.  Synchronous. */
int gb_memcpy(void* dst, const void* src, size_t bytes, int32_t kind);
int gb_memset_zero(void* ptr_dev, size_t bytes);
int gb_fill_f64(double* ptr_dev, int64_t n, double value, gb_stream_t stream);
int gb_stream_synchronize(gb_stream_t stream);
/* Where a pointer lives: 0 host (pageable or pinned), 1 device, 2 managed. */
int gb_pointer_kind(const void* ptr);

/* ---------------------------------------------------------------------- */
/* All-pairs softened gravity right-hand side (FP64).                      */
/* Replaces: NBodyODE<double, 6N>::operator() and acc() with               */
/* nbody_init_dxdt_kernel and nbody_acc_kernel                              */
/* (src/ode/NBodyODE.hpp:31-46, 51-56, 68-133).                            */
/* acc_i = mass * sum_{j != i} (x_j - x_i) / ((|x_j - x_i|^2 + eps^2)^{1/2} */
/*        * (|x_j - x_i|^2 + eps^2)), every operation IEEE-rounded with no */
/* contraction, as the reference evaluates it.  With masses_dev != NULL    */
/* each term is weighted by m_j instead (the masses branch commented out in */
/* NBodyODE.hpp:104-124) and `mass` is ignored.                            */
/* Tiling: each body's sum runs over partner indices in ascending order    */
/* split into `j_split` contiguous chunks (thread-block cluster ranks) and */
/* `lanes` interleaved lanes (warp-shuffle partial sums), combined in a    */
/* fixed order.  j_split = lanes = 1 reproduces the reference's serial     */
/* executor bit for bit; 0 lets the library choose.                        */
/* ---------------------------------------------------------------------- */
typedef struct {
  int32_t j_split;       /* CTAs per thread-block cluster sharing one i-tile: 1,2,4,8,16
                            (0 = auto; 16 is a non-portable cluster size).  The
                            integrator's mixed stage with one lane per body (packed
                            loops, from N = 8192 by default) reads it as independent
                            partner chunks per i-tile, no clusters: 2..32 */
  int32_t lanes;         /* lanes per body inside a warp: 1,2,4,8 (0 = auto) */
  int32_t bodies_per_cta;/* i-bodies per CTA: 32..256 (0 = auto) */
  int32_t mixed_variant; /* mixed-precision pair loop: 0 = auto (3), 1 = scalar FP32 (two
                            bodies per thread, any masses), 2 = packed f32x2 over pairs of
                            partners with two bodies per thread, 3 = the same with one
                            body per thread; the packed loops need uniform masses
                            (per-body masses run the scalar loop) */
  int32_t f64_pair;      /* FP64 pair term: 0 = the entry point's default, 1 = r^-3 from a
                            Newton-refined reciprocal square root with fused multiply-add
                            sums (a few ulp per term, ~2.5x fewer FP64 operations), 2 = the
                            reference's operation order (IEEE sqrt and divisions,
                            NBodyODE.hpp:89-98).  The standalone right-hand sides default to
                            2; the integrator's FP64 stages default to 1 (exact mode: 2) */
} gb_force_tiling;

int gb_nbody_rhs_f64(const double* x_dev, double* dxdt_dev, int64_t n_particles,
                     double softening, double mass, const double* masses_dev,
                     const gb_force_tiling* tiling, gb_stream_t stream);
/* acc (3N) only; accumulate != 0 adds into acc_dev instead of overwriting. */
int gb_nbody_acc_f64(const double* pos_dev, double* acc_dev, int64_t n_particles,
                     double softening, double mass, const double* masses_dev, int32_t accumulate,
                     const gb_force_tiling* tiling, gb_stream_t stream);

/* Mixed precision: FP32 pair arithmetic on positions split into hi + lo  */
/* FP32 parts relative to a reference point, rsqrt on the SFU, FP32 sums   */
/* per j-tile with Kahan-compensated accumulation across tiles, FP64 state */
/* in and out.  Requires softening > 0.  `work_dev` holds the packed       */
/* j-bodies: gb_nbody_mixed_workspace_bytes(n) bytes, 16-byte aligned.     */
size_t gb_nbody_mixed_workspace_bytes(int64_t n_particles);
int gb_nbody_rhs_mixed(const double* x_dev, double* dxdt_dev, int64_t n_particles,
                       double softening, double mass, const double* masses_dev, void* work_dev,
                       const gb_force_tiling* tiling, gb_stream_t stream);

/* The same mixed-precision right-hand side on spatially sorted tiles: the */
/* bodies are ordered along a Morton curve, every 128-body tile carries its */
/* centroid and radius, and partners in a tile whose gap to the i-tile is   */
/* at least that tile's radius use FP32 coordinates relative to the tile    */
/* centroid (one subtraction per component; relative error <= 4 * 2^-24);  */
/* nearer tiles use the hi/lo difference.  Rows are returned in body order. */
/* work_dev: gb_nbody_mixed_sorted_workspace_bytes(n) bytes, 256-aligned.   */
size_t gb_nbody_mixed_sorted_workspace_bytes(int64_t n_particles);
int gb_nbody_rhs_mixed_sorted(const double* x_dev, double* dxdt_dev, int64_t n_particles,
                              double softening, double mass, const double* masses_dev,
                              void* work_dev, size_t work_bytes, const gb_force_tiling* tiling,
                              gb_stream_t stream);

/* No counterpart in the reference.  The same mixed-precision right-hand   */
/* side for callers that cannot allocate device memory (a host that gives  */
/* the library a fixed slice of device memory and refuses further          */
/* cudaMalloc, or a per-stage caller that cannot pay for cudaMalloc /      */
/* cudaFree, whose free waits for the whole device).  The workspace is a   */
/* fixed array inside the library (2 MiB + 256 B per GPU that loads it,    */
/* held until exit), so n_particles may not exceed                         */
/* gb_nbody_rhs_mixed_noalloc_max_bodies() (65536); larger n returns       */
/* GB_ERR_CAPACITY.  The first call on each device looks the array's       */
/* device address up (cudaGetSymbolAddress); make that first call before   */
/* any stream capture.  All calls share the one array, so calls that       */
/* overlap on the GPU (other streams, other threads) race and must be      */
/* serialised by the caller.  Nothing in it needs to start at zero.  The  */
/* looked-up address is kept for the life of the process: after           */
/* cudaDeviceReset the module is reloaded at a possibly different address, */
/* so this entry point must not be called after a reset.  It checks its    */
/* arguments as gb_nbody_rhs_mixed does and gives the same bits.           */
int64_t gb_nbody_rhs_mixed_noalloc_max_bodies(void);
int gb_nbody_rhs_mixed_noalloc(const double* x_dev, double* dxdt_dev, int64_t n_particles,
                               double softening, double mass, const double* masses_dev,
                               const gb_force_tiling* tiling, gb_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Element-wise embedded-RK kernels with a host-scalar dt.                 */
/* ---------------------------------------------------------------------- */
/* Replaces rk_stage_kernel (RKEmbeddedParallel.hpp:91-101):
 * temp = x0 + dt * sum_{j<stage} a[stage-1][j] * ks[j*n_var + i]. */
int gb_rk_stage_f64(const gb_tableau* tab, int32_t stage, double dt, const double* x0_dev,
                    const double* ks_dev, double* temp_dev, int64_t n_var, gb_stream_t stream);
/* Replaces update_state_and_error_kernel (:103-123). */
int gb_rk_update_state_and_error_f64(const gb_tableau* tab, double dt, const double* x0_dev,
                                     const double* ks_dev, double* x_dev, double* err_dev,
                                     int64_t n_var, gb_stream_t stream);
/* Replaces update_error_target_kernel (:125-130):
 * target = atol + rtol * max(|x|, |x0|). */
int gb_rk_error_target_f64(const double* atol_dev, const double* rtol_dev, const double* x_dev,
                           const double* x0_dev, double* target_dev, int64_t n_var,
                           gb_stream_t stream);
/* Replaces rk_norm + scaled_value_squared_kernel (:132-149) run through
 * CudaExecutor::transform_reduce (src/par_exec/CudaExecutor.cuh:97-125):
 * *norm_dev = sqrt(sum_i (v_i / scale_i)^2 / n).  Deterministic two-level
 * reduction; the per-block partial sums live in `work_dev`
 * (gb_rk_norm_workspace_bytes(n) bytes).  The result stays on the device. */
size_t gb_rk_norm_workspace_bytes(int64_t n);
int gb_rk_norm_f64(const double* v_dev, const double* scale_dev, int64_t n, void* work_dev,
                   size_t work_bytes, double* norm_dev, gb_stream_t stream);
/* Replaces the executor's transform_reduce<double, add, scaled_value_squared>
 * with its host result: returns sum_i (v_i/scale_i)^2 in *sum_host
 * (synchronises the stream). */
int gb_rk_scaled_sq_sum_f64(const double* v_dev, const double* scale_dev, int64_t n,
                            void* work_dev, size_t work_bytes, double* sum_host,
                            gb_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Device-resident adaptive integrator for one N-body system.              */
/* Replaces RKEmbeddedParallel<BT>::integrate (RKEmbeddedParallel.hpp:13-81)*/
/* with estimate_initial_step (:170-200), run entirely on the GPU: every    */
/* stage is one fused kernel (force + stage combination for the next stage  */
/* in the epilogue), the last stage also forms x, the error estimate, the   */
/* error target, the scaled RMS norm and the step-size decision on the      */
/* device.  Attempts are replayed from a CUDA graph; the host only polls a  */
/* completion flag every `attempts_per_sync` attempts.                      */
/* ---------------------------------------------------------------------- */
/* ---------------------------------------------------------------------- */
/* Learned step-size proposer (no counterpart in the reference): MLP       */
/* 16 -> 64 -> 64 -> 1 with SiLU.  FP32 master weights for training, a    */
/* BF16-weight / FP32-accumulate copy inside the controller.  Its output is */
/* log(dt_next / dt); the embedded error estimate still accepts or rejects, */
/* and every rejection falls back to the PI controller.                    */
/* ---------------------------------------------------------------------- */
#define GB_MLP_IN 16
#define GB_MLP_HIDDEN 64

typedef struct {
  float w1[GB_MLP_HIDDEN][GB_MLP_IN];
  float b1[GB_MLP_HIDDEN];
  float w2[GB_MLP_HIDDEN][GB_MLP_HIDDEN];
  float b2[GB_MLP_HIDDEN];
  float w3[GB_MLP_HIDDEN];
  float b3;
  float in_mean[GB_MLP_IN];  /* feature normalisation: (f - mean) * scale */
  float in_scale[GB_MLP_IN];
  float out_scale;           /* prediction = out_scale * y + out_bias */
  float out_bias;
} gb_mlp;

/* One controller log record per attempt (see gb_integrate_opts.log_steps). */
typedef struct {
  float feat[GB_MLP_IN];
  float log_dt;       /* attempted step */
  float log_err;      /* scaled error norm it produced */
  float accepted;
  float log_dt_ideal; /* the elementary controller's proposal after it */
} gb_step_log;

/* Seeded initialisation (uniform +-sqrt(6/(fan_in+fan_out)), zero biases,
 * identity normalisation). Host memory. */
int gb_mlp_init(gb_mlp* m_host, uint64_t seed);
/* Forward pass over a batch in FP32: x_dev [B][16] -> y_dev [B].  When
 * act_dev is not NULL it receives the pre-activations needed by the
 * backward pass: gb_mlp_act_floats(B) floats. */
int64_t gb_mlp_act_floats(int64_t batch);
int gb_mlp_forward_f32(const gb_mlp* w_dev, const float* x_dev, float* y_dev, int64_t batch,
                       float* act_dev, gb_stream_t stream);
/* Backward pass of L = sum_b loss(y_b) given dL/dy in dy_dev [B]: writes the
 * parameter gradients (same layout as gb_mlp, normalisation fields zero) to
 * grad_dev.  Deterministic (fixed-order block partials). work_dev holds
 * gb_mlp_backward_workspace_bytes(B) bytes. */
size_t gb_mlp_backward_workspace_bytes(int64_t batch);
int gb_mlp_backward_f32(const gb_mlp* w_dev, const float* x_dev, const float* act_dev,
                        const float* dy_dev, gb_mlp* grad_dev, int64_t batch, void* work_dev,
                        gb_stream_t stream);
/* Adam update of every trainable parameter (normalisation untouched). */
int gb_mlp_adam_step(gb_mlp* w_dev, const gb_mlp* grad_dev, gb_mlp* m_dev, gb_mlp* v_dev,
                     float lr, float beta1, float beta2, float eps, int32_t step,
                     gb_stream_t stream);
/* BF16-weight / FP32-accumulate inference over a batch (the controller's
 * arithmetic, exposed for tests): x_dev [B][16] -> y_dev [B]. */
int gb_mlp_infer_bf16(const gb_mlp* w_dev, const float* x_dev, float* y_dev, int64_t batch,
                      gb_stream_t stream);
/* Full-batch training loop on the device: `epochs` Adam steps on the
 * asymmetric squared error (over-predictions weighted by `over_weight`)
 * between the network output and target_dev [B]; x_dev [B][16].  Returns
 * the final mean loss in *loss_host. */
int gb_mlp_train(gb_mlp* w_dev, const float* x_dev, const float* target_dev, int64_t batch,
                 int32_t epochs, float lr, float over_weight, float* loss_host,
                 gb_stream_t stream);

enum { GB_PREC_F64 = 0, GB_PREC_MIXED = 1 };
enum {
  GB_CTRL_REFERENCE = 0, /* the reference's elementary controller (:58-79) */
  GB_CTRL_PI = 1,        /* PI controller (beta = 0.04 by default) */
  GB_CTRL_LEARNED = 2    /* MLP proposal, embedded error decides, PI fallback */
};

typedef struct {
  int64_t n_particles;
  double softening;
  double mass;             /* uniform mass when masses_dev == NULL */
  const double* masses_dev;/* optional per-body masses */
} gb_nbody_system;

typedef struct {
  int32_t precision;          /* GB_PREC_* */
  int32_t controller;         /* GB_CTRL_* */
  int32_t fsal;               /* reuse the last stage as the next first stage when the
                                 tableau allows it (bit-identical results) */
  int32_t exact;              /* serial-order forces and norm (reference bit pattern) */
  int32_t attempts_per_sync;  /* attempts per graph replay (0 = 16) */
  int32_t record;             /* deliver every accepted state to the save callback */
  int64_t max_attempts;       /* 0 = unlimited (the reference has no bound) */
  double host_wait_timeout_s; /* bound on one host wait (0 = 600 s) */
  double pi_beta;             /* PI controller beta (0 = 0.04) */
  gb_force_tiling tiling;     /* 0 fields = auto */
  const void* mlp;            /* gb_mlp* weights for GB_CTRL_LEARNED (device-resident copy made) */
  int32_t log_steps;          /* record per-attempt controller logs on the device */
  int32_t spatial_sort;       /* mixed precision: 0 = default (uniform masses, N >= 8192:
                                 the partner-chunk stage on Morton-sorted bodies, where
                                 64-partner quarter tiles whose boxes are far from every
                                 body of a warp skip the close-pair test), 1 = Morton-sorted tiles with the
                                 tile-centroid far-field path, 2 = the sorted chunk stage
                                 without that culling (the same bits as 0), 3 = the
                                 chunk stage in body order */
} gb_integrate_opts;

typedef struct {
  int64_t n_accepted;
  int64_t n_rejected;
  int64_t n_attempts;
  int64_t n_rhs;             /* right-hand side evaluations (initial step included) */
  int64_t n_rhs_saved;       /* evaluations skipped by FSAL */
  double t;                  /* current time */
  double dt;                 /* next step size */
  double dt_initial;
  double err_last;           /* last scaled error norm */
  double interactions;       /* ordered pair interactions evaluated, N(N-1) per RHS */
  int32_t status;            /* gb_status of the integration */
  int32_t done;
  int64_t n_learned_proposals;
  int64_t n_learned_rejected;
} gb_integrate_stats;

typedef void (*gb_save_fn)(void* user, double t, const double* x_host, int64_t n_var);

typedef struct gb_integrator_s* gb_integrator;

/* The integrator runs on `stream` when it is not the legacy default stream
 * (NULL), otherwise on a stream it owns; CUDA graphs are replayed there. */
int gb_integrator_create(const gb_tableau* tab, const gb_nbody_system* sys,
                         const gb_integrate_opts* opts, gb_stream_t stream, gb_integrator* out);
/* Copies x0 (device), sets t0/tf and tolerances (device vectors of n_var, or
 * scalars when the pointers are NULL), estimates the initial step on the
 * device and, when recording, delivers (t0, x0) to `save`. */
int gb_integrator_start(gb_integrator it, const double* x0_dev, double t0, double tf,
                        const double* atol_dev, const double* rtol_dev, double atol_scalar,
                        double rtol_scalar, gb_save_fn save, void* user);
/* Runs attempts until t >= tf, a failure, or `max_attempts` more attempts
 * (<= 0: no bound here).  Accepted states go to `save` in order when
 * recording.  Returns the integration status. */
int gb_integrator_advance(gb_integrator it, int64_t max_attempts, gb_save_fn save, void* user);
/* Enqueues `n_replays` graph replays without waiting (benchmarking); call
 * gb_integrator_sync afterwards. */
int gb_integrator_enqueue(gb_integrator it, int64_t n_replays);
int gb_integrator_sync(gb_integrator it);
int gb_integrator_stats(gb_integrator it, gb_integrate_stats* out);
/* Copies the current state x0 to x_dev (device) and the time to *t_host. */
int gb_integrator_state(gb_integrator it, double* x_dev, double* t_host);
int gb_integrator_destroy(gb_integrator it);
/* Profiling: launches the fused kernel of one stage of the current attempt
 * on the integrator's stream without the end-of-attempt controller.  The
 * buffers it writes are recomputed by the next attempt. */
int gb_integrator_launch_stage(gb_integrator it, int32_t stage);
/* Launch geometry chosen for the fused stage kernel (mixed_variant = the pair loop in use, per
 * CTA) and the number of CTAs per launch. */
int gb_integrator_geometry(gb_integrator it, gb_force_tiling* out, int64_t* n_ctas);
/* Dense output (DOPRI5 only, the continuous extension of NumericalRecipes/ */
/* StepperDopr5.hpp:179-219, which the template integrator lacks): states  */
/* at the given ascending times are evaluated on the device after each     */
/* accepted step, without shortening any step.  Call between create and    */
/* start; gb_integrator_dense_output copies those computed so far.         */
int gb_integrator_set_dense_output(gb_integrator it, const double* times_host, int64_t n_times);
int gb_integrator_dense_output(gb_integrator it, double* x_host, int64_t capacity, int64_t* count);
/* Copies up to `capacity` controller log records (opts.log_steps > 0). */
int gb_integrator_log(gb_integrator it, gb_step_log* host_records, int64_t capacity,
                      int64_t* count);

/* One-call form: integrate and write the final state. */
int gb_integrate_nbody(const gb_tableau* tab, const gb_nbody_system* sys,
                       const gb_integrate_opts* opts, const double* x0_dev, double t0, double tf,
                       const double* atol_dev, const double* rtol_dev, double atol_scalar,
                       double rtol_scalar, gb_save_fn save, void* user, double* x_final_dev,
                       gb_integrate_stats* stats, gb_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Batched integrator: many independent N-body systems of uneven size,     */
/* each following RKEmbeddedParallel<BT>::integrate's loop with its own    */
/* step size, decision and status.  No counterpart in the reference (its   */
/* state size is a compile-time constant, src/state/ODEState.hpp:7-23).    */
/* Work units (system, i-tile) are ordered by cost and taken round-robin by */
/* a persistent stage kernel (small systems can share a CTA, one warp      */
/* group each: gb_batch_tiling.systems_per_cta); one warp per system runs  */
/* its controller; an                                                      */
/* attempt is one CUDA graph replay.  Equal masses per system; scalar      */
/* tolerances per system.  States are concatenated: system k occupies      */
/* x[6*B_k .. 6*(B_k+N_k)) with B_k = N_0 + ... + N_{k-1}.                  */
/* ---------------------------------------------------------------------- */
typedef struct {
  int32_t threads_per_cta;   /* 64, 128, 256 (0 = 128) */
  int32_t lanes;             /* lanes per body: 1, 2, 4 (0 = 2) */
  int32_t bodies_per_thread; /* mixed precision: 1 or 2 bodies per thread; the packed
                                f32x2 loop over pairs of partners at threads_per_cta <= 128,
                                the scalar FP32 loop at 256 (0 = 1) */
  int32_t grid_ctas;         /* persistent grid (0 = 8 CTAs per SM) */
  int32_t systems_per_cta;   /* 1, 2 or 4 (0 = 1): with G > 1, every system whose bodies fit
                                one warp group's tile (N <= bodies per CTA tile / G) is
                                integrated by a group of threads_per_cta / G threads, and
                                G such systems share a CTA; larger systems take whole CTAs */
} gb_batch_tiling;

typedef struct {
  int32_t precision;         /* GB_PREC_* */
  int32_t controller;        /* GB_CTRL_* */
  int32_t fsal;
  int32_t attempts_per_sync; /* attempts per graph replay (0 = 8) */
  int64_t max_attempts;      /* per system, 0 = unlimited */
  double host_wait_timeout_s;
  double pi_beta;
  gb_batch_tiling tiling;
  const void* mlp;           /* gb_mlp* (host) for GB_CTRL_LEARNED */
} gb_batch_opts;

typedef struct gb_batch_s* gb_batch;

int gb_batch_create(const gb_tableau* tab, int32_t n_systems, const int64_t* n_particles,
                    const double* softening, const double* mass, const gb_batch_opts* opts,
                    gb_stream_t stream, gb_batch* out);
/* x0_dev: concatenated states; t0, tf, atol, rtol: host arrays, one per system. */
int gb_batch_start(gb_batch b, const double* x0_dev, const double* t0, const double* tf,
                   const double* atol, const double* rtol);
/* Replays attempts until every system reaches its tf (or max_replays graph
 * replays, 0 = no bound); returns the first failing system's status. */
int gb_batch_advance(gb_batch b, int64_t max_replays);
int gb_batch_enqueue(gb_batch b, int64_t n_replays);
int gb_batch_sync(gb_batch b);
/* totals: sums over systems (t = the smallest time); per_sys: n_systems entries or NULL. */
int gb_batch_stats(gb_batch b, gb_integrate_stats* totals, gb_integrate_stats* per_sys);
int gb_batch_state(gb_batch b, double* x_dev, double* t_host);
int gb_batch_launch_stage(gb_batch b, int32_t stage);
/* Times each candidate tile geometry and grid size on this batch and keeps
 * the fastest (call after gb_batch_start). */
int gb_batch_autotune(gb_batch b, int32_t reps, gb_batch_tiling* chosen, double* best_ms);
int gb_batch_geometry(gb_batch b, gb_batch_tiling* out, int64_t* n_units);
int gb_batch_destroy(gb_batch b);

/* ---------------------------------------------------------------------- */
/* Fixed-step kick-drift-kick leapfrog on the same force kernels.           */
/* Replaces ParallelLeapfrogIntegrator::integrate                           */
/* (src/integrator/leapfrog/LeapfrogParallel.hpp:11-41, kernels :57-73):    */
/* same update formulas and order; x_dev is advanced in place; `save`       */
/* receives t0 and every step's state (host copy).                         */
/* ---------------------------------------------------------------------- */
int gb_leapfrog_nbody(const gb_nbody_system* sys, double* x_dev, double t0, double tf, double dt,
                      int32_t precision, const gb_force_tiling* tiling, gb_save_fn save,
                      void* user, int64_t* n_steps, gb_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Trajectory files in the reference's binary format                        */
/* (src/demo/nbody_io.hpp:4-22; read by scripts/nbody_io/bin_reader.py):   */
/* uint64 n_times, uint64 n_var, float64 softening, then per saved state    */
/* float64 t and n_var float64 values.  Records are written by a background */
/* thread as they arrive; gb_trajectory_close patches n_times.  Pass        */
/* gb_trajectory_save with the writer as `user` to the integrator to stream */
/* every accepted state to disk (the reference keeps them all in memory and */
/* writes at the end).                                                     */
/* ---------------------------------------------------------------------- */
typedef struct gb_trajectory_s* gb_trajectory;

int gb_trajectory_open(const char* path, int64_t n_var, double softening, gb_trajectory* out);
int gb_trajectory_append(gb_trajectory w, double t, const double* x_host);
void gb_trajectory_save(void* user, double t, const double* x_host, int64_t n_var);
int gb_trajectory_close(gb_trajectory w, int64_t* n_times);

/* ---------------------------------------------------------------------- */
/* Energy and momentum diagnostics (FP64).                                 */
/* Replaces the softened potential and kinetic energies of                */
/* scripts/nbody_physics/energy.py:146-192 (unit masses there), with       */
/* masses: out_dev[0] kinetic, [1] potential, [2..4] linear momentum,      */
/* [5..7] angular momentum about the origin.                               */
/* ---------------------------------------------------------------------- */
size_t gb_nbody_energy_workspace_bytes(int64_t n_particles);
int gb_nbody_energy_f64(const double* x_dev, int64_t n_particles, double softening, double mass,
                        const double* masses_dev, void* work_dev, size_t work_bytes,
                        double* out_dev, gb_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Seeded initial conditions (host memory, reference state layout, G = 1,  */
/* total mass 1 with equal masses 1/N, centre of mass at rest at 0).       */
/* Replace the scenario generators of src/demo/n_body_scenarios/ and the   */
/* seeded cube of src/test/SpinningCubeNBodyTest.hpp:37-57 for the         */
/* benchmark configurations.                                               */
/* ---------------------------------------------------------------------- */
int gb_ic_uniform_ball(int64_t n, uint64_t seed, double sigma_v, double* x_host);
int gb_ic_plummer(int64_t n, uint64_t seed, double scale_radius, double* x_host);
int gb_ic_set_virial_ratio(int64_t n, double q, double softening, double* x_host);
int gb_ic_cold_sphere(int64_t n, uint64_t seed, double noise, double* x_host);
int gb_ic_binary_plummer(int64_t n, uint64_t seed, double binary_frac, double amin, double amax,
                         double* x_host);

#ifdef __cplusplus
}
#endif

#endif /* GBODE_H_ */
