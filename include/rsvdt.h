/*
 * rsvdt.h -- C ABI of the GB300 RSVD-Delta-t time-stepping library.
 *
 * One context owns one GPU stream and every device buffer of one resolvent
 * problem. It replaces the reference's PETSc-typed hot-path functions
 * (AliFarghadan/RSVD-Delta-t, SourceCode/): the entry points below name the
 * reference function each one stands in for.
 *
 * Conventions
 *  - Complex values cross this interface as interleaved (re, im) doubles,
 *    layout-compatible with C99 `double _Complex` and PETSc's complex
 *    PetscScalar. "count complex values" means 2*count doubles.
 *  - Spectral blocks (forcing F_hat, response Y_hat, modes U/V) use the
 *    reference's layout: rows x (k*Nw_eff), column-major, column iw*k+ik
 *    (frequency-major; SourceCode/CreateRandomMat.c:34,
 *    SourceCode/PermuteMat.c:24-34), leading dimension `ld` >= rows.
 *  - Sparse matrices are CSR with int64 row pointers and column indices
 *    (PETSc 64-bit-index AIJ). Host arrays are caller-owned and copied.
 *  - Every call returns an rsvdt_status; 0 is success. rsvdt_last_error()
 *    gives the message of the last failure on that context. A context is
 *    not thread-safe; separate contexts may be used from separate threads.
 *  - There is no CPU fallback: without a usable GPU rsvdt_create fails with
 *    RSVDT_ERR_CUDA.
 */
#ifndef RSVDT_H
#define RSVDT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  RSVDT_OK = 0,
  RSVDT_ERR_ARG = 1,      /* invalid argument or size mismatch (SETERRQ PETSC_ERR_USER) */
  RSVDT_ERR_IO = 2,       /* file could not be read or written */
  RSVDT_ERR_OOM = 3,      /* device or host allocation failed */
  RSVDT_ERR_CUDA = 4,     /* CUDA runtime error */
  RSVDT_ERR_NOT_SPD = 5,  /* Cholesky of a Gram matrix failed (rank-deficient block) */
  RSVDT_ERR_DIVERGED = 6, /* NaN or Inf in the state */
  RSVDT_ERR_TIMEOUT = 7,  /* a bounded device wait gave up */
  RSVDT_ERR_STATE = 8     /* call out of order (e.g. action before operator) */
} rsvdt_status;

typedef enum { RSVDT_ADJOINT = 0, RSVDT_DIRECT = 1 } rsvdt_dir;

typedef enum {
  RSVDT_PREC_C128 = 0,       /* plain form: complex128 throughout */
  RSVDT_PREC_C64 = 1,        /* precision form: complex64 operator/state/stages, FP32
                                accumulation; FP64 DFT, QR, SVD and spectral blocks */
  RSVDT_PREC_C64_REFINE = 2  /* precision form with one FP64 sweep: every action in
                                complex64 except the last adjoint action of
                                rsvdt_run, which runs in complex128 (the gains it
                                yields then carry the complex64 subspace error only
                                to second order) */
} rsvdt_precision;

/* Weight / input / output matrices (SourceCode/Variables.h:69-80). */
typedef enum {
  RSVDT_W_F_SQRT_INV = 0, /* W_f^{-1/2}, Nb x Nb */
  RSVDT_B = 1,            /* B, N x Nb */
  RSVDT_C = 2,            /* C, Nc x N */
  RSVDT_W_Q_SQRT = 3,     /* W_q^{1/2}, Nc x Nc */
  RSVDT_W_Q_SQRT_INV = 4  /* W_q^{-1/2}, Nc x Nc */
} rsvdt_weight;

/* Mirrors RSVD_vars / TS_vars / Discounting (SourceCode/Variables.h:5-41)
 * and the variables.yaml keys of the same names. */
typedef struct {
  int64_t k;               /* test vectors */
  int64_t q;               /* power iterations */
  int64_t Nw;              /* frequencies */
  double w;                /* base frequency (multiplied by 2*pi when TwoPI) */
  int32_t TwoPI;           /* bool */
  double dt;               /* requested time step (adjusted as SetupTimeFreqGrid does) */
  double TransientLength;  /* transient length */
  int32_t TransientRemoval;/* bool: Galerkin transient removal */
  int32_t DiscFlg;         /* bool: A <- A - beta*I */
  double beta;             /* discount */
  int32_t precision;       /* rsvdt_precision */
  int32_t Display;         /* 0 silent, 1 phases, 2 progress (stdout) */
} rsvdt_params;

/* Derived time grid (SourceCode/SetupTimeFreqGrid.c:16-21). */
typedef struct {
  double w;        /* effective base frequency */
  double dt;       /* adjusted time step */
  int64_t Ns;      /* steps per period */
  int64_t Nt;      /* transient steps */
  int64_t ResRatio;/* Ns / Nw */
  int64_t Nw_eff;  /* effective frequencies (Nw, or Nw/2 for a real operator) */
  int64_t N, Nb, Nc;
} rsvdt_grid;

typedef struct rsvdt_ctx rsvdt_ctx;

/* Fills defaults of SourceCode/ReadUserInput.c (k=3, q=0, Display=2, ...). */
void rsvdt_default_params(rsvdt_params *p);

/* Validates params, selects the CUDA device, creates the stream.
 * Replaces SourceCode/PreProcessing.c:27-36 (ReadUserInput's checks and
 * SetupTimeFreqGrid); the grid is final once the operator is set. */
rsvdt_status rsvdt_create(const rsvdt_params *p, rsvdt_ctx **out);
void rsvdt_destroy(rsvdt_ctx *ctx);
const char *rsvdt_last_error(const rsvdt_ctx *ctx);

/* Operator A (N x N), copied to the device together with its explicit
 * conjugate transpose for the adjoint. Detects a real operator
 * (||Im A||_F < 1e-12) and applies discounting.
 * Replaces SourceCode/LNSStructure.c:22-56 (after MatLoad) and
 * SourceCode/CreateDFTiDFTMats.c:5-97. */
rsvdt_status rsvdt_set_operator(rsvdt_ctx *ctx, int64_t N, const int64_t *rowptr,
                                const int64_t *col, const double *val);

/* Block-CSR operator with dense bs x bs blocks (row-major inside a block);
 * nb = N/bs block rows. Same semantics as rsvdt_set_operator. */
rsvdt_status rsvdt_set_operator_bcsr(rsvdt_ctx *ctx, int64_t nb, int32_t bs,
                                     const int64_t *browptr, const int64_t *bcol,
                                     const double *val);

/* Weight / input / output matrix as CSR (rows x cols). A matrix whose
 * nonzeros are exactly its diagonal takes a fused diagonal path.
 * Replaces SourceCode/ReadWeightMats.c:26-99 (after MatLoad). */
rsvdt_status rsvdt_set_weight(rsvdt_ctx *ctx, rsvdt_weight which, int64_t rows, int64_t cols,
                              const int64_t *rowptr, const int64_t *col, const double *val);

/* Grid after rsvdt_set_operator. */
rsvdt_status rsvdt_get_grid(const rsvdt_ctx *ctx, rsvdt_grid *g);

/* Sketch F_hat (Nb x ncols, frequency-major) copied into the working block
 * Y_hat; k becomes ncols / Nw_eff as in SourceCode/CreateRandomMat.c:28-30
 * (ncols must be a multiple of Nw_eff). Replaces
 * SourceCode/CreateRandomMat.c:23-31 (InputForcingDir). */
rsvdt_status rsvdt_set_sketch(rsvdt_ctx *ctx, const double *F, int64_t ld, int64_t ncols);

/* Random sketch: i.i.d. standard complex normal entries from a counter-based
 * generator seeded by `seed` (SourceCode/CreateRandomMat.c:33-39, which
 * draws from PETSc's generator instead). */
rsvdt_status rsvdt_random_sketch(rsvdt_ctx *ctx, uint64_t seed);

/* Copies the working block Y_hat (rows x k*Nw_eff) to the host; rows is Nb
 * or Nc depending on the last action. */
rsvdt_status rsvdt_get_block(rsvdt_ctx *ctx, double *Y, int64_t ld, int64_t *rows);

/* Direct (R) or adjoint (R^H) resolvent action on the working block,
 * weights included. Replaces SourceCode/DirectActionRK4.c:7-32 and
 * SourceCode/AdjointActionRK4.c:7-32 with everything below them
 * (TSActionRK4, TSRK4, CreateForcingOnFly, SaveSnapshots, DFT,
 * TransientRemovalStrategy, ApplyWeightMats). */
rsvdt_status rsvdt_action(rsvdt_ctx *ctx, rsvdt_dir dir);

/* Orthonormalises each frequency's rows x k block in place (batched
 * CholQR2). Replaces SourceCode/QRAllFreqs.c:5-46. */
rsvdt_status rsvdt_qr_all_freqs(rsvdt_ctx *ctx);

/* Per-frequency thin SVD of the working block. before_adjoint = 1: the
 * block becomes its left singular vectors and is stored as U
 * (SourceCode/SVDAllFreqsBeforeAdjoint.c:5-68 + SourceCode/StoreU.c:5-19).
 * before_adjoint = 0: left singular vectors become V, singular values the
 * gains, and the inverse weights are applied to U and V
 * (SourceCode/SVDAllFreqs.c:5-79). */
rsvdt_status rsvdt_svd_all_freqs(rsvdt_ctx *ctx, int32_t before_adjoint);

/* Power iteration loop (SourceCode/PowerIterationRK4.c:8-36). */
rsvdt_status rsvdt_power_iteration(rsvdt_ctx *ctx);

/* Checkpoint hook of the power iteration. The reference's only resume path
 * is to feed a forcing matrix back through InputForcingDir
 * (SourceCode/CreateRandomMat.c:10-11,23-31); this hook produces such a
 * matrix. fn(user, sweep, ctx) is called after the second QR of every sweep
 * (sweep = 1..q), when the working block holds the forcing of that sweep's
 * direct action; fn may read it with rsvdt_get_block. Setting that block as
 * the sketch (rsvdt_set_sketch, or InputForcingDir in the drop-in driver) and
 * running with q - sweep power iterations continues the sequence exactly
 * (identical results). A non-zero return stops rsvdt_power_iteration and
 * rsvdt_run with RSVDT_ERR_STATE. fn = NULL removes the hook. */
typedef int (*rsvdt_checkpoint_fn)(void *user, int32_t sweep, rsvdt_ctx *ctx);
rsvdt_status rsvdt_set_checkpoint(rsvdt_ctx *ctx, rsvdt_checkpoint_fn fn, void *user);

/* The whole RSVD-Delta-t sequence of SourceCode/main.c:134-144 on the
 * current sketch. */
rsvdt_status rsvdt_run(rsvdt_ctx *ctx);

/* Results of rsvdt_run: U (Nc x k*Nw_eff), V (Nb x k*Nw_eff) in the
 * frequency-major layout, S (k x Nw_eff, column-major) gains. Any pointer
 * may be NULL. Replaces reading Res_mat in SourceCode/SaveResults.c:32-85. */
rsvdt_status rsvdt_get_results(rsvdt_ctx *ctx, double *U, int64_t ldu, double *V, int64_t ldv,
                               double *S);

/* Advances the RK4 state of every test vector by nsteps forced steps
 * starting at step index i0 (1-based, as SourceCode/TSRK4.c's i), with the
 * forcing built from the working block. Host state y (N x k, column-major,
 * complex) and F3 (forcing at the start of step i0, N x k) are read and
 * updated (for the stage engine, the uploads run on a second stream while
 * the first step's forcing is synthesised, and F3 is downloaded while the
 * last step's stages 2-4 run). In the precision form (RSVDT_PREC_C64) the
 * host values are rounded to complex64 on upload and widened back on
 * download. For kernel-level tests and benchmarks;
 * rsvdt_action is the normal entry. Replaces SourceCode/TSRK4.c:6-51
 * called in the loop of SourceCode/TSActionRK4.c:116-122. */
rsvdt_status rsvdt_rk4_steps(rsvdt_ctx *ctx, rsvdt_dir dir, int64_t i0, int64_t nsteps, double *y,
                             double *F3);

/* Device-resident variant of rsvdt_rk4_steps for timing: the state stays
 * on the device between calls (reset by rsvdt_rk4_reset), nothing is
 * copied. */
rsvdt_status rsvdt_rk4_reset(rsvdt_ctx *ctx, rsvdt_dir dir);
rsvdt_status rsvdt_rk4_advance(rsvdt_ctx *ctx, rsvdt_dir dir, int64_t i0, int64_t nsteps);

/* Runs nsteps device-resident steps (as rsvdt_rk4_advance) launching the
 * four RK4 stage kernels one by one with CUDA events between them on the
 * context's stream; stage_ms[0..3] receive each stage's total time in
 * milliseconds (stage 1 including the forcing-block kernel when the forcing
 * is synthesised ahead, see rsvdt_set_forcing_block). For benchmarks and
 * roofline measurements. */
rsvdt_status rsvdt_rk4_profile(rsvdt_ctx *ctx, rsvdt_dir dir, int64_t i0, int64_t nsteps,
                               double *stage_ms);
/* As rsvdt_rk4_profile, with the forcing-block kernel timed on its own:
 * times_ms[0..3] the four stages, times_ms[4] the forcing-block launches (0
 * when stage 1 synthesises the forcing). */
rsvdt_status rsvdt_rk4_profile_ex(rsvdt_ctx *ctx, rsvdt_dir dir, int64_t i0, int64_t nsteps,
                                  double *times_ms);

/* Forcing synthesis of the complex64 block-row stages (5x5 block-CSR
 * operator, k in {2, 4, 6, 8, 10, 16}, Nw_eff in {8, 16, 32, 64}): the
 * forcing at the two times of each step (SourceCode/CreateForcingOnFly.c:
 * 17-19, called twice per step by SourceCode/TSRK4.c:21-27) is a sum over
 * the Nw_eff frequency coefficients of each (row, test vector). steps = 0:
 * stage 1 forms it every step, reading all the coefficients every step.
 * steps = G (1, 2, 4, 8 or 16): one kernel forms the forcings of G steps at
 * once, reading the coefficients once per G steps, into a buffer of
 * 2 G N k complex64 values that stages 1-4 read (same operations in the same
 * order: identical results). The buffer is the half of the forcing-slab
 * buffer that complex64 slabs leave unused (no extra memory) when G <=
 * Nw_eff / 2; a longer block gets its own allocation if 4 GiB of device
 * memory stay free, else the stage-1 synthesis runs. -1 (default): the
 * largest of 16, 8, 4, 2, 1 that fits in the slab buffer's spare half.
 * Other stage kernels ignore it. */
rsvdt_status rsvdt_set_forcing_block(rsvdt_ctx *ctx, int32_t steps);
/* Block length in use by the last complex64 stepping (0 = none). */
int32_t rsvdt_get_forcing_block(const rsvdt_ctx *ctx);

/* ----------------------------------------------------------- capacity mode
 * For problems whose spectral blocks do not fit several times in device
 * memory (N = 10.5M, k = 16, Nw = 64: one block is 172 GB in complex128):
 * every action runs its test vectors in chunks of kc (kc divides k; 0 picks
 * the largest chunk that fits) and writes each chunk's response into its own
 * columns of the one working block; the weight products and the SVDs work in
 * place; U is kept in host memory (complex64 when u_c64 is set) from the SVD
 * before the adjoint to the end. Results equal the resident mode's to
 * rounding. Call before the sketch (best right after rsvdt_create, so that
 * the resident buffers are never allocated); set the weights before the
 * sketch too. rsvdt_rk4_steps is not available in this mode. */
rsvdt_status rsvdt_set_capacity_mode(rsvdt_ctx *ctx, int64_t kc, int32_t u_c64);
/* Chunk size in use (0 when the context is not in capacity mode). */
rsvdt_status rsvdt_get_capacity(const rsvdt_ctx *ctx, int64_t *kc);

/* Lanes per (row, test vector) of the RK4 stages: 1 = one thread per row
 * (the stage kernels for large problems), 2 / 4 / 8 = that many lanes
 * splitting a row's nonzeros and forcing slabs (the batched stage kernel,
 * for small problems), 0 = chosen from the problem size (default). The
 * results agree to rounding (summation order). */
rsvdt_status rsvdt_set_lanes_per_row(rsvdt_ctx *ctx, int32_t lanes);
int32_t rsvdt_get_lanes_per_row(const rsvdt_ctx *ctx);

/* Stepping engine. STAGES: four stage launches per step (replayed from CUDA
 * graphs; lanes per row as above). CLUSTER (problems with at most 512 rows
 * x test vectors per SM of the cluster, 8192 for a cluster of 16): the
 * forcing of 64 steps at a time over the whole GPU, then the 64 steps'
 * stages on one thread-block cluster with a hardware cluster barrier
 * between stages, no launch per stage; the same operations in the same
 * order as the one-lane stage kernels (bit-identical). AUTO (default) picks
 * CLUSTER for problems of at most 8192 values where the device can launch
 * such a cluster; the lanes-per-row setting then applies only where the
 * STAGES engine runs. */
typedef enum { RSVDT_ENGINE_AUTO = 0, RSVDT_ENGINE_STAGES = 1, RSVDT_ENGINE_CLUSTER = 2 } rsvdt_step_engine;
rsvdt_status rsvdt_set_step_engine(rsvdt_ctx *ctx, int32_t engine);
int32_t rsvdt_get_step_engine(const rsvdt_ctx *ctx);

/* Wall time per phase since creation (or the last reset) as a JSON object:
 * actions run per direction, RK4 steps, seconds spent preparing actions
 * (weights, forcing slabs), stepping, finishing them (DFT or transient
 * removal, weights), in QR and in SVD, the mean step time, the lanes per
 * row and the capacity chunk. The reference prints the same phases as
 * elapsed times (SourceCode/TSActionRK4.c:150-160, DisplayProgress.c);
 * with Display >= 1 the library prints them too. */
rsvdt_status rsvdt_get_timings(const rsvdt_ctx *ctx, char *json, int64_t len);
rsvdt_status rsvdt_reset_timings(rsvdt_ctx *ctx);

/* 1 for the bounds-checked debug build (compiled with RSVDT_DEBUG: the
 * stage kernels check every gathered column and ring slot, skip an access
 * that fails and make the action return RSVDT_ERR_ARG), 0 otherwise. */
int32_t rsvdt_debug_build(void);

/* Free and total memory of the current CUDA device, in bytes (for callers
 * deciding on the capacity mode before they create the buffers). */
rsvdt_status rsvdt_device_memory(int64_t *free_bytes, int64_t *total_bytes);

/* Columns cols[0..ncols) (indices iw*k + ik) of U (Nc rows) and V (Nb rows)
 * after rsvdt_run, column-major with leading dimensions ldu / ldv; U or V
 * may be NULL. For results too large to fetch whole (e.g. the files of
 * SourceCode/SaveResults.c:46-85, one test vector or one frequency at a
 * time). */
rsvdt_status rsvdt_get_result_cols(rsvdt_ctx *ctx, const int64_t *cols, int64_t ncols, double *U, int64_t ldu,
                                   double *V, int64_t ldv);

/* ------------------------------------------------------ transient simulation
 * The initial-value problem dq/dt = A q (A discounted when DiscFlg) by
 * unforced RK4 from a given initial vector, with the norm checked every
 * save_mod steps. Replaces SourceCode/TransientRunRK4.c:11-228 with
 * SourceCode/TSTransRK4.c:5-40 and SourceCode/TransientRemovalEst.c:6-129
 * (the file writing stays with the caller, through the callbacks). */
typedef struct {
  int64_t periods;     /* TransPeriods: integrate periods * Nt_period steps */
  int64_t save_mod;    /* TransSaveMod (>= 1): norm checked every save_mod steps */
  double div_val;      /* TransDivVal: stop when the norm exceeds it */
  double con_val;      /* TransConVal: stop when the norm falls below it */
  int32_t save;        /* TransSave: pass every checked snapshot to on_snapshot */
  int32_t removal_est; /* TransRemovalEst: transient-removal estimate every period */
} rsvdt_trans_params;

typedef enum {
  RSVDT_TRANS_DONE = 0,      /* all steps taken */
  RSVDT_TRANS_NAN = 1,       /* a checked norm was NaN */
  RSVDT_TRANS_DIVERGED = 2,  /* a checked norm exceeded div_val */
  RSVDT_TRANS_CONVERGED = 3  /* a checked norm fell below con_val */
} rsvdt_trans_stop;

typedef struct {
  double dt;          /* T/Nw / ceil((T/Nw) / dt_grid) (TransientRunRK4.c:42) */
  int64_t Nt_period;  /* round(T / dt) */
  int64_t rend;       /* Nt_period * periods */
  int64_t n_saved;    /* floor(rend / save_mod) + 1: length of `norms` */
  int64_t steps;      /* steps taken */
  int32_t stop;       /* rsvdt_trans_stop */
  double last_norm;   /* norm at the stop (or at the last check) */
} rsvdt_trans_info;

/* Called with snapshot number pos (= step / save_mod, 0 for the initial
 * vector) and the N complex values of the state; nonzero aborts the run
 * with RSVDT_ERR_IO. */
typedef int (*rsvdt_trans_snapshot_fn)(void *user, int64_t pos, const double *q, int64_t n);
/* Called at the end of every period p >= 1 with the Nw/2 initial and
 * updated transient norms of TransientRemovalEst; nonzero aborts. */
typedef int (*rsvdt_trans_estimate_fn)(void *user, int64_t period, const double *initial,
                                       const double *updated, int64_t count);

/* Time grid of a transient run (info->dt, Nt_period, rend, n_saved) without
 * running it. */
rsvdt_status rsvdt_trans_grid(rsvdt_ctx *ctx, const rsvdt_trans_params *tp, rsvdt_trans_info *info);

/* Runs the transient simulation. q: N complex values, the initial vector on
 * entry and the last snapshot on return. norms: n_saved doubles, zeroed
 * then filled at every check that passed (norms[0] = |q0|). Callbacks may be
 * NULL. A stop on NaN / divergence / convergence is not an error: it is
 * reported in info->stop, as the reference prints it and saves what it has. */
rsvdt_status rsvdt_trans_run(rsvdt_ctx *ctx, const rsvdt_trans_params *tp, double *q, double *norms,
                             rsvdt_trans_snapshot_fn on_snapshot, rsvdt_trans_estimate_fn on_estimate,
                             void *user, rsvdt_trans_info *info);

/* ---------------------------------------------------------------- batching
 * Many independent problems of uneven size (own operator, k, Nw, time
 * grid, q) solved together: every action of the sequence runs for all
 * problems at once, their RK4 steps advancing in lockstep with one launch
 * per RK4 stage covering every problem's rows, replayed from a CUDA graph.
 * The launch shape (threads per block, lanes per row) is chosen at the
 * first run by timing candidates on the batch itself. The batch form of
 * running SourceCode/main.c:134-144 for each problem in turn. */
typedef struct rsvdt_batch rsvdt_batch;

/* precision: RSVDT_PREC_C128, RSVDT_PREC_C64, or RSVDT_PREC_C64_REFINE
 * (complex64 actions, the last adjoint action of every problem batched in
 * complex128). */
rsvdt_status rsvdt_batch_create(int32_t precision, rsvdt_batch **out);
void rsvdt_batch_destroy(rsvdt_batch *b);
const char *rsvdt_batch_last_error(const rsvdt_batch *b);
/* Adds a problem with CSR operator A (as rsvdt_set_operator); the batch's
 * precision overrides p->precision. *index receives its position. */
rsvdt_status rsvdt_batch_add(rsvdt_batch *b, const rsvdt_params *p, int64_t N, const int64_t *rowptr,
                             const int64_t *col, const double *val, int32_t *index);
rsvdt_status rsvdt_batch_set_sketch(rsvdt_batch *b, int32_t index, const double *F, int64_t ld,
                                    int64_t ncols);
rsvdt_status rsvdt_batch_random_sketch(rsvdt_batch *b, int32_t index, uint64_t seed);
/* Runs the whole sequence for every problem (q per problem). */
rsvdt_status rsvdt_batch_run(rsvdt_batch *b);
rsvdt_status rsvdt_batch_get_results(rsvdt_batch *b, int32_t index, double *U, int64_t ldu, double *V,
                                     int64_t ldv, double *S);
rsvdt_status rsvdt_batch_get_grid(const rsvdt_batch *b, int32_t index, rsvdt_grid *g);
/* Launch shape chosen by the autotuner and its time per batched step. */
rsvdt_status rsvdt_batch_get_tuning(const rsvdt_batch *b, int32_t *threads, int32_t *lanes_per_row,
                                    double *ms_per_step);
/* Test vectors per lane of the chosen shape: 1, or 2 (complex64 stages,
 * every problem's k even: 16-byte accesses). */
int32_t rsvdt_batch_values_per_lane(const rsvdt_batch *b);
/* Fixes the launch shape instead of autotuning it (threads 128 or 256,
 * lanes per row 1/2/4/8, values per lane 1 or 2); threads = 0 returns to
 * the autotuner. Call after the last rsvdt_batch_add. */
rsvdt_status rsvdt_batch_set_launch_shape(rsvdt_batch *b, int32_t threads, int32_t lanes_per_row,
                                          int32_t values_per_lane);
int64_t rsvdt_batch_launch_count(const rsvdt_batch *b);

/* ------------------------------------------------------- learned sketch
 * Multilayer perceptron (GELU between layers, linear output) that maps a
 * problem's parameters to the coefficients of a warm-start test matrix in
 * a POD basis. bf16 weights, FP32 activations, products and gradients;
 * trained with Adam on a mean-squared-error loss. Inference and training
 * kernels are the library's own. No counterpart in the reference, whose
 * sketch is always random (SourceCode/CreateRandomMat.c:33-39). */
typedef struct rsvdt_mlp rsvdt_mlp;

/* widths: n_layers + 1 entries (input, hidden..., output). */
rsvdt_status rsvdt_mlp_create(int32_t n_layers, const int32_t *widths, uint64_t seed, rsvdt_mlp **out);
void rsvdt_mlp_destroy(rsvdt_mlp *n);
const char *rsvdt_mlp_last_error(const rsvdt_mlp *n);
/* Flat FP32 parameters: for each layer, W (out x in, row-major) then b. */
int64_t rsvdt_mlp_param_count(const rsvdt_mlp *n);
rsvdt_status rsvdt_mlp_set_params(rsvdt_mlp *n, const float *params);
rsvdt_status rsvdt_mlp_get_params(rsvdt_mlp *n, float *params);
/* Y (rows x out) = network(X (rows x in)); host arrays. */
rsvdt_status rsvdt_mlp_forward(rsvdt_mlp *n, const float *X, int64_t rows, float *Y);
/* Mean squared error against T and its gradient (flat, like the params). */
rsvdt_status rsvdt_mlp_gradients(rsvdt_mlp *n, const float *X, const float *T, int64_t rows, float *loss,
                                 float *grads);
/* Adam (lr, beta1 0.9, beta2 0.999) for `steps` minibatches of `batch`
 * rows drawn without replacement per epoch; the data set is copied to the
 * device once. final_loss: loss of the last minibatch. */
rsvdt_status rsvdt_mlp_train(rsvdt_mlp *n, const float *X, const float *T, int64_t samples, int64_t batch,
                             int64_t steps, float lr, uint64_t seed, float *final_loss);

/* QR of every frequency block without allocating device memory.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc (work issued while another stream is being captured into a
 * CUDA graph, host frameworks whose pool owns all device memory, services
 * that forbid allocation after start-up). It needs no context.
 *
 * Y (input) and Q (output) are caller-allocated device arrays of rows x nw
 * x k complex128 values in the library's spectral-block layout
 * Y[(row*nw + iw)*k + j]; Q may equal Y. Each row-frequency block is
 * orthonormalised with the same shifted CholQR passes as
 * rsvdt_qr_all_freqs, on `stream` (a cudaStream_t), and the call returns
 * after the stream has finished this work (it waits for a 4-byte status
 * read back into host memory).
 *
 * Stream: NULL is the legacy default stream, which synchronises with every
 * blocking stream of the device; while another stream is being captured
 * that implicit synchronisation invalidates the capture. Callers in that
 * situation must pass a non-blocking stream of their own
 * (cudaStreamNonBlocking) or cudaStreamPerThread.
 *
 * Scratch comes from a fixed 4 MiB device array inside the library, one
 * per device context that loads the library's device code, held as long as
 * that context lives (until the process exits, or until the context is torn
 * down, e.g. by cudaDeviceReset). Limits: k <= 32 and nw*k*k <= 65535;
 * larger sizes return RSVDT_ERR_ARG without touching the GPU. Every call
 * looks up the array's device address in the current context
 * (cudaGetSymbolAddress, a host-side query that allocates nothing); the
 * first call in a context may load the library's device code, so make that
 * first call before any stream capture. Every call reuses the same array,
 * so calls that overlap on the GPU (from two streams or two host threads at
 * once) race and must be serialised by the caller. The Gram products form
 * the full k x k matrices (twice the work of rsvdt_qr_all_freqs, which forms
 * one triangle); the QR stages are a small part of a solve. errbuf
 * (optional, errlen bytes) receives a message on failure. */
rsvdt_status rsvdt_qr_all_freqs_noalloc(const double *Y, double *Q, int64_t rows, int64_t nw,
                                        int64_t k, void *stream, char *errbuf, int64_t errlen);

/* Waits for the context's stream. */
rsvdt_status rsvdt_synchronize(rsvdt_ctx *ctx);

/* The context's cudaStream_t, for timing with events on the launching
 * stream. */
void *rsvdt_stream(rsvdt_ctx *ctx);

/* Number of kernels the context has launched so far. */
int64_t rsvdt_launch_count(const rsvdt_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
