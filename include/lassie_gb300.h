/*
 * lassie_gb300.h -- C ABI of the GB300-native LASSIE integrator.
 *
 * The reference (aresio/LASSIE) has no library interface: its boundary is the
 * command line `LASSIE input_folder output_folder` (src/c++/simulator.cu:29)
 * and the files of those folders.  Behind its CLI the engine is one class,
 * Simulation<T>::run (src/c++/header/Simulation.cuh:230-981), which parses the
 * folder, compiles the network, integrates on the GPU and writes the outputs.
 * The entry points below are that engine split at the natural seams, with
 * plain pointers and sizes so any host (the bundled C++ CLI, Python ctypes,
 * cgo, JNI) can bind them.  Each cites the reference code it replaces.
 *
 * Conventions: every function returns LASSIE_OK (0) or a negative status;
 * host buffers are caller-owned; device memory is owned by the library and
 * released by the matching destroy call.  A model handle may be shared by
 * concurrent solves; a batch handle is not thread-safe.  `stream` arguments
 * are cudaStream_t values passed as void* (NULL = the legacy stream).
 */
#ifndef LASSIE_GB300_H
#define LASSIE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------- statuses */
#define LASSIE_OK 0
/* -1 .. -13 are the reference's process exit codes (simulator.cu:66-335,
   Simulation.cuh:43-1010); the CLI exits with them. */
#define LASSIE_ERR_INPUT_FOLDER (-1)
#define LASSIE_ERR_MANDATORY (-4)
#define LASSIE_ERR_MODELKIND (-7)
#define LASSIE_ERR_VOLUME (-8)
#define LASSIE_ERR_ORDER (-12)
#define LASSIE_ERR_CUDA (-13)
/* new statuses of the library */
#define LASSIE_ERR_ARGS (-20)        /* invalid argument */
#define LASSIE_ERR_MAX_STEPS (-21)   /* opts.max_steps loop iterations reached */
#define LASSIE_ERR_ALLOC (-22)       /* host or device allocation failed */
#define LASSIE_ERR_TOO_LARGE (-23)   /* network does not fit the engine */
#define LASSIE_ERR_DEADLINE (-24)    /* opts.deadline_s elapsed on the device */
#define LASSIE_ERR_NO_DEVICE (-25)   /* no CUDA device / not sm_103 */
#define LASSIE_ERR_RECORD_FULL (-26) /* adjoint step record capacity reached */
#define LASSIE_ERR_STEP_TOO_SMALL (-27) /* BDF controller: step below 10 ulp of t */

/* step control (lassie_opts.controller) */
#define LASSIE_CTRL_COMPAT 0 /* LASSIE's loop: RKF45 + fixed-step backward Euler
                                (Simulation.cuh:632-925) */
#define LASSIE_CTRL_BDF 1    /* variable-order BDF 1-5 with rtol/atol error control
                                (the reference's unused BDF2-6 correctors,
                                kernels.cuh:302-457, with step and order
                                selection); N <= 512.  precision FP64: FP64
                                LU; MIXED: an FP32 Gauss-Jordan inverse refined
                                in FP64 as the Newton solve; a step that
                                fails on FP32 factors is retried on FP64
                                factors, and an instance keeps FP64 factors
                                after 4 such failures without an FP32
                                success in between */

/* precision of the Newton matrix factorisation */
#define LASSIE_PREC_FP64 0  /* FP64 LU: the plain FP64 GPU form */
#define LASSIE_PREC_MIXED 1 /* FP32 LU + FP64 iterative refinement */
#define LASSIE_PREC_FLOAT 2 /* the reference's -p float mode (Simulation<float>,
                               simulator.cu:289-294): state, rate constants,
                               stages and Newton matrix in float, double
                               temporaries where the reference has them;
                               LASSIE's controller, networks of at most 512
                               species */

typedef struct lassie_model lassie_model;
typedef struct lassie_batch lassie_batch;

/* Integration options.  Defaults (lassie_opts_default) are the reference's
   optional-file defaults, Simulation.cuh:272-354. */
typedef struct {
    double rkf_step;      /* initial RKF45 step, file rkf_step (1e-3) */
    double be_step;       /* backward-Euler step, file be_step (0.01) */
    double newton_tol;    /* Newton ||dx||_2 tolerance, file newton_tol (1e-6) */
    double stiffness_tol; /* stiffness switch threshold, file stiffness_tol (1e-6) */
    int64_t newton_iter;  /* Newton iteration cap, file newton_iter (10000) */
    int64_t max_steps;    /* loop-iteration cap per instance, 0 = none */
    double deadline_s;    /* device wall-clock limit per launch, 0 = none */
    int32_t precision;    /* LASSIE_PREC_* */
    int32_t refine_max;   /* refinement sweeps per linear solve (mixed), 0 = 8 */
    int32_t quarter_root; /* RKF45 step factor (atol/R)^(1/4): LASSIE_ROOT_POW
                             = pow(x, 0.25) as kernels.cuh:193 (default);
                             LASSIE_ROOT_SQRT = sqrt(sqrt(x)), correctly rounded
                             on every platform (matches the CPU restatement) */
    int32_t lu_reuse;     /* mixed form: 1 (default) lets a backward-Euler step
                             precondition its refinement with the FP32 factors
                             of an earlier step of the same step size while they
                             contract the residual by 2e-3 or better per sweep
                             (the refinement still converges to the FP64 solve of
                             the current matrix); 0 factors at every step */
    int32_t tensor_cores; /* wide engine (networks above 512 species), mixed
                             form: LASSIE_TC_TF32 runs the rank-128
                             super-panel updates of the Gauss-Jordan
                             factorisation on the tensor cores (tcgen05,
                             TF32 products of split operands, close to FP32),
                             LASSIE_TC_BF16 with BF16 operands and FP32
                             accumulation (factors good to about 2^-9; the FP64
                             refinement takes more sweeps), LASSIE_TC_OFF on
                             the FP32 pipes; default LASSIE_TC_TF32.  The
                             rank-32 updates within a super-panel run on the
                             FP32 pipes in every setting */
    int32_t controller;   /* LASSIE_CTRL_* (default LASSIE_CTRL_COMPAT) */
    /* LASSIE_CTRL_BDF only: */
    double rtol;          /* relative tolerance (1e-6) */
    double atol;          /* absolute tolerance when an instance has no atol
                             vector (1e-9); an instance's atol vector is used
                             as absolute tolerances per species */
    double first_step;    /* 0 = chosen from f(x0) */
    double max_step;      /* 0 = unbounded */
    int32_t max_order;    /* 1..5 (5) */
    /* Rows per thread of the per-CTA factorisation's trailing-update tiles
       (128 x 16*rows): 0 (default) lets the autotuner time 8, 4 and 2 per
       network-size band on the device when the batch is created (once per
       process, device, band and precision) and store its choice in the
       batch; 8, 4 or 2 fix it.  Every choice gives the same factors bit for
       bit (each entry sums the same products in the same order); only the
       speed differs.  Replaces the fixed launch heuristic of the reference
       (Simulation.cuh:583-600). */
    int32_t tile_rows;
} lassie_opts;

#define LASSIE_TC_OFF 0
#define LASSIE_TC_TF32 1
#define LASSIE_TC_BF16 2

#define LASSIE_ROOT_POW 0
#define LASSIE_ROOT_SQRT 1

/* Per-instance counters; status is the instance's LASSIE_* result. */
typedef struct {
    int64_t outer_iters;
    int64_t rkf_accepts;
    int64_t rkf_retries;
    int64_t be_steps;
    int64_t newton_iters;
    int64_t lu_factorisations;
    int64_t lu_failures;
    int64_t nan_reverts;
    int64_t refine_sweeps;
    /* SM clock cycles spent (thread 0 of the instance's CTA) in the RKF45
       attempts, the Newton-matrix assembly, the LU, and the linear solves */
    int64_t cycles_rkf;
    int64_t cycles_matrix;
    int64_t cycles_lu;
    int64_t cycles_solve;
    /* parts of cycles_lu: panel factorisation, row moves + U12 solve, trailing
       update */
    int64_t cycles_lu_panel;
    int64_t cycles_lu_rows;
    int64_t cycles_lu_trailing;
    /* part of cycles_solve: the FP32 triangular solves (mixed form) */
    int64_t cycles_solve_tri;
    double t_final;
    double dt_be_final;   /* BDF controller: the last step size */
    int32_t status;
    int32_t pad;
    /* BDF controller (be_steps counts its accepted steps, rkf_retries its
       error-test rejections, lu_failures its Newton failures, outer_iters
       its attempts) */
    int64_t jac_evals;
    int64_t rhs_evals;
    int32_t order_final;
    int32_t pad2;
    /* SM clock cycles of the instance's whole integration (thread 0 of its
       CTA); lassie_batch_order_by_cost orders later runs by it */
    int64_t cycles_total;
} lassie_stats;

/* One instance of a batch: a network, its parameterisation and its outputs.
   feed, atol and cs may be NULL (no feed, atol 1e-12, all species). */
typedef struct {
    const lassie_model *model;
    const double *k;    /* [R] rate constants */
    const double *x0;   /* [N] initial state */
    const double *feed; /* [N] fed (constant) species, 0 = not fed */
    const double *atol; /* [N] RKF45 absolute tolerance per unit time */
    const double *t;    /* [nt] sampling times */
    int32_t nt;
    int32_t ncs;
    const int32_t *cs;  /* [ncs] sampled species */
    double *out;        /* [nt * ncs] host output, row per sample */
} lassie_instance;

void lassie_opts_default(lassie_opts *opts);
const char *lassie_status_string(int status);
/* Text of the last CUDA or argument error on the calling thread. */
const char *lassie_last_error(void);
/* 1 if an sm_103 device is visible and the kernels load, else 0 */
int lassie_device_ok(void);

/* Model compiler: replaces Simulation.cuh:397-418 (createTransposte,
   create_sparse, create_sparse2) with int32 CSR (no int16 cap).
   left/right: dense R x N row-major reactant/product stoichiometries, the
   contents of the left_side / right_side files (Reader.h:104-124). */
int lassie_model_create_dense(int32_t n_species, int32_t n_reactions,
                              const int32_t *left, const int32_t *right,
                              lassie_model **out);
/* Same network given by reaction: reactants react_ptr[R+1] / react_species /
   react_stoich and products prod_ptr[R+1] / prod_species / prod_stoich
   (repeated species are summed). */
int lassie_model_create_csr(int32_t n_species, int32_t n_reactions,
                            const int32_t *react_ptr, const int32_t *react_species,
                            const int32_t *react_stoich, const int32_t *prod_ptr,
                            const int32_t *prod_species, const int32_t *prod_stoich,
                            lassie_model **out);
void lassie_model_destroy(lassie_model *model);
int lassie_model_info(const lassie_model *model, int32_t *n_species,
                      int32_t *n_reactions, int32_t *nnz_reactants,
                      int32_t *nnz_net);

/* One integration, host buffers in and out: the time loop of
   Simulation.cuh:632-925 plus the sampling of :674-690 and the D2H copy of
   :942.  out has nt*ncs doubles (cs NULL: ncs = N). */
int lassie_solve(const lassie_model *model, const double *k, const double *x0,
                 const double *feed, const double *atol, const double *t,
                 int32_t nt, const int32_t *cs, int32_t ncs,
                 const lassie_opts *opts, double *out, lassie_stats *stats);

/* Many independent instances of possibly different networks and sizes in
   one persistent launch (no reference counterpart: the reference runs one
   model per process).  Host buffers in and out; stats may be NULL. */
int lassie_solve_batch(const lassie_instance *inst, int32_t n,
                       const lassie_opts *opts, lassie_stats *stats);

/* Device-resident batch: upload once, run many times (inputs stay in HBM),
   read back on demand.  lassie_batch_run only launches on `stream`;
   lassie_batch_sync waits and returns the first failing instance status. */
int lassie_batch_create(const lassie_instance *inst, int32_t n,
                        const lassie_opts *opts, lassie_batch **out);
int lassie_batch_run(lassie_batch *batch, void *stream);
int lassie_batch_sync(lassie_batch *batch);
int lassie_batch_read(lassie_batch *batch, const lassie_instance *inst,
                      lassie_stats *stats);
/* kernel launches one lassie_batch_run issues (for launch accounting) */
int lassie_batch_launches(const lassie_batch *batch);
/* Orders the batch's later runs by the last run's per-instance integration
   times (lassie_stats.cycles_total), longest first, so that the persistent
   work queue ends with short instances (replaces the launch heuristic of
   Simulation.cuh:583-600 for repeated runs; the reference runs one model per
   process).  Results of every instance do not depend on the order.  A batch
   that has not run keeps its creation order (largest network first).  Waits
   for the batch's stream; refused while that stream is being captured.
   A captured run replays with the new order. */
int lassie_batch_order_by_cost(lassie_batch *batch);
/* bytes lassie_solve_batch moves host->device (inputs) and device->host
   (trajectories and stats) for this batch */
int lassie_batch_bytes(const lassie_batch *batch, int64_t *h2d, int64_t *d2h);
void lassie_batch_destroy(lassie_batch *batch);

/* Discrete adjoint (no reference counterpart).  Integrates the instances in
   the form opts->precision names (mixed or FP64), recording the step
   sequence, then runs the backward pass
   of that exact step sequence for
       L_q = sum over samples i and sampled species j of (y_ij - target_ij)^2
   and returns loss[q], grad_logk[q][R] = dL_q/dlog k and (when grad_x0 is
   not NULL) grad_x0[q][N] = dL_q/dx0.  targets[q] has the layout of
   inst[q].out, which also receives the forward trajectory.  Backward-Euler
   steps are differentiated as exactly solved; steps that reverted species
   or failed to factor are treated as the identity.  Accepted RKF45 steps
   store their output every ckpt_every steps (0 = 8) and are recomputed in
   between; max_record caps the recorded steps per instance (0 = 100000).
   opts->controller must be LASSIE_CTRL_COMPAT (LASSIE_ERR_ARGS otherwise). */
int lassie_adjoint_batch(const lassie_instance *inst, int32_t n, const double *const *targets,
                         const lassie_opts *opts, int32_t ckpt_every, int32_t max_record,
                         double *loss, double *const *grad_logk, double *const *grad_x0,
                         lassie_stats *stats);

/* Self-test of the tensor-core (tcgen05) tile product, one K = 32 chunk of
   the wide engine's rank-128 updates (no reference counterpart): on device buffers,
   D[128 x 128] = A[128 x 32] * B[32 x 128], row-major FP32, computed as three
   TF32 products of the operands split into TF32 high and low parts; status[0]
   becomes 1, or 2 if the tensor core did not complete.  Launches one CTA on
   `stream`. */
int lassie_tc_selftest(const float *d_a, const float *d_b, float *d_d, int *d_status,
                       void *stream);
/* The same tile product with BF16 operands (each entry rounded to nearest
   BF16) and FP32 accumulation, two kind::f16 MMAs of K = 16: the wide
   engine's LASSIE_TC_BF16 rank updates (no reference counterpart). */
int lassie_tc_selftest_bf16(const float *d_a, const float *d_b, float *d_d, int *d_status,
                            void *stream);

/* The trailing-update rows per thread that the batch uses for each
   instance (8, 4 or 2; see lassie_opts.tile_rows), rows[n].  Host only. */
int lassie_batch_tile_rows(const lassie_batch *batch, int32_t *rows);

/* One integration that allocates no device memory (no counterpart in the
   reference, which allocates in every solve).  For callers that cannot call
   cudaMalloc: code running under another framework's memory pool that owns
   all device memory, plugins that may not allocate after start-up,
   real-time loops that must not wait on the allocator.  All working memory
   (network structure, descriptor, Newton matrix, result) lives in one
   static device arena of LASSIE_NOALLOC_ARENA_BYTES that every device which
   loads the library keeps until the process exits.  d_k[R], d_x0[N], d_t[nt]
   and d_out[nt*N] (all species sampled) are device buffers owned by the
   caller; stats is host memory (may be NULL).  Networks above the limits
   below are rejected with LASSIE_ERR_TOO_LARGE.  The first call on a device
   looks up the arena's device address and keeps it (it does not survive a
   cudaDeviceReset): make that first call before any stream capture.
   Calls share the arena and keep its last contents (the queue counter and
   the result are cleared per call); calls that overlap on the GPU race, so
   serialise them.  Returns the instance status; synchronises `stream`, and
   therefore returns LASSIE_ERR_ARGS without doing anything while `stream`
   is being captured. */
#define LASSIE_NOALLOC_MAX_SPECIES 128
#define LASSIE_NOALLOC_MAX_REACTIONS 256
#define LASSIE_NOALLOC_MAX_SAMPLES 4096
#define LASSIE_NOALLOC_ARENA_BYTES (512 * 1024)
int lassie_solve_noalloc(const lassie_model *model, const double *d_k, const double *d_x0,
                         const double *d_t, int32_t nt, const lassie_opts *opts, double *d_out,
                         lassie_stats *stats, void *stream);

/* ---------------------------------------------------- single evaluations */
/* dx = f(x) for n_inst parameterisations of one network, device buffers,
   instance-major: k [n_inst][R], x and dx [n_inst][N].  Replaces
   generate_ode (kernels.cuh:5-50). */
int lassie_rhs_device(const lassie_model *model, int32_t n_inst, const double *k,
                      const double *x, double *dx, void *stream);
/* Host-buffer wrappers (one instance) used by parity tests. */
int lassie_rhs(const lassie_model *model, const double *k, const double *x,
               double *dx);
/* M = I - h*J(x), dense row-major N x N FP64, J with the reference's
   createJac semantics (kernels.cuh:205-271, 393-402). */
int lassie_newton_matrix(const lassie_model *model, const double *k,
                         const double *x, double h, double *M);
/* M_b = I - h*J(x_b) for n_inst parameterisations of one network, device
   buffers, instance-major: k [n_inst][R], x [n_inst][N], M [n_inst][N][N]
   row-major, FP64 (precision LASSIE_PREC_FP64) or FP32 (LASSIE_PREC_MIXED,
   the entries rounded once from their FP64 value).  Same entries as
   lassie_newton_matrix.  Replaces the Newton-matrix launches of the
   backward-Euler step, createJac + aggiorna_Jacobiano1 + transposteJacobian
   (Simulation.cuh:828-862; kernels.cuh:206-287, 394-402), for many
   instances at once.  Requires N + R <= 20480. */
int lassie_newton_matrix_device(const lassie_model *model, int32_t n_inst, double h,
                                const double *k, const double *x, void *M,
                                int32_t precision, void *stream);
/* Structural nonzeros of J, the entries createJac fills (kernels.cuh:219-271):
   column g is in row i when a reaction with net stoichiometry in species i
   has g among its reactants.  Host only (no device needed).  The pattern is
   row_ptr[N+1] and cols[nnz] (columns ascending per row), the nonzeros the
   batched Newton-matrix call writes besides the identity. */
int lassie_jacobian_nnz(const lassie_model *model, int64_t *nnz);
int lassie_jacobian_pattern(const lassie_model *model, int32_t *row_ptr, int32_t *cols);
/* Factor a row-major n x n matrix with the engine's LU (precision as in
   lassie_opts) and solve A x = b; returns 1 + column of the first exactly
   zero pivot when singular.  Replaces linearSolverLU (Simulation.cuh:1280). */
int lassie_lu_solve(int32_t n, const double *a, const double *b, double *x,
                    int32_t precision);

#ifdef __cplusplus
}
#endif
#endif
