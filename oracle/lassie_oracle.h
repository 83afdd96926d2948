/*
 * lassie_oracle.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement (plain C, FP64) of the LASSIE deterministic integrator
 * (mass-action RHS, analytic Jacobian, RKF45 with LASSIE's stiffness switch,
 * backward-Euler modified Newton with a dense partial-pivot LU).  It is the
 * checker for the CUDA path: only tests/, the smoke check and the CPU-baseline
 * leg of bench.py may load it.  The product never links or calls it.
 *
 * Arithmetic contract shared with the FP64 CUDA form (so that the two agree
 * bit for bit on the same inputs):
 *   - every expression is evaluated in the order the reference source writes
 *     it, with no contraction (compiled with -ffp-contract=off);
 *   - the LU and the triangular solves accumulate with fma() in ascending
 *     pivot order (forward) and descending order (backward);
 *   - the RKF45 step-size factor (atol/R)^(1/4) is sqrt(sqrt(atol/R)), the
 *     same on every IEEE platform, or (use_pow) pow(atol/R, 0.25) as the
 *     reference writes it, which the C library and CUDA both round
 *     correctly on the golden cases;
 *   - the Newton norm squares are rounded to float before summation, as the
 *     reference's `square` functor does (Simulation.cuh:58-64).
 */
#ifndef LASSIE_ORACLE_H
#define LASSIE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n_species;
    int n_reactions;
    /* reactant CSR by reaction (A), species ascending (Simulation.cuh:1107-1130) */
    int *rxn_ptr;     /* R+1 */
    int *rxn_species; /* nnzA */
    int *rxn_stoich;  /* nnzA */
    /* net-stoichiometry CSR by species (H = (B-A)^T), reaction ascending
       (Simulation.cuh:1061-1105) */
    int *sp_ptr;      /* N+1 */
    int *sp_rxn;      /* nnzH */
    int *sp_coef;     /* nnzH */
    int nnz_a;
    int nnz_h;
} lo_model;

typedef struct {
    double rkf_step;       /* default 1e-3  (Simulation.cuh:281-288) */
    double be_step;        /* default 0.01  (Simulation.cuh:272-279) */
    double newton_tol;     /* default 1e-6  (Simulation.cuh:299-306) */
    double stiffness_tol;  /* default 1e-6  (Simulation.cuh:308-315) */
    int64_t newton_iter;   /* default 10000 (Simulation.cuh:290-297) */
    int64_t max_steps;     /* loop-iteration cap; <=0 means unlimited */
    int32_t use_pow;       /* (atol/R)^(1/4), the reference's pow() call
                              (kernels.cuh:193): 0 (default) sqrt(sqrt());
                              1 the C library's pow(); 2 correctly rounded
                              (lo_qroot_rn) */
    int32_t pad;
} lo_opts;

typedef struct {
    int64_t outer_iters;
    int64_t rkf_accepts;
    int64_t rkf_retries;
    int64_t be_steps;
    int64_t newton_iters;
    int64_t lu_factorisations;
    int64_t lu_failures;
    int64_t nan_reverts;
    double t_final;
    double dt_be_final;
} lo_stats;

/* status codes (shared numbering with the CUDA C-ABI) */
#define LO_OK 0
#define LO_ERR_ARGS (-20)
#define LO_ERR_MAX_STEPS (-21)
#define LO_ERR_ALLOC (-22)

/* Tests only: multiply each Newton correction componentwise by (1 +- rel)
   with seeded signs (rel = 0 turns it off); process-global, not thread safe. */
void lo_set_solve_perturbation(double rel, uint64_t seed);
/* Tests only: move each Newton correction component by +- rel * max|dx|
   instead (a normwise-accurate solver); rel = 0 turns it off. */
void lo_set_solve_perturbation_normwise(double rel, uint64_t seed);
/* Tests only: scale every RKF45 quarter root (atol/R)^(1/4) by (1 +- rel)
   with seeded signs (rel = 0 turns it off); process-global, not thread safe. */
void lo_set_root_perturbation(double rel, uint64_t seed);
/* Tests only: append every Newton right-hand side and correction and every
   accepted RKF45 state to buf (at most cap doubles); NULL turns it off. */
void lo_set_trace(double *buf, int64_t cap);
int64_t lo_trace_len(void);
/* Tests only: pick the LU's rounding order (0 default; 1 the triangular
   solves, 2 the Schur update, 3 both, round products and sums separately
   instead of using fma); process-global, not thread safe. */
void lo_set_lu_variant(int v);

int lo_model_build(int n_reactions, int n_species, const int32_t *left,
                   const int32_t *right, lo_model *out);
void lo_model_free(lo_model *m);

/* x^(1/4) rounded to nearest (x > 0 finite; otherwise sqrt(sqrt(x))) */
double lo_qroot_rn(double x);

/* dx = f(x) -- kernels.cuh:5-63 */
void lo_rhs(const lo_model *m, const double *k, const double *x, double *dx);
/* dense row-major Jacobian J[i*N+g] with the reference's stoichiometry
   handling (kernels.cuh:205-271) */
void lo_jacobian(const lo_model *m, const double *k, const double *x, double *J);
/* in-place LU with partial pivoting on a row-major n x n matrix.
   Returns 0, or j+1 when the pivot of column j is exactly zero. */
int lo_lu_factor(int n, double *a, int *piv);
void lo_lu_solve(int n, const double *lu, const int *piv, double *b);

/* The full integration (Simulation.cuh:632-925).
   k[R], x0[N], feed[N] (may be NULL), atol[N] (may be NULL -> 1e-12),
   t[nt], cs[ncs] (may be NULL -> all species), out[nt*ncs]. */
int lo_solve_compat(const lo_model *m, const double *k, const double *x0,
                    const double *feed, const double *atol, const double *t,
                    int nt, const int *cs, int ncs, const lo_opts *opts,
                    double *out, lo_stats *stats);

/* The reference's -p float loop (Simulation<float>): as lo_solve_compat with
   float state, rate constants, stages, step sizes and Newton matrix and the
   reference's double temporaries; IEEE float division, powf and sqrtf.  The
   perturbation probes apply with float-sized factors (rel = 2^-23 moves a
   float by an ulp). */
int lo_solve_compat_f32(const lo_model *m, const double *k, const double *x0,
                        const double *feed, const double *atol, const double *t,
                        int nt, const int *cs, int ncs, const lo_opts *opts,
                        double *out, lo_stats *stats);

/* As lo_solve_compat, recording the step sequence: kind[n] (0 accepted
   RKF45, 1 backward Euler, 2 state unchanged, 3 reverted species) and dt[n]
   of every state-changing step, *nsteps, and samp[i] = steps taken before
   sample i.  Returns LO_ERR_MAX_STEPS when more than cap steps are taken. */
int lo_solve_compat_rec(const lo_model *m, const double *k, const double *x0,
                        const double *feed, const double *atol, const double *t,
                        int nt, const int *cs, int ncs, const lo_opts *opts,
                        double *out, lo_stats *stats, int cap, int *kind, double *dt,
                        int *nsteps, int *samp);

/* Batch of independent instances solved on `threads` host threads
   (the CPU baseline).  Arrays are per-instance pointers. */
int lo_solve_batch(int n_inst, const lo_model *const *models,
                   const double *const *k, const double *const *x0,
                   const double *const *t, const int *nt,
                   const lo_opts *opts, double *const *out, lo_stats *stats,
                   int *status, int threads);

/* ------------------------------------------------ standard controller
   Variable-order (1..max_order <= 5), quasi-constant-step BDF in backward-
   difference form with rtol/atol error control (Shampine & Reichelt, "The
   MATLAB ODE Suite", 1997, with kappa = 0: plain BDF).  At a constant step h
   and order k its corrector is the classical BDFk formula of the
   reference's unused kernels (kernels.cuh:289-370; BDF5 with the
   denominator 137) and its Newton matrix is I - beta_k h J
   (aggiorna_Jacobiano1..5, kernels.cuh:393-447), beta_k = 1/sum_{j<=k} 1/j.
   J is the exact analytic Jacobian.  Samples come from the interpolating
   polynomial of the differences.  Arithmetic shared with the FP64 CUDA
   form: RMS norms sum like the 512-thread block reduction of the kernel
   (lo_block_sum512), step-size factors are rounded down to multiples of
   2^-10 so that a last-bit difference in pow() cannot change h. */
typedef struct {
    double rtol;          /* relative tolerance (default 1e-6) */
    double atol;          /* absolute tolerance when atol[] is NULL (1e-9) */
    double first_step;    /* 0 = automatic */
    double max_step;      /* 0 = unbounded */
    int32_t max_order;    /* 1..5 (default 5) */
    int32_t pad;
    int64_t max_steps;    /* step attempts; <= 0 unlimited */
} lo_bdf_opts;

typedef struct {
    int64_t steps;             /* accepted */
    int64_t rejected;          /* error-test failures */
    int64_t newton_failures;   /* steps retried after Newton failed */
    int64_t newton_iters;
    int64_t jac_evals;
    int64_t lu_factorisations;
    int64_t rhs_evals;
    int32_t order_final;
    int32_t pad;
    double h_final;
    double t_final;
} lo_bdf_stats;

#define LO_ERR_STEP_TOO_SMALL (-27)

/* Exact dense Jacobian (each other reactant with its stoichiometry), in the
   FP64 CUDA form's operation order. */
void lo_jacobian_exact(const lo_model *m, const double *k, const double *x, double *J);
/* sum of v[0..n) in the order of the CUDA kernels' 512-thread block sum */
double lo_block_sum512(const double *v, int n);
void lo_bdf_opts_default(lo_bdf_opts *o);
/* k[R], x0[N], feed[N] (NULL: none), atol[N] (NULL: opts->atol), t[nt]
   ascending with t[0] the start, cs[ncs] (NULL: all), out[nt*ncs]. */
int lo_solve_bdf(const lo_model *m, const double *k, const double *x0, const double *feed,
                 const double *atol, const double *t, int nt, const int *cs, int ncs,
                 const lo_bdf_opts *opts, double *out, lo_bdf_stats *stats);

#ifdef __cplusplus
}
#endif
#endif
