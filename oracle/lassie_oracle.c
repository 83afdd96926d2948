/*
 * lassie_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement of the LASSIE deterministic integrator.  Each function cites
 * the reference file:line it follows (paths inside the LASSIE project).
 * Build with -ffp-contract=off (see oracle/Makefile): the arithmetic order is
 * part of the contract with the FP64 CUDA form.
 */
#include "lassie_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ model */

/* Simulation.cuh:1061-1130: H = (B-A)^T stored by species with reactions in
   ascending order; A stored by reaction with species in ascending order.
   int32 indices instead of the reference's int16 (no 32767 cap). */
int lo_model_build(int R, int N, const int32_t *left, const int32_t *right,
                   lo_model *m) {
    memset(m, 0, sizeof(*m));
    if (R <= 0 || N <= 0 || !left || !right) return LO_ERR_ARGS;
    m->n_species = N;
    m->n_reactions = R;
    int nnz_a = 0, nnz_h = 0;
    for (int64_t q = 0; q < (int64_t)R * N; q++) {
        if (left[q] != 0) nnz_a++;
        if (right[q] - left[q] != 0) nnz_h++;
    }
    m->nnz_a = nnz_a;
    m->nnz_h = nnz_h;
    m->rxn_ptr = (int *)malloc(sizeof(int) * (R + 1));
    m->rxn_species = (int *)malloc(sizeof(int) * (nnz_a ? nnz_a : 1));
    m->rxn_stoich = (int *)malloc(sizeof(int) * (nnz_a ? nnz_a : 1));
    m->sp_ptr = (int *)malloc(sizeof(int) * (N + 1));
    m->sp_rxn = (int *)malloc(sizeof(int) * (nnz_h ? nnz_h : 1));
    m->sp_coef = (int *)malloc(sizeof(int) * (nnz_h ? nnz_h : 1));
    if (!m->rxn_ptr || !m->rxn_species || !m->rxn_stoich || !m->sp_ptr ||
        !m->sp_rxn || !m->sp_coef) {
        lo_model_free(m);
        return LO_ERR_ALLOC;
    }
    int c = 0;
    for (int j = 0; j < R; j++) {
        m->rxn_ptr[j] = c;
        for (int s = 0; s < N; s++) {
            int a = left[(int64_t)j * N + s];
            if (a != 0) {
                m->rxn_species[c] = s;
                m->rxn_stoich[c] = a;
                c++;
            }
        }
    }
    m->rxn_ptr[R] = c;
    c = 0;
    for (int s = 0; s < N; s++) {
        m->sp_ptr[s] = c;
        for (int j = 0; j < R; j++) {
            int h = right[(int64_t)j * N + s] - left[(int64_t)j * N + s];
            if (h != 0) {
                m->sp_rxn[c] = j;
                m->sp_coef[c] = h;
                c++;
            }
        }
    }
    m->sp_ptr[N] = c;
    return LO_OK;
}

void lo_model_free(lo_model *m) {
    free(m->rxn_ptr);
    free(m->rxn_species);
    free(m->rxn_stoich);
    free(m->sp_ptr);
    free(m->sp_rxn);
    free(m->sp_coef);
    memset(m, 0, sizeof(*m));
}

/* kernels.cuh:52-63 (myPow): repeated multiplication, 1 for ex <= 0 */
static inline double lo_pow(double base, int ex) {
    double p = 1.0;
    while (ex > 0) {
        p = p * base;
        ex--;
    }
    return p;
}

/* kernels.cuh:5-50 (generate_ode).  For species i, each reaction of its H row
   in ascending order contributes ((s*k)*x_a^ea)*x_b^eb..., or s*k for a
   zero-order reaction, added left to right onto 0. */
void lo_rhs(const lo_model *m, const double *k, const double *x, double *dx) {
    const int N = m->n_species;
    for (int i = 0; i < N; i++) {
        double acc = 0.0;
        for (int e = m->sp_ptr[i]; e < m->sp_ptr[i + 1]; e++) {
            const int y = m->sp_rxn[e];
            const int s = m->sp_coef[e];
            const int b = m->rxn_ptr[y], en = m->rxn_ptr[y + 1];
            if (en > b) {
                double temp = 0.0;
                for (int j = b; j < en; j++) {
                    if (j == b)
                        temp += (double)s * k[y] *
                                lo_pow(x[m->rxn_species[j]], m->rxn_stoich[j]);
                    else
                        temp *= lo_pow(x[m->rxn_species[j]], m->rxn_stoich[j]);
                }
                acc = acc + temp;
            } else {
                acc = acc + (double)s * k[y];
            }
        }
        dx[i] = acc;
    }
}

/* kernels.cuh:205-271 (createJac/createJac_).  Entry (i, g) sums, over the
   reactions of H row i in ascending order, the partial derivative of that
   reaction's term with respect to x_g; the other reactants are multiplied in
   once each, whatever their stoichiometry (exact for total order <= 2). */
void lo_jacobian(const lo_model *m, const double *k, const double *x,
                 double *J) {
    const int N = m->n_species;
    memset(J, 0, sizeof(double) * (size_t)N * N);
    for (int i = 0; i < N; i++) {
        double *row = J + (size_t)i * N;
        for (int e = m->sp_ptr[i]; e < m->sp_ptr[i + 1]; e++) {
            const int y = m->sp_rxn[e];
            const int s = m->sp_coef[e];
            const int b = m->rxn_ptr[y], en = m->rxn_ptr[y + 1];
            for (int j = b; j < en; j++) {
                const int g = m->rxn_species[j];
                const int a = m->rxn_stoich[j];
                double temp = 0.0;
                if (a == 1) {
                    temp = temp + (double)s * k[y];
                } else if (a > 1) {
                    temp = temp + (double)s * k[y] * (double)a * lo_pow(x[g], a - 1);
                } else {
                    continue; /* neither branch of kernels.cuh:241/254 */
                }
                for (int jj = b; jj < en; jj++)
                    if (m->rxn_species[jj] != g) temp = temp * x[m->rxn_species[jj]];
                row[g] = row[g] + temp;
            }
        }
    }
}

/* Dense LU with partial pivoting (replaces cusolverDnDgetrf,
   Simulation.cuh:1280-1326).  Pivot = first index of max |a|; failure when the
   pivot is exactly zero (getrf's info > 0).  Right-looking: every trailing
   element is updated as a = fma(-l, u, a) once per pivot, in pivot order. */
/* LU-order variant (tests only, process-global, like the perturbation
   below): 0 the default order above the GPU form shares; 1 the triangular
   solves round the products and sums separately (no fma); 2 the Schur
   update rounds them separately; 3 both.  Each is a valid partial-pivot FP64
   LU solve that differs from the default in the last bits only -- as another
   library's getrf/getrs (the reference calls cuSOLVER) does. */
static int g_lu_variant = 0;

void lo_set_lu_variant(int v) { g_lu_variant = v; }

int lo_lu_factor(int n, double *a, int *piv) {
    const int split = (g_lu_variant & 2) != 0;
    for (int j = 0; j < n; j++) {
        int p = j;
        double best = fabs(a[(size_t)j * n + j]);
        for (int i = j + 1; i < n; i++) {
            double v = fabs(a[(size_t)i * n + j]);
            if (v > best) {
                best = v;
                p = i;
            }
        }
        piv[j] = p;
        if (a[(size_t)p * n + j] == 0.0) return j + 1;
        if (p != j) {
            double *rj = a + (size_t)j * n, *rp = a + (size_t)p * n;
            for (int c = 0; c < n; c++) {
                double tmp = rj[c];
                rj[c] = rp[c];
                rp[c] = tmp;
            }
        }
        const double d = a[(size_t)j * n + j];
        const double *uj = a + (size_t)j * n;
        for (int i = j + 1; i < n; i++) {
            double *ri = a + (size_t)i * n;
            const double l = ri[j] / d;
            ri[j] = l;
            if (split) {
                for (int c = j + 1; c < n; c++) {
                    const double prod = l * uj[c];
                    ri[c] = ri[c] - prod;
                }
            } else {
                for (int c = j + 1; c < n; c++) ri[c] = fma(-l, uj[c], ri[c]);
            }
        }
    }
    return 0;
}

/* getrs with one right-hand side: row interchanges in pivot order, unit-lower
   forward substitution (ascending), upper backward substitution (descending
   accumulation, then one division by the diagonal). */
void lo_lu_solve(int n, const double *lu, const int *piv, double *b) {
    for (int j = 0; j < n; j++) {
        int p = piv[j];
        if (p != j) {
            double tmp = b[j];
            b[j] = b[p];
            b[p] = tmp;
        }
    }
    const int split = (g_lu_variant & 1) != 0;
    for (int i = 0; i < n; i++) {
        double acc = b[i];
        const double *ri = lu + (size_t)i * n;
        if (split) {
            for (int j = 0; j < i; j++) {
                const double prod = ri[j] * b[j];
                acc = acc - prod;
            }
        } else {
            for (int j = 0; j < i; j++) acc = fma(-ri[j], b[j], acc);
        }
        b[i] = acc;
    }
    for (int i = n - 1; i >= 0; i--) {
        double acc = b[i];
        const double *ri = lu + (size_t)i * n;
        if (split) {
            for (int j = n - 1; j > i; j--) {
                const double prod = ri[j] * b[j];
                acc = acc - prod;
            }
        } else {
            for (int j = n - 1; j > i; j--) acc = fma(-ri[j], b[j], acc);
        }
        b[i] = acc / ri[i];
    }
}

/* ------------------------------------------------- quarter root, exactly
   x^(1/4) rounded to nearest, for x > 0 finite: start from sqrt(sqrt(x))
   (within an ulp or two) and move to a neighbour while the midpoint between
   the two lies on the other side of x^(1/4), deciding each step by an exact
   integer comparison of the midpoint's fourth power with x (the midpoint
   m = M 2^e has a 54-bit odd M, so m^4 is never a double and no tie
   occurs). */
typedef struct {
    uint64_t w[4]; /* little-endian 64-bit limbs */
} lo_u256;

static void u256_add_at(lo_u256 *a, int limb, unsigned __int128 v) {
    for (int i = limb; i < 4 && v; i++) {
        unsigned __int128 t = (unsigned __int128)a->w[i] + (uint64_t)v;
        a->w[i] = (uint64_t)t;
        v = (v >> 64) + (t >> 64);
    }
}

static int u256_bitlen(const lo_u256 *a) {
    for (int i = 3; i >= 0; i--)
        if (a->w[i]) return 64 * i + 64 - __builtin_clzll(a->w[i]);
    return 0;
}

/* sign of (M^4 2^(4e)) - (X 2^f), M < 2^55, X < 2^53, both > 0 */
static int cmp_pow4(uint64_t M, int e, uint64_t X, int f) {
    const unsigned __int128 m2 = (unsigned __int128)M * M; /* < 2^110 */
    const uint64_t lo = (uint64_t)m2, hi = (uint64_t)(m2 >> 64);
    lo_u256 P = {{0, 0, 0, 0}};
    u256_add_at(&P, 0, (unsigned __int128)lo * lo);
    u256_add_at(&P, 1, (unsigned __int128)lo * hi);
    u256_add_at(&P, 1, (unsigned __int128)lo * hi);
    u256_add_at(&P, 2, (unsigned __int128)hi * hi);
    const int d = f - 4 * e; /* compare P with X 2^d */
    const int bp = u256_bitlen(&P), bx = 64 - __builtin_clzll(X);
    if (bp != bx + d) return bp > bx + d ? 1 : -1;
    /* same bit length, d = bp - bx >= 0: X << d fits in 256 bits */
    lo_u256 Q = {{0, 0, 0, 0}};
    const int limb = d / 64, sh = d % 64;
    Q.w[limb] = X << sh;
    if (sh && limb + 1 < 4) Q.w[limb + 1] = X >> (64 - sh);
    for (int i = 3; i >= 0; i--)
        if (P.w[i] != Q.w[i]) return P.w[i] > Q.w[i] ? 1 : -1;
    return 0;
}

/* v = V 2^ev with V a 53-bit (or shorter, subnormal) integer */
static void split_double(double v, uint64_t *V, int *ev) {
    int e;
    const double fr = frexp(v, &e);
    *V = (uint64_t)ldexp(fr, 53);
    *ev = e - 53;
}

/* sign of ((a + b) / 2)^4 - x for adjacent positive doubles a < b */
static int mid4_cmp(double a, double x) {
    uint64_t A, X;
    int ea, ex;
    split_double(a, &A, &ea);
    split_double(x, &X, &ex);
    return cmp_pow4(2 * A + 1, ea - 1, X, ex);
}

double lo_qroot_rn(double x) {
    if (!(x > 0) || isinf(x)) return sqrt(sqrt(x));
    double y = sqrt(sqrt(x));
    for (int it = 0; it < 8; it++) {
        const double up = nextafter(y, INFINITY);
        if (mid4_cmp(y, x) < 0) { /* x^(1/4) above the midpoint to up */
            y = up;
            continue;
        }
        const double dn = nextafter(y, 0.0);
        if (dn > 0 && mid4_cmp(dn, x) > 0) { /* below the midpoint to dn */
            y = dn;
            continue;
        }
        break;
    }
    return y;
}

/* ------------------------------------------------------------- integrator */

/* Simulation.cuh:632-925 with kernels.cuh:68-199, 289-300, 393-402, 462-477,
   512-521.  Differences, all documented in the design notes:
   - the stage vector u starts at 0 (the reference never writes u for feed
     species and leaves it uninitialised);
   - the loop stops right after the last sample instead of taking one more
     step with t1 read past the end of t_vector (Simulation.cuh:689);
   - the LU is factored once per backward-Euler step: the reference refactors
     the identical matrix at every Newton iteration, with identical results;
   - the Newton norm sums in index order (thrust's order in the reference);
     only its comparison with newton_tol is used. */
typedef struct {
    int cap;
    int *kind;     /* 0 accepted RKF45, 1 backward Euler, 2 unchanged, 3 reverted */
    double *dt;
    int *nsteps;
    int *samp;     /* steps taken before each sample */
} lo_record;

/* Decision-sensitivity probe (tests only): when g_perturb_rel > 0, every
   Newton correction from the LU solve is multiplied componentwise by
   (1 +- g_perturb_rel), signs from a seeded xorshift stream -- a stand-in for
   a linear solver that differs from this one in the last bits (another LU
   order, cuSOLVER, FP32 LU + refinement).  Process-global and not thread
   safe: set it, solve on one thread, reset it to 0. */
static double g_perturb_rel = 0.0;
static uint64_t g_perturb_state = 0;
static int g_perturb_normwise = 0;

void lo_set_solve_perturbation(double rel, uint64_t seed) {
    g_perturb_rel = rel;
    g_perturb_state = seed * 0x9E3779B97F4A7C15ull + 1;
    g_perturb_normwise = 0;
}

/* The same with every component moved by +- rel * max|dx| (seeded signs):
   a solver whose error is bounded normwise, as an iterative refinement that
   stops on max|correction| <= rel * max|dx| is. */
void lo_set_solve_perturbation_normwise(double rel, uint64_t seed) {
    lo_set_solve_perturbation(rel, seed);
    g_perturb_normwise = rel > 0;
}

/* The same for the RKF45 step-size factor: (atol/R)^(1/4) scaled by
   (1 +- g_root_rel), a quarter root one ulp away from this one on every
   evaluation (the reference's CUDA pow() is not correctly rounded on every
   input). */
static double g_root_rel = 0.0;
static uint64_t g_root_state = 0;

void lo_set_root_perturbation(double rel, uint64_t seed) {
    g_root_rel = rel;
    g_root_state = seed * 0xD1B54A32D192ED03ull + 7;
}

static double lo_root_perturb(double v) {
    uint64_t z = g_root_state;
    z ^= z << 13;
    z ^= z >> 7;
    z ^= z << 17;
    g_root_state = z;
    return v * ((z & 1) ? 1.0 + g_root_rel : 1.0 - g_root_rel);
}

/* Trace (tests only): when set, every Newton right-hand side and correction
   and every accepted RKF45 state is appended to the caller's buffer, to
   compare two builds of this file step by step.  Process-global. */
static double *g_trace = NULL;
static int64_t g_trace_cap = 0, g_trace_n = 0;

void lo_set_trace(double *buf, int64_t cap) {
    g_trace = buf;
    g_trace_cap = buf ? cap : 0;
    g_trace_n = 0;
}

int64_t lo_trace_len(void) { return g_trace_n; }

static void lo_trace(const double *v, int n) {
    if (g_trace && g_trace_n + n <= g_trace_cap) {
        memcpy(g_trace + g_trace_n, v, sizeof(double) * (size_t)n);
        g_trace_n += n;
    }
}

static void lo_perturb(int n, double *dx) {
    double mx = 0.0;
    if (g_perturb_normwise)
        for (int s = 0; s < n; s++)
            if (fabs(dx[s]) > mx) mx = fabs(dx[s]);
    for (int s = 0; s < n; s++) {
        uint64_t z = g_perturb_state;
        z ^= z << 13;
        z ^= z >> 7;
        z ^= z << 17;
        g_perturb_state = z;
        if (g_perturb_normwise)
            dx[s] = dx[s] + ((z & 1) ? g_perturb_rel : -g_perturb_rel) * mx;
        else
            dx[s] = dx[s] * ((z & 1) ? 1.0 + g_perturb_rel : 1.0 - g_perturb_rel);
    }
}

static int lo_solve_impl(const lo_model *m, const double *k, const double *x0,
                         const double *feed, const double *atol, const double *tv,
                         int nt, const int *cs, int ncs, const lo_opts *opts_in,
                         double *out, lo_stats *st_out, lo_record *rec);

int lo_solve_compat(const lo_model *m, const double *k, const double *x0,
                    const double *feed, const double *atol, const double *tv,
                    int nt, const int *cs, int ncs, const lo_opts *opts_in,
                    double *out, lo_stats *st_out) {
    return lo_solve_impl(m, k, x0, feed, atol, tv, nt, cs, ncs, opts_in, out, st_out, NULL);
}

/* As lo_solve_compat, also recording the step sequence (kind and step size
   of every state-changing step, and the steps taken before each sample) for
   the sensitivity checks of the adjoint. */
int lo_solve_compat_rec(const lo_model *m, const double *k, const double *x0,
                        const double *feed, const double *atol, const double *tv,
                        int nt, const int *cs, int ncs, const lo_opts *opts_in,
                        double *out, lo_stats *st_out, int cap, int *kind, double *dt,
                        int *nsteps, int *samp) {
    lo_record r = {cap, kind, dt, nsteps, samp};
    *nsteps = 0;
    return lo_solve_impl(m, k, x0, feed, atol, tv, nt, cs, ncs, opts_in, out, st_out, &r);
}

static int lo_solve_impl(const lo_model *m, const double *k, const double *x0,
                         const double *feed, const double *atol, const double *tv,
                         int nt, const int *cs, int ncs, const lo_opts *opts_in,
                         double *out, lo_stats *st_out, lo_record *rec) {
    lo_opts o;
    if (opts_in)
        o = *opts_in;
    else {
        o.rkf_step = 1e-3;
        o.be_step = 0.01;
        o.newton_tol = 1e-6;
        o.stiffness_tol = 1e-6;
        o.newton_iter = 10000;
        o.max_steps = 0;
        o.use_pow = 0;
        o.pad = 0;
    }
    lo_stats st;
    memset(&st, 0, sizeof(st));
    const int N = m->n_species;
    if (nt < 0 || (nt > 0 && (!tv || !out))) return LO_ERR_ARGS;
    if (!cs) ncs = N;
    for (int j = 0; cs && j < ncs; j++)
        if (cs[j] < 0 || cs[j] >= N) return LO_ERR_ARGS;

    double *buf = (double *)calloc((size_t)N * 16, sizeof(double));
    double *M = (double *)malloc(sizeof(double) * (size_t)N * N);
    int *piv = (int *)malloc(sizeof(int) * (size_t)N);
    if (!buf || !M || !piv) {
        free(buf);
        free(M);
        free(piv);
        return LO_ERR_ALLOC;
    }
    double *y1 = buf, *u = buf + N, *k1 = buf + 2 * N, *k2 = buf + 3 * N,
           *k3 = buf + 4 * N, *k4 = buf + 5 * N, *k5 = buf + 6 * N,
           *k6 = buf + 7 * N, *w1 = buf + 8 * N, *w2 = buf + 9 * N,
           *delta = buf + 10 * N, *yv = buf + 11 * N, *xr = buf + 12 * N,
           *fd = buf + 13 * N, *tol = buf + 14 * N, *dx = buf + 15 * N;
    for (int s = 0; s < N; s++) {
        y1[s] = x0[s];
        fd[s] = feed ? feed[s] : 0.0;
        tol[s] = atol ? atol[s] : 1e-12;
    }

    int status = LO_OK;
    int i = 0;
    double t1 = nt > 0 ? tv[0] : 0.0;
    double t = 0.0;
    double dt = o.rkf_step;
    double newDtBDF = o.be_step;

    while (i < nt) {
        if (o.max_steps > 0 && st.outer_iters >= o.max_steps) {
            status = LO_ERR_MAX_STEPS;
            break;
        }
        st.outer_iters++;
        /* Simulation.cuh:674-690 */
        if (fabs(t1 - t) < 1e-5) {
            for (int j = 0; j < ncs; j++) out[(size_t)i * ncs + j] = y1[cs ? cs[j] : j];
            if (rec) rec->samp[i] = *rec->nsteps;
            i++;
            if (i >= nt) break;
            t1 = tv[i];
        }
        /* RKF45 attempt: Simulation.cuh:692-735, kernels.cuh:68-199 */
        lo_rhs(m, k, y1, k1);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k1[s] = fd[s];
            else {
                k1[s] = k1[s] * dt;
                u[s] = y1[s] + k1[s] / 4.0;
            }
        }
        lo_rhs(m, k, u, k2);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k2[s] = fd[s];
            else {
                k2[s] = k2[s] * dt;
                u[s] = y1[s] + (3.0 * k1[s]) / 32.0 + (9.0 * k2[s]) / 32.0;
            }
        }
        lo_rhs(m, k, u, k3);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k3[s] = fd[s];
            else {
                k3[s] = k3[s] * dt;
                u[s] = y1[s] + (1932.0 * k1[s]) / 2197.0 - (7200.0 * k2[s]) / 2197.0 +
                       (7296.0 * k3[s]) / 2197.0;
            }
        }
        lo_rhs(m, k, u, k4);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k4[s] = fd[s];
            else {
                k4[s] = k4[s] * dt;
                u[s] = y1[s] + (439.0 * k1[s]) / 216.0 - (8.0 * k2[s]) +
                       (3680.0 * k3[s]) / 513.0 - (845.0 * k4[s]) / 4104.0;
            }
        }
        lo_rhs(m, k, u, k5);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k5[s] = fd[s];
            else {
                k5[s] = k5[s] * dt;
                u[s] = y1[s] - (8.0 * k1[s]) / 27.0 + (2.0 * k2[s]) -
                       (3544.0 * k3[s]) / 2565.0 + (1859.0 * k4[s]) / 4104.0 -
                       (11.0 * k5[s]) / 40.0;
            }
        }
        lo_rhs(m, k, u, k6);
        int count = 0;
        double dmin = 0.0;
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k6[s] = fd[s];
            else k6[s] = k6[s] * dt;
            if (fd[s] != 0.0) {
                w1[s] = fd[s];
                w2[s] = fd[s];
            } else {
                w1[s] = y1[s] + (25.0 * k1[s]) / 216.0 + (1408.0 * k3[s]) / 2565.0 +
                        (2197.0 * k4[s]) / 4104.0 - k5[s] / 5.0;
                w2[s] = y1[s] + (16.0 * k1[s]) / 135.0 + (6656.0 * k3[s]) / 12825.0 +
                        (28561.0 * k4[s]) / 56430.0 - (9.0 * k5[s] / 50.0) +
                        (2.0 * k6[s]) / 55.0;
            }
            /* kernels.cuh:184-199 */
            double R = fabs(w1[s] - w2[s]) / dt;
            const double q = tol[s] / R;
            double qr = o.use_pow == 1 ? pow(q, 0.25) : o.use_pow == 2 ? lo_qroot_rn(q)
                                                                       : sqrt(sqrt(q));
            if (g_root_rel > 0) qr = lo_root_perturb(qr);
            delta[s] = 0.84 * qr;
            if (R <= tol[s] && !isnan(R) && !isinf(R) && w1[s] > 0) count++;
            /* thrust::min_element: first element, replaced only by a strictly
               smaller one (a leading NaN therefore sticks) */
            if (s == 0 || delta[s] < dmin) dmin = delta[s];
        }
        if (count == N) {
            /* accept: Simulation.cuh:742-768 */
            memcpy(y1, w1, sizeof(double) * N);
            lo_trace(y1, N);
            if (rec) {
                if (*rec->nsteps >= rec->cap) {
                    status = LO_ERR_MAX_STEPS;
                    break;
                }
                rec->kind[*rec->nsteps] = 0;
                rec->dt[*rec->nsteps] = dt;
                (*rec->nsteps)++;
            }
            double d_temp = dt * dmin;
            if ((t + d_temp) > t1) dt = fabs(t1 - t);
            else dt = d_temp;
            t = t + dt;
            st.rkf_accepts++;
        } else {
            /* reject: Simulation.cuh:769-921 */
            double dt_old = dt;
            dt = dt * dmin;
            if ((dt < o.stiffness_tol) | isnan(dt) | isinf(dt) |
                (fabs(dt_old - dt) < 1e-3)) {
                dt = newDtBDF;
                if ((t + dt) > t1) dt = fabs(t1 - t);
                memcpy(yv, y1, sizeof(double) * N);
                int64_t itN = 0;
                double errN = 1000;
                int luFail = 0;
                st.be_steps++;
                while ((itN < o.newton_iter) & (errN > o.newton_tol)) {
                    lo_rhs(m, k, yv, xr);
                    /* kernels.cuh:289-300 */
                    for (int s = 0; s < N; s++) xr[s] = -(yv[s] - y1[s] - dt * xr[s]);
                    if (itN == 0) {
                        /* kernels.cuh:205-271, 393-402: M = I - dt*J */
                        lo_jacobian(m, k, yv, M);
                        for (int r = 0; r < N; r++)
                            for (int c = 0; c < N; c++) {
                                double I = (r == c) ? 1.0 : 0.0;
                                M[(size_t)r * N + c] = I - dt * M[(size_t)r * N + c];
                            }
                        st.lu_factorisations++;
                        if (lo_lu_factor(N, M, piv) != 0) luFail = 1;
                    }
                    if (luFail) {
                        /* Simulation.cuh:869-875, kernels.cuh:512-521 */
                        for (int s = 0; s < N; s++)
                            if (isnan(yv[s]) || isinf(yv[s]) || yv[s] < 0) yv[s] = y1[s];
                        newDtBDF = dt * 0.1;
                        st.lu_failures++;
                        break;
                    }
                    memcpy(dx, xr, sizeof(double) * N);
                    lo_trace(xr, N);
                    lo_lu_solve(N, M, piv, dx);
                    lo_trace(dx, N);
                    if (g_perturb_rel > 0) lo_perturb(N, dx);
                    /* kernels.cuh:462-477 and Simulation.cuh:883-890 */
                    double sum = 0.0;
                    for (int s = 0; s < N; s++) {
                        double old = yv[s];
                        if (fd[s] == 0) yv[s] = yv[s] + dx[s];
                        else yv[s] = fd[s];
                        dx[s] = yv[s] - old;
                        sum = sum + (double)(float)(dx[s] * dx[s]);
                    }
                    errN = sqrt(sum);
                    itN = itN + 1;
                    st.newton_iters++;
                }
                int reverted = 0;
                if (!luFail) {
                    /* Simulation.cuh:894-909 */
                    int bad = 0;
                    for (int s = 0; s < N; s++)
                        if (isnan(yv[s]) || isinf(yv[s]) || yv[s] < 0) bad++;
                    if (bad > 0) {
                        for (int s = 0; s < N; s++)
                            if (isnan(yv[s]) || isinf(yv[s]) || yv[s] < 0) yv[s] = y1[s];
                        newDtBDF = dt * 0.1;
                        st.nan_reverts++;
                        reverted = 1;
                    }
                }
                if (rec) {
                    if (*rec->nsteps >= rec->cap) {
                        status = LO_ERR_MAX_STEPS;
                        break;
                    }
                    rec->kind[*rec->nsteps] = luFail ? 2 : (reverted ? 3 : 1);
                    rec->dt[*rec->nsteps] = dt;
                    (*rec->nsteps)++;
                }
                memcpy(y1, yv, sizeof(double) * N);
                t = t + dt;
            } else {
                st.rkf_retries++;
            }
        }
    }
    st.t_final = t;
    st.dt_be_final = newDtBDF;
    if (st_out) *st_out = st;
    free(buf);
    free(M);
    free(piv);
    return status;
}

/* ------------------------------------------------------------------ batch */

typedef struct {
    int n_inst;
    const lo_model *const *models;
    const double *const *k;
    const double *const *x0;
    const double *const *t;
    const int *nt;
    const lo_opts *opts;
    double *const *out;
    lo_stats *stats;
    int *status;
    int next;
    pthread_mutex_t mu;
} lo_batch_ctx;

static void *lo_batch_worker(void *arg) {
    lo_batch_ctx *c = (lo_batch_ctx *)arg;
    for (;;) {
        pthread_mutex_lock(&c->mu);
        int q = c->next++;
        pthread_mutex_unlock(&c->mu);
        if (q >= c->n_inst) break;
        c->status[q] = lo_solve_compat(c->models[q], c->k[q], c->x0[q], NULL, NULL,
                                       c->t[q], c->nt[q], NULL, 0, c->opts,
                                       c->out[q], c->stats ? &c->stats[q] : NULL);
    }
    return NULL;
}

int lo_solve_batch(int n_inst, const lo_model *const *models,
                   const double *const *k, const double *const *x0,
                   const double *const *t, const int *nt, const lo_opts *opts,
                   double *const *out, lo_stats *stats, int *status,
                   int threads) {
    if (n_inst < 0 || threads < 1) return LO_ERR_ARGS;
    lo_batch_ctx c;
    c.n_inst = n_inst;
    c.models = models;
    c.k = k;
    c.x0 = x0;
    c.t = t;
    c.nt = nt;
    c.opts = opts;
    c.out = out;
    c.stats = stats;
    c.status = status;
    c.next = 0;
    pthread_mutex_init(&c.mu, NULL);
    if (threads > n_inst) threads = n_inst > 0 ? n_inst : 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    if (!th) return LO_ERR_ALLOC;
    for (int q = 0; q < threads; q++) pthread_create(&th[q], NULL, lo_batch_worker, &c);
    for (int q = 0; q < threads; q++) pthread_join(th[q], NULL);
    free(th);
    pthread_mutex_destroy(&c.mu);
    return LO_OK;
}

/* ------------------------------------------------- single-precision mode
   The reference's -p float (Simulation<float>, simulator.cu:289-294):
   Simulation.cuh:632-925 with T = float.  The state, rate constants, stage
   vectors, step sizes and the Newton matrix are float; C's promotion rules
   put the RHS term products and the RKF45 combinations in double exactly as
   in kernels.cuh (double temporaries, float stores).  IEEE float division,
   powf and sqrtf here; the reference's --use_fast_math build uses faster
   approximations of the first two, so the two agree until the first step
   decision that those last bits move.  The Newton matrix is factored with
   partial pivoting (largest |value|, first on ties) and solved by row
   interchanges, forward and backward substitution; the norm sums the float
   squares in index order. */

static double lo_powf_d(float base, int ex) { /* myPow<float> */
    float potenza = 1.0f;
    while (ex > 0) {
        potenza = potenza * base;
        ex--;
    }
    return potenza;
}

static float lo_rhs_f(const lo_model *m, const float *c, const float *y0, int i) {
    float y1 = 0;
    for (int e = m->sp_ptr[i]; e < m->sp_ptr[i + 1]; e++) {
        const int y = m->sp_rxn[e];
        const int signum = m->sp_coef[e];
        const int b = m->rxn_ptr[y], en = m->rxn_ptr[y + 1];
        double temp = 0;
        if (en > b) {
            for (int j = b; j < en; j++) {
                if (j == b)
                    temp += signum * c[y] * lo_powf_d(y0[m->rxn_species[j]], m->rxn_stoich[j]);
                else
                    temp *= lo_powf_d(y0[m->rxn_species[j]], m->rxn_stoich[j]);
            }
            y1 = y1 + temp;
        } else {
            y1 = y1 + signum * c[y];
        }
    }
    return y1;
}

static float lo_jac_f(const lo_model *m, const float *c, const float *y0, int row, int gid) {
    float y1 = 0;
    for (int e = m->sp_ptr[row]; e < m->sp_ptr[row + 1]; e++) {
        const int y = m->sp_rxn[e];
        const int signum = m->sp_coef[e];
        const int b = m->rxn_ptr[y], en = m->rxn_ptr[y + 1];
        double temp = 0;
        for (int j = b; j < en; j++) {
            const int sp = m->rxn_species[j], st = m->rxn_stoich[j];
            if (st == 1 && sp == gid) {
                temp = temp + signum * c[y];
                for (int jj = b; jj < en; jj++)
                    if (m->rxn_species[jj] != gid) temp = temp * y0[m->rxn_species[jj]];
            } else if (st > 1 && sp == gid) {
                temp = temp + signum * c[y] * st * lo_powf_d(y0[sp], st - 1);
                for (int jj = b; jj < en; jj++)
                    if (m->rxn_species[jj] != gid) temp = temp * y0[m->rxn_species[jj]];
            }
        }
        y1 = y1 + temp;
    }
    return y1;
}

static int lo_bad_f(float v) { return isnan(v) || isinf(v) || v < 0; }

int lo_solve_compat_f32(const lo_model *m, const double *k, const double *x0,
                        const double *feed_in, const double *atol, const double *tv, int nt,
                        const int *cs, int ncs, const lo_opts *opts_in, double *out,
                        lo_stats *st_out) {
    lo_opts o;
    if (opts_in)
        o = *opts_in;
    else {
        o.rkf_step = 1e-3;
        o.be_step = 0.01;
        o.newton_tol = 1e-6;
        o.stiffness_tol = 1e-6;
        o.newton_iter = 10000;
        o.max_steps = 0;
        o.use_pow = 0;
        o.pad = 0;
    }
    lo_stats st;
    memset(&st, 0, sizeof(st));
    const int N = m->n_species, R = m->n_reactions;
    if (nt < 0 || (nt > 0 && (!tv || !out))) return LO_ERR_ARGS;
    float *buf = (float *)calloc((size_t)16 * N + R + (size_t)N * N, sizeof(float));
    int *piv = (int *)calloc((size_t)N + 1, sizeof(int));
    if (!buf || !piv) {
        free(buf);
        free(piv);
        return LO_ERR_ALLOC;
    }
    float *y1 = buf, *u = buf + N, *k1 = buf + 2 * N, *k2 = buf + 3 * N, *k3 = buf + 4 * N,
          *k4 = buf + 5 * N, *k5 = buf + 6 * N, *k6 = buf + 7 * N, *w1 = buf + 8 * N,
          *w2 = buf + 9 * N, *fd = buf + 10 * N, *tol = buf + 11 * N, *yv = buf + 12 * N,
          *x = buf + 13 * N, *dx = buf + 14 * N, *c = buf + 16 * N, *M = c + R;
    for (int j = 0; j < R; j++) c[j] = (float)k[j];
    for (int s = 0; s < N; s++) {
        y1[s] = (float)x0[s];
        fd[s] = feed_in ? (float)feed_in[s] : 0.0f;
        tol[s] = atol ? (float)atol[s] : (float)1e-12;
    }
    const float isStiff = (float)o.stiffness_tol, tollN = (float)o.newton_tol;
    int i = 0, status = LO_OK;
    float t1 = nt > 0 ? (float)tv[0] : 0.0f, t = 0, dt = (float)o.rkf_step;
    float newDtBDF = (float)o.be_step;
    while (i < nt) {
        if (o.max_steps > 0 && st.outer_iters >= o.max_steps) {
            status = LO_ERR_MAX_STEPS;
            break;
        }
        st.outer_iters++;
        if (fabs(t1 - t) < 1e-5) {
            for (int j = 0; j < ncs; j++) out[(size_t)i * ncs + j] = y1[cs ? cs[j] : j];
            i++;
            if (i >= nt) break;
            t1 = (float)tv[i];
        }
        for (int s = 0; s < N; s++) k1[s] = lo_rhs_f(m, c, y1, s);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k1[s] = fd[s];
            else {
                k1[s] = k1[s] * dt;
                u[s] = y1[s] + k1[s] / 4.0;
            }
        }
        for (int s = 0; s < N; s++) k2[s] = lo_rhs_f(m, c, u, s);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k2[s] = fd[s];
            else {
                k2[s] = k2[s] * dt;
                u[s] = y1[s] + (3.0 * k1[s]) / 32.0 + (9.0 * k2[s]) / 32.0;
            }
        }
        for (int s = 0; s < N; s++) k3[s] = lo_rhs_f(m, c, u, s);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k3[s] = fd[s];
            else {
                k3[s] = k3[s] * dt;
                u[s] = y1[s] + (1932.0 * k1[s]) / 2197.0 - (7200.0 * k2[s]) / 2197.0 +
                       (7296.0 * k3[s]) / 2197.0;
            }
        }
        for (int s = 0; s < N; s++) k4[s] = lo_rhs_f(m, c, u, s);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k4[s] = fd[s];
            else {
                k4[s] = k4[s] * dt;
                u[s] = y1[s] + (439.0 * k1[s]) / 216.0 - (8.0 * k2[s]) + (3680.0 * k3[s]) / 513.0 -
                       (845.0 * k4[s]) / 4104.0;
            }
        }
        for (int s = 0; s < N; s++) k5[s] = lo_rhs_f(m, c, u, s);
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k5[s] = fd[s];
            else {
                k5[s] = k5[s] * dt;
                u[s] = y1[s] - (8.0 * k1[s]) / 27.0 + (2.0 * k2[s]) - (3544.0 * k3[s]) / 2565.0 +
                       (1859.0 * k4[s]) / 4104.0 - (11.0 * k5[s]) / 40.0;
            }
        }
        for (int s = 0; s < N; s++) k6[s] = lo_rhs_f(m, c, u, s);
        int count = 0;
        double dmin = 0.0;
        for (int s = 0; s < N; s++) {
            if (fd[s] != 0.0) k6[s] = fd[s];
            else k6[s] = k6[s] * dt;
            if (fd[s] != 0.0) {
                w1[s] = fd[s];
                w2[s] = fd[s];
            } else {
                w1[s] = y1[s] + (25.0 * k1[s]) / 216.0 + (1408.0 * k3[s]) / 2565.0 +
                        (2197.0 * k4[s]) / 4104.0 - k5[s] / 5.0;
                w2[s] = y1[s] + (16.0 * k1[s]) / 135.0 + (6656.0 * k3[s]) / 12825.0 +
                        (28561.0 * k4[s]) / 56430.0 - (9.0 * k5[s] / 50.0) + (2.0 * k6[s]) / 55.0;
            }
            const float Rr = fabsf(w1[s] - w2[s]) / dt;
            const float ex = 0.25f;
            float qr = powf(tol[s] / Rr, ex);
            if (g_root_rel > 0) qr = (float)lo_root_perturb((double)qr);
            const float delta = 0.84 * qr;
            if (Rr <= tol[s] && !isnan(Rr) && !isinf(Rr) && w1[s] > 0) count++;
            const double dd = (double)delta;
            if (s == 0 || dd < dmin) dmin = dd;
        }
        if (count == N) {
            memcpy(y1, w1, sizeof(float) * N);
            float d_temp = (float)dmin;
            d_temp = dt * d_temp;
            if ((t + d_temp) > t1) dt = fabsf(t1 - t);
            else dt = d_temp;
            t = t + dt;
            st.rkf_accepts++;
            continue;
        }
        {
            const float d_temp = (float)dmin;
            const float dt_old = dt;
            dt = dt * d_temp;
            if (!((dt < isStiff) | isnan(dt) | isinf(dt) | (fabsf(dt_old - dt) < 1e-3))) {
                st.rkf_retries++;
                continue;
            }
        }
        dt = newDtBDF;
        if ((t + dt) > t1) dt = fabsf(t1 - t);
        memcpy(yv, y1, sizeof(float) * N);
        st.be_steps++;
        int64_t itN = 0;
        float errN = 1000;
        int luFail = 0;
        while ((itN < o.newton_iter) & (errN > tollN)) {
            for (int s = 0; s < N; s++) x[s] = lo_rhs_f(m, c, yv, s);
            for (int s = 0; s < N; s++) x[s] = -(yv[s] - y1[s] - dt * x[s]);
            if (itN == 0) {
                for (int r = 0; r < N; r++)
                    for (int g = 0; g < N; g++) {
                        const float J = lo_jac_f(m, c, yv, r, g);
                        const float I = (r == g) ? 1.0f : 0.0f;
                        M[(size_t)r * N + g] = I - dt * J;
                    }
                st.lu_factorisations++;
                for (int j = 0; j < N && !luFail; j++) {
                    int p = j;
                    float best = fabsf(M[(size_t)j * N + j]);
                    for (int r = j + 1; r < N; r++) {
                        const float v = fabsf(M[(size_t)r * N + j]);
                        if (v > best) {
                            best = v;
                            p = r;
                        }
                    }
                    piv[j] = p;
                    if (!(best > 0.0f)) {
                        luFail = 1;
                        break;
                    }
                    if (p != j)
                        for (int cc = 0; cc < N; cc++) {
                            const float tmp = M[(size_t)j * N + cc];
                            M[(size_t)j * N + cc] = M[(size_t)p * N + cc];
                            M[(size_t)p * N + cc] = tmp;
                        }
                    const float d = M[(size_t)j * N + j];
                    for (int r = j + 1; r < N; r++) M[(size_t)r * N + j] /= d;
                    for (int r = j + 1; r < N; r++)
                        for (int cc = j + 1; cc < N; cc++)
                            M[(size_t)r * N + cc] -= M[(size_t)r * N + j] * M[(size_t)j * N + cc];
                }
            }
            if (luFail) {
                for (int s = 0; s < N; s++)
                    if (lo_bad_f(yv[s])) yv[s] = y1[s];
                newDtBDF = dt * 0.1f;
                st.lu_failures++;
                break;
            }
            memcpy(dx, x, sizeof(float) * N);
            for (int j = 0; j < N; j++) {
                const int p = piv[j];
                if (p != j) {
                    const float tmp = dx[j];
                    dx[j] = dx[p];
                    dx[p] = tmp;
                }
            }
            for (int r = 0; r < N; r++) {
                float acc = dx[r];
                for (int j = 0; j < r; j++) acc -= M[(size_t)r * N + j] * dx[j];
                dx[r] = acc;
            }
            for (int r = N - 1; r >= 0; r--) {
                float acc = dx[r];
                for (int j = r + 1; j < N; j++) acc -= M[(size_t)r * N + j] * dx[j];
                dx[r] = acc / M[(size_t)r * N + r];
            }
            if (g_perturb_rel > 0)
                for (int s = 0; s < N; s++) {
                    uint64_t z = g_perturb_state;
                    z ^= z << 13;
                    z ^= z >> 7;
                    z ^= z << 17;
                    g_perturb_state = z;
                    dx[s] = dx[s] * ((z & 1) ? 1.0f + (float)g_perturb_rel : 1.0f - (float)g_perturb_rel);
                }
            float sum = 0.0f;
            for (int s = 0; s < N; s++) {
                const float old = yv[s];
                if (fd[s] == 0) yv[s] = yv[s] + dx[s];
                else yv[s] = fd[s];
                dx[s] = yv[s] - old;
                sum = sum + dx[s] * dx[s];
            }
            errN = sqrtf(sum);
            itN = itN + 1;
            st.newton_iters++;
        }
        if (!luFail) {
            int anybad = 0;
            for (int s = 0; s < N; s++) anybad |= lo_bad_f(yv[s]);
            if (anybad) {
                for (int s = 0; s < N; s++)
                    if (lo_bad_f(yv[s])) yv[s] = y1[s];
                newDtBDF = dt * 0.1f;
                st.nan_reverts++;
            }
        }
        memcpy(y1, yv, sizeof(float) * N);
        t = t + dt;
    }
    st.t_final = t;
    st.dt_be_final = newDtBDF;
    if (st_out) *st_out = st;
    free(buf);
    free(piv);
    return status;
}
