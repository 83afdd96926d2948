/*
 * lassie_oracle_bdf.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement of the standard (rtol/atol) controller: variable-order,
 * quasi-constant-step BDF in backward-difference form (Shampine & Reichelt,
 * "The MATLAB ODE Suite", SIAM J. Sci. Comput. 18, 1997; kappa = 0).  It is
 * the checker of the CUDA path bdf_integrate, written in the same operation
 * order so that the FP64 CUDA form agrees with it bit for bit.  The
 * constant-step correctors are the classical BDF1-5 formulas of LASSIE's
 * unused kernels (kernels.cuh:289-370, BDF5 with the denominator 137
 * instead of the 147 written there), the Newton matrix is theirs
 * (aggiorna_Jacobiano1..5, kernels.cuh:393-447) with the exact Jacobian.
 *
 * Per step (t -> t + h, order q, differences D[0..q+2]):
 *   prediction  y0 = D[0] + ... + D[q]
 *   psi         = (gamma_1 D[1] + ... + gamma_q D[q]) / gamma_q,
 *               gamma_j = 1 + 1/2 + ... + 1/j
 *   corrector   y = y0 + d with d - c f(y0 + d) + psi = 0,  c = h / gamma_q,
 *               by at most 4 modified Newton iterations on I - c J
 *   error       err = d / (q + 1), RMS norm weighted by atol + rtol |y|
 *   accepted    D[q+2] = d - D[q+1], D[q+1] = d, D[i] += D[i+1] (i = q..0);
 *               after q + 1 equal steps the order moves to whichever of
 *               q-1, q, q+1 allows the largest step
 *   step change D[0..q] <- (R(f) U)^T D[0..q] (interpolation on the new grid)
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "lassie_oracle.h"

enum { kBdfMaxOrder = 5, kNewtonMaxIter = 4, kBlock = 512 };
static const double kMinFactor = 0.2, kMaxFactor = 10.0;

void lo_bdf_opts_default(lo_bdf_opts *o) {
    memset(o, 0, sizeof(*o));
    o->rtol = 1e-6;
    o->atol = 1e-9;
    o->max_order = kBdfMaxOrder;
}

/* kernels.cuh:52-63 (myPow) */
static inline double bdf_pow(double base, int ex) {
    if (ex == 1) return base;
    double p = 1.0;
    while (ex > 0) {
        p = p * base;
        ex--;
    }
    return p;
}

/* Exact Jacobian, the order of assemble_newton_matrix(exact) in the CUDA
   engine: entry (i,g) = 0.0 + the terms of the reactions of H row i in
   ascending order, each s*k [*a*x_g^(a-1)] * x_o^a_o over the other
   reactants o in reactant order. */
void lo_jacobian_exact(const lo_model *m, const double *k, const double *x, double *J) {
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
                if (a == 1) temp = temp + (double)s * k[y];
                else if (a > 1) temp = temp + (double)s * k[y] * (double)a * bdf_pow(x[g], a - 1);
                else continue;
                for (int jj = b; jj < en; jj++)
                    if (m->rxn_species[jj] != g)
                        temp = temp * bdf_pow(x[m->rxn_species[jj]], m->rxn_stoich[jj]);
                row[g] = row[g] + temp;
            }
        }
    }
}

/* The kernels' block_sum over 512 threads: thread t first sums v[t],
   v[t+512], ... onto 0.0; each warp of 32 then adds lane l and lane l^o for
   o = 16, 8, 4, 2, 1; the 16 warp sums are combined the same way with
   o = 8, 4, 2, 1. */
double lo_block_sum512(const double *v, int n) {
    double p[kBlock];
    for (int t = 0; t < kBlock; t++) {
        double a = 0.0;
        for (int s = t; s < n; s += kBlock) a = a + v[s];
        p[t] = a;
    }
    double q[32];
    double w[16];
    for (int wi = 0; wi < 16; wi++) {
        double *x = p + 32 * wi;
        for (int o = 16; o > 0; o >>= 1) {
            for (int l = 0; l < 32; l++) q[l] = x[l] + x[l ^ o];
            memcpy(x, q, sizeof(q));
        }
        w[wi] = x[0];
    }
    for (int o = 8; o > 0; o >>= 1) {
        double r[16];
        for (int l = 0; l < 16; l++) r[l] = w[l] + w[l ^ o];
        memcpy(w, r, sizeof(r));
    }
    return w[0];
}

/* RMS of v[i] / scale[i] */
static double bdf_rms(const double *v, const double *scale, int n, double *tmp) {
    for (int i = 0; i < n; i++) {
        const double q = v[i] / scale[i];
        tmp[i] = q * q;
    }
    return sqrt(lo_block_sum512(tmp, n) / (double)n);
}

/* a step-size factor rounded down to a multiple of 2^-10 */
static inline double bdf_quantize(double f) { return floor(f * 1024.0) / 1024.0; }

/* RU = R(factor) U with R(f)[i][j] = prod_{r=1..i} (r - 1 - f j) / r
   (row 0 and column 0 of the product as the cumulative product of a matrix
   whose first row is 1), U = R(1); then D[0..q] <- RU^T D[0..q]. */
static void bdf_change_d(double *D, int N, int q, double factor) {
    double R[kBdfMaxOrder + 1][kBdfMaxOrder + 1], U[kBdfMaxOrder + 1][kBdfMaxOrder + 1];
    double RU[kBdfMaxOrder + 1][kBdfMaxOrder + 1];
    for (int pass = 0; pass < 2; pass++) {
        const double f = pass == 0 ? factor : 1.0;
        double (*M)[kBdfMaxOrder + 1] = pass == 0 ? R : U;
        for (int j = 0; j <= q; j++) M[0][j] = 1.0;
        for (int i = 1; i <= q; i++)
            for (int j = 0; j <= q; j++) {
                const double mij = j == 0 ? 0.0 : ((double)(i - 1) - f * (double)j) / (double)i;
                M[i][j] = M[i - 1][j] * mij;
            }
    }
    for (int i = 0; i <= q; i++)
        for (int j = 0; j <= q; j++) {
            double a = 0.0;
            for (int l = 0; l <= q; l++) a = a + R[i][l] * U[l][j];
            RU[i][j] = a;
        }
    for (int s = 0; s < N; s++) {
        double nv[kBdfMaxOrder + 1];
        for (int j = 0; j <= q; j++) {
            double a = 0.0;
            for (int i = 0; i <= q; i++) a = a + RU[i][j] * D[(size_t)i * N + s];
            nv[j] = a;
        }
        for (int j = 0; j <= q; j++) D[(size_t)j * N + s] = nv[j];
    }
}

typedef struct {
    const lo_model *m;
    const double *k;
    const unsigned char *fed;
    int64_t *rhs_evals;
} bdf_fun;

/* f(x) with fed species held constant (zero slope) */
static void bdf_f(const bdf_fun *F, const double *x, double *f) {
    lo_rhs(F->m, F->k, x, f);
    (*F->rhs_evals)++;
    if (F->fed)
        for (int s = 0; s < F->m->n_species; s++)
            if (F->fed[s]) f[s] = 0.0;
}

int lo_solve_bdf(const lo_model *m, const double *k, const double *x0, const double *feed,
                 const double *atol_v, const double *t, int nt, const int *cs, int ncs,
                 const lo_bdf_opts *opts_in, double *out, lo_bdf_stats *stats) {
    lo_bdf_opts opts;
    if (opts_in) opts = *opts_in;
    else lo_bdf_opts_default(&opts);
    const int N = m->n_species;
    if (!k || !x0 || !t || nt < 1 || !out || opts.rtol <= 0.0 || opts.max_order < 1 ||
        opts.max_order > kBdfMaxOrder)
        return LO_ERR_ARGS;
    for (int i = 1; i < nt; i++)
        if (!(t[i] >= t[i - 1])) return LO_ERR_ARGS;
    const int ncs_eff = cs ? ncs : N;
    lo_bdf_stats st;
    memset(&st, 0, sizeof(st));

    const int Q = kBdfMaxOrder + 3;
    double *mem = (double *)calloc((size_t)N * (Q + 12) + (size_t)N * N * 2, sizeof(double));
    int *piv = (int *)calloc((size_t)N > 0 ? (size_t)N : 1, sizeof(int));
    unsigned char *fed = feed ? (unsigned char *)calloc((size_t)N, 1) : NULL;
    if (!mem || !piv || (feed && !fed)) {
        free(mem);
        free(piv);
        free(fed);
        return LO_ERR_ALLOC;
    }
    double *D = mem;                    /* Q x N differences */
    double *y = D + (size_t)Q * N;      /* current state */
    double *ypred = y + N, *psi = ypred + N, *d = psi + N, *ynew = d + N;
    double *f = ynew + N, *dy = f + N, *scale = dy + N, *atol = scale + N, *tmp = atol + N;
    double *err = tmp + N, *aux = err + N;
    double *J = aux + N, *LU = J + (size_t)N * N;

    for (int s = 0; s < N; s++) {
        atol[s] = atol_v ? atol_v[s] : opts.atol;
        y[s] = x0[s];
        if (feed && feed[s] != 0.0) {
            fed[s] = 1;
            y[s] = feed[s];
        }
    }
    bdf_fun F = {m, k, fed, &st.rhs_evals};
    const double rtol = opts.rtol;
    const double newton_tol = fmax(10.0 * DBL_EPSILON / rtol, fmin(0.03, sqrt(rtol)));
    double gamma[kBdfMaxOrder + 2], econst[kBdfMaxOrder + 2];
    gamma[0] = 0.0;
    for (int j = 1; j <= kBdfMaxOrder + 1; j++) gamma[j] = gamma[j - 1] + 1.0 / (double)j;
    for (int j = 0; j <= kBdfMaxOrder + 1; j++) econst[j] = 1.0 / (double)(j + 1);

    double tc = t[0];
    const double t_end = t[nt - 1];
    int isample = 0;
    /* samples at the start */
    while (isample < nt && t[isample] <= tc) {
        for (int c = 0; c < ncs_eff; c++) out[(size_t)isample * ncs_eff + c] = y[cs ? cs[c] : c];
        isample++;
    }
    int rc = LO_OK;
    if (isample < nt) {
        bdf_f(&F, y, f);
        /* initial step (Hairer, Norsett & Wanner, II.4, order 1) */
        double h;
        if (opts.first_step > 0.0) {
            h = opts.first_step;
        } else {
            for (int s = 0; s < N; s++) scale[s] = atol[s] + fabs(y[s]) * rtol;
            const double d0 = bdf_rms(y, scale, N, tmp), d1 = bdf_rms(f, scale, N, tmp);
            double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
            h0 = fmin(h0, t_end - tc);
            for (int s = 0; s < N; s++) ynew[s] = y[s] + h0 * f[s];
            bdf_f(&F, ynew, dy);
            for (int s = 0; s < N; s++) aux[s] = dy[s] - f[s];
            const double d2 = bdf_rms(aux, scale, N, tmp) / h0;
            const double h1 = (d1 <= 1e-15 && d2 <= 1e-15) ? fmax(1e-6, h0 * 1e-3)
                                                           : sqrt(0.01 / fmax(d1, d2));
            h = fmin(fmin(100.0 * h0, h1), t_end - tc);
        }
        if (opts.max_step > 0.0 && h > opts.max_step) h = opts.max_step;
        memset(D, 0, sizeof(double) * (size_t)Q * N);
        for (int s = 0; s < N; s++) {
            D[s] = y[s];
            D[N + s] = h * f[s];
        }
        int q = 1, n_equal = 0;
        /* J at the start; it counts as current only within the step that
           evaluated it */
        int jac_current = 0, lu_valid = 0;
        lo_jacobian_exact(m, k, y, J);
        st.jac_evals++;
        if (fed)
            for (int s = 0; s < N; s++)
                if (fed[s]) memset(J + (size_t)s * N, 0, sizeof(double) * N);
        int64_t attempts = 0;
        while (isample < nt) {
            /* one accepted step */
            int accepted = 0;
            int n_iter = 0;
            double err_norm = 0.0;
            while (!accepted) {
                if (opts.max_steps > 0 && attempts >= opts.max_steps) {
                    rc = LO_ERR_MAX_STEPS;
                    goto done;
                }
                attempts++;
                const double min_step = 10.0 * (nextafter(tc, INFINITY) - tc);
                if (opts.max_step > 0.0 && h > opts.max_step) {
                    const double fct = opts.max_step / h;
                    bdf_change_d(D, N, q, fct);
                    h = opts.max_step;
                    n_equal = 0;
                    lu_valid = 0;
                }
                if (h < min_step) {
                    rc = LO_ERR_STEP_TOO_SMALL;
                    goto done;
                }
                double t_new = tc + h;
                if (t_new > t_end) {
                    t_new = t_end;
                    const double fct = (t_end - tc) / h;
                    bdf_change_d(D, N, q, fct);
                    h = t_end - tc;
                    n_equal = 0;
                    lu_valid = 0;
                }
                for (int s = 0; s < N; s++) {
                    double a = D[s];
                    for (int j = 1; j <= q; j++) a = a + D[(size_t)j * N + s];
                    ypred[s] = a;
                    scale[s] = atol[s] + rtol * fabs(a);
                    double p = 0.0;
                    for (int j = 1; j <= q; j++) p = p + gamma[j] * D[(size_t)j * N + s];
                    psi[s] = p / gamma[q];
                }
                const double c = h / gamma[q];
                int converged = 0;
                for (;;) {
                    if (!lu_valid) {
                        for (int i = 0; i < N; i++)
                            for (int g = 0; g < N; g++)
                                LU[(size_t)i * N + g] =
                                    (i == g ? 1.0 : 0.0) - c * J[(size_t)i * N + g];
                        const int info = lo_lu_factor(N, LU, piv);
                        st.lu_factorisations++;
                        lu_valid = info == 0;
                    }
                    converged = 0;
                    n_iter = 0;
                    if (lu_valid) {
                        /* modified Newton from the prediction */
                        memcpy(ynew, ypred, sizeof(double) * N);
                        memset(d, 0, sizeof(double) * N);
                        double dy_old = -1.0;
                        for (int it = 0; it < kNewtonMaxIter; it++) {
                            bdf_f(&F, ynew, f);
                            int finite = 1;
                            for (int s = 0; s < N; s++)
                                if (!isfinite(f[s])) finite = 0;
                            if (!finite) break;
                            for (int s = 0; s < N; s++) dy[s] = c * f[s] - psi[s] - d[s];
                            lo_lu_solve(N, LU, piv, dy);
                            n_iter = it + 1;
                            st.newton_iters++;
                            const double dyn = bdf_rms(dy, scale, N, tmp);
                            double rate = -1.0;
                            if (dy_old >= 0.0) rate = dyn / dy_old;
                            if (rate >= 0.0) {
                                double rp = 1.0;
                                for (int r = 0; r < kNewtonMaxIter - it; r++) rp = rp * rate;
                                if (rate >= 1.0 || rp / (1.0 - rate) * dyn > newton_tol) break;
                            }
                            for (int s = 0; s < N; s++) {
                                ynew[s] = ynew[s] + dy[s];
                                d[s] = d[s] + dy[s];
                            }
                            if (dyn == 0.0 || (rate >= 0.0 && rate / (1.0 - rate) * dyn < newton_tol)) {
                                converged = 1;
                                break;
                            }
                            dy_old = dyn;
                        }
                    }
                    if (converged || jac_current) break;
                    lo_jacobian_exact(m, k, ypred, J);
                    st.jac_evals++;
                    if (fed)
                        for (int s = 0; s < N; s++)
                            if (fed[s]) memset(J + (size_t)s * N, 0, sizeof(double) * N);
                    jac_current = 1;
                    lu_valid = 0;
                }
                if (!converged) {
                    st.newton_failures++;
                    bdf_change_d(D, N, q, 0.5);
                    h = h * 0.5;
                    n_equal = 0;
                    lu_valid = 0;
                    continue;
                }
                const double safety =
                    0.9 * (double)(2 * kNewtonMaxIter + 1) / (double)(2 * kNewtonMaxIter + n_iter);
                for (int s = 0; s < N; s++) {
                    scale[s] = atol[s] + rtol * fabs(ynew[s]);
                    err[s] = econst[q] * d[s];
                }
                err_norm = bdf_rms(err, scale, N, tmp);
                if (err_norm > 1.0) {
                    /* Newton converged: the factors stay (modified Newton
                       with the previous c until the next refactoring) */
                    st.rejected++;
                    double fct = safety * pow(err_norm, -1.0 / (double)(q + 1));
                    fct = bdf_quantize(fmax(kMinFactor, fct));
                    bdf_change_d(D, N, q, fct);
                    h = h * fct;
                    n_equal = 0;
                    continue;
                }
                /* accepted */
                accepted = 1;
                st.steps++;
                n_equal++;
                const double t_old = tc;
                tc = t_new;
                memcpy(y, ynew, sizeof(double) * N);
                jac_current = 0;
                for (int s = 0; s < N; s++) {
                    D[(size_t)(q + 2) * N + s] = d[s] - D[(size_t)(q + 1) * N + s];
                    D[(size_t)(q + 1) * N + s] = d[s];
                }
                for (int i = q; i >= 0; i--)
                    for (int s = 0; s < N; s++)
                        D[(size_t)i * N + s] = D[(size_t)i * N + s] + D[(size_t)(i + 1) * N + s];
                /* samples in (t_old, tc] from the step's interpolant (degree
                   q, before the order and step change below) */
                while (isample < nt && t[isample] <= tc) {
                    const double ts = t[isample];
                    double pj[kBdfMaxOrder + 1];
                    double p = 1.0;
                    for (int j = 0; j < q; j++) {
                        p = p * ((ts - (tc - h * (double)j)) / (h * (double)(1 + j)));
                        pj[j] = p;
                    }
                    for (int c2 = 0; c2 < ncs_eff; c2++) {
                        const int s = cs ? cs[c2] : c2;
                        double a = D[s];
                        if (ts != tc)
                            for (int j = 1; j <= q; j++) a = a + D[(size_t)j * N + s] * pj[j - 1];
                        out[(size_t)isample * ncs_eff + c2] = a;
                    }
                    isample++;
                }
                (void)t_old;
                if (n_equal < q + 1) break;
                /* order and step for the next step */
                double e_m = INFINITY, e_p = INFINITY;
                if (q > 1) {
                    for (int s = 0; s < N; s++) aux[s] = econst[q - 1] * D[(size_t)q * N + s];
                    e_m = bdf_rms(aux, scale, N, tmp);
                }
                if (q < opts.max_order) {
                    for (int s = 0; s < N; s++) aux[s] = econst[q + 1] * D[(size_t)(q + 2) * N + s];
                    e_p = bdf_rms(aux, scale, N, tmp);
                }
                const double en[3] = {e_m, err_norm, e_p};
                double fq[3];
                for (int i = 0; i < 3; i++) {
                    /* err^(-1/(q+i)); err = 0 allows the largest step */
                    fq[i] = en[i] == 0.0 ? INFINITY
                                         : (isinf(en[i]) ? 0.0
                                                         : pow(en[i], -1.0 / (double)(q + i)));
                    fq[i] = bdf_quantize(fmin(kMaxFactor, safety * fq[i]));
                }
                int best = 0;
                for (int i = 1; i < 3; i++)
                    if (fq[i] > fq[best]) best = i;
                q += best - 1;
                const double fct = fq[best];
                h = h * fct;
                bdf_change_d(D, N, q, fct);
                n_equal = 0;
                lu_valid = 0;
            }
        }
        st.order_final = q;
        st.h_final = h;
    }
done:
    st.t_final = tc;
    if (stats) *stats = st;
    free(mem);
    free(piv);
    free(fed);
    return rc;
}
