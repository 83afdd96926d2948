// Persistent batched integrator with LASSIE's step control.
//
// One CTA of 512 threads integrates one instance at a time, taking instances
// from a work queue (largest first), and runs the reference's whole time loop
// (Simulation.cuh:632-925) on the device: RKF45 attempt, accept/reject,
// stiffness switch, backward-Euler modified Newton with a dense LU of
// M = I - h*J factored once per step.  State, stage vectors, rate constants
// and per-reaction partial products live in shared memory; the Newton matrix
// lives in a per-CTA global workspace (L2-resident at these sizes).
//
// Arithmetic contract (FP64 form, LT = double): every expression is
// evaluated in the reference source's order without contraction (this file
// is compiled with --fmad=false); the LU and triangular solves use explicit
// fma in pivot order.  The CPU oracle follows the same contract, so the two
// agree bit for bit.  Mixed form (LT = float): FP32 LU, FP64 iterative
// refinement against the matrix-free FP64 product M*v = v - h*J(x)*v.
#include <cmath>
#include <cstdint>
#include <type_traits>

#include "common.cuh"

namespace lassie {

// ------------------------------------------------------------ utilities

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// kernels.cuh:52-63 (myPow): repeated multiplication, 1 for ex <= 0.
__device__ __forceinline__ double mypow(double b, int e) {
    if (e == 1) return b;  // 1.0 * b == b exactly
    double p = 1.0;
    while (e > 0) {
        p = p * b;
        --e;
    }
    return p;
}

__device__ __forceinline__ bool bad_value(double v) {
    return isnan(v) || isinf(v) || v < 0;
}

// Mixed form, reuse of FP32 factors across backward-Euler steps: a step
// reuses them when the last solve that used them contracted by kReuseRate or
// better per refinement sweep; a solve with reused factors gives up and
// refactors when a sweep contracts by less than kBailRate.
constexpr double kReuseRate = 2e-3;
constexpr double kBailRate = 2e-2;

template <typename T> __device__ __forceinline__ T lt_fma(T a, T b, T c);
template <> __device__ __forceinline__ float lt_fma(float a, float b, float c) {
    return __fmaf_rn(a, b, c);
}
template <> __device__ __forceinline__ double lt_fma(double a, double b, double c) {
    return __fma_rn(a, b, c);
}

// Block sum of doubles in a fixed order (deterministic run to run).
__device__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    // every warp adds the kWarps partials in the same fixed tree
    double s = l < kWarps ? red[l] : 0.0;
    for (int o = kWarps / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return __shfl_sync(0xffffffffu, s, 0);
}

// Block max of non-negative doubles (NaN propagates), on their IEEE bit
// patterns: for non-negative values the patterns order like the values and
// every NaN pattern sorts above +inf, so no FP64 instruction is needed.
__device__ double block_max(double v, double *red) {
    long long b = __double_as_longlong(fabs(v));
    for (int o = 16; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(0xffffffffu, b, o);
        b = u > b ? u : b;
    }
    long long *ired = reinterpret_cast<long long *>(red);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) ired[w] = b;
    __syncthreads();
    long long s = ired[l < kWarps ? l : 0];
    for (int o = kWarps / 2; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(0xffffffffu, s, o);
        s = u > s ? u : s;
    }
    return __longlong_as_double(__shfl_sync(0xffffffffu, s, 0));
}

// |v| as an IEEE bit pattern, NaN as 0: running maxima of these integers
// equal fmax(acc, fabs(v)) (which ignores a NaN operand) without FP64
// instructions, the slow pipe on this GPU.
__device__ __forceinline__ long long absbits_nonan(double v) {
    const long long b = __double_as_longlong(v) & 0x7fffffffffffffffLL;
    return b > 0x7ff0000000000000LL ? 0 : b;
}

// Block max of two non-negative values at once (same rules as block_max).
__device__ void block_max2(double &a, double &b, double *red) {
    long long x = __double_as_longlong(fabs(a)), y = __double_as_longlong(fabs(b));
    for (int o = 16; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(0xffffffffu, x, o);
        const long long v = __shfl_xor_sync(0xffffffffu, y, o);
        x = u > x ? u : x;
        y = v > y ? v : y;
    }
    long long *ired = reinterpret_cast<long long *>(red);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) {
        ired[w] = x;
        ired[kWarps + w] = y;
    }
    __syncthreads();
    x = ired[l < kWarps ? l : 0];
    y = ired[kWarps + (l < kWarps ? l : 0)];
    for (int o = kWarps / 2; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(0xffffffffu, x, o);
        const long long v = __shfl_xor_sync(0xffffffffu, y, o);
        x = u > x ? u : x;
        y = v > y ? v : y;
    }
    a = __longlong_as_double(__shfl_sync(0xffffffffu, x, 0));
    b = __longlong_as_double(__shfl_sync(0xffffffffu, y, 0));
}

// Block minimum of the non-NaN values among non-negative doubles (+inf if
// none), on bit patterns as above (NaN counts as +inf).
__device__ double block_min_nonnan(double v, double *red) {
    const long long kInf = 0x7ff0000000000000LL;
    long long b = isnan(v) ? kInf : __double_as_longlong(fabs(v));
    for (int o = 16; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(0xffffffffu, b, o);
        b = u < b ? u : b;
    }
    long long *ired = reinterpret_cast<long long *>(red);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) ired[w] = b;
    __syncthreads();
    long long s = ired[l < kWarps ? l : 0];
    for (int o = kWarps / 2; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(0xffffffffu, s, o);
        s = u < s ? u : s;
    }
    return __longlong_as_double(__shfl_sync(0xffffffffu, s, 0));
}

// --------------------------------------------------------------- model

struct Net {
    int n, r, nnz_a;
    const int *rent;  // reactant entries
    const int *sptr;  // species row pointers
    const int *sent;  // species entries
    const int *rptr;               // reaction pointers (shared)
    const double *kk;              // rate constants (shared)
};

// RHS phase 1: pw[q] = x_s^a for every reactant entry q.
__device__ __forceinline__ void rhs_phase1(const Net &m, const double *x, double *pw) {
    for (int q = threadIdx.x; q < m.nnz_a; q += kThreads) {
        const int e = m.rent[q];
        pw[q] = mypow(x[ent_index(e)], ent_coef(e));
    }
}

// RHS phase 2 for species i (kernels.cuh:5-50): over the reactions of its H
// row in ascending order, ((s*k)*pw0)*pw1..., or s*k for zero order, summed
// left to right from 0.  The reference's `temp = 0; temp += ...` differs from
// this only in the sign of a zero, which cannot change the sum.
__device__ __forceinline__ double rhs_species(const Net &m, int i, const double *pw) {
    double acc = 0.0;
    const int e0 = m.sptr[i], e1 = m.sptr[i + 1];
    for (int e = e0; e < e1; e++) {
        const int ent = m.sent[e];
        const int y = ent_index(ent);
        double v = (double)ent_coef(ent) * m.kk[y];
        const int b = m.rptr[y], en = m.rptr[y + 1];
        for (int q = b; q < en; q++) v = v * pw[q];
        acc = acc + v;
    }
    return acc;
}

// The same RHS with the reaction products formed once per reaction:
// rate[y] = ((k_y * pw_0) * pw_1) ... in reactant order, and pw[q] as above.
// A net coefficient of +-1 contributes +-rate[y], which equals the per-entry
// product ((+-1 * k_y) * pw_0) * ... bit for bit (negation commutes with
// rounding); other coefficients use the per-entry product.  On this GPU the
// FP64 pipe, not HBM, bounds the RHS, so the per-entry FP64 work matters.
__device__ __forceinline__ void rhs_rates(const Net &m, const double *x, double *pw,
                                          double *rate) {
    for (int y = threadIdx.x; y < m.r; y += kThreads) {
        double r = m.kk[y];
        for (int q = m.rptr[y]; q < m.rptr[y + 1]; q++) {
            const int e = m.rent[q];
            const double p = mypow(x[ent_index(e)], ent_coef(e));
            pw[q] = p;
            r = r * p;
        }
        rate[y] = r;
    }
}

// The sum starts from its first term instead of 0.0 + term, and a -1 entry
// subtracts (acc - r is acc + (-r) in IEEE arithmetic), so each entry costs
// one FP64 addition.  Only an all-zero sum can differ, in its sign (0.0 +
// -0.0 is +0.0, and no other partial sum is -0.0 in round-to-nearest): the
// last line restores it.
__device__ __forceinline__ double rhs_species_r(const Net &m, int i, const double *pw,
                                                const double *rate) {
    const int e0 = m.sptr[i], e1 = m.sptr[i + 1];
    if (e0 == e1) return 0.0;
    auto scaled = [&](int y, int c) {
        double v = (double)c * m.kk[y];
        for (int q = m.rptr[y]; q < m.rptr[y + 1]; q++) v = v * pw[q];
        return v;
    };
    double acc;
    {
        const int ent = m.sent[e0];
        const int y = ent_index(ent), c = ent_coef(ent);
        acc = c == 1 ? rate[y]
                     : (c == -1 ? __longlong_as_double(__double_as_longlong(rate[y]) ^
                                                       (long long)0x8000000000000000ull)
                                : scaled(y, c));
    }
    for (int e = e0 + 1; e < e1; e++) {
        const int ent = m.sent[e];
        const int y = ent_index(ent), c = ent_coef(ent);
        if (c == 1) acc = acc + rate[y];
        else if (c == -1) acc = acc - rate[y];
        else acc = acc + scaled(y, c);
    }
    if (__double_as_longlong(acc) == (long long)0x8000000000000000ull) acc = 0.0;
    return acc;
}

// (J v)_i for the reference's Jacobian (kernels.cuh:205-271) at x, without
// forming J: per reaction the directional derivative of k*prod(x), with the
// other reactants multiplied in once each as createJac does, then the same
// species sums as the RHS.  Phase 1 writes qr[R].
// exact = true: the exact derivative (the other reactants with their
// stoichiometry), as assemble_newton_matrix(exact) for the BDF controller.
__device__ __forceinline__ double jv_reaction(const Net &m, const double *x, const double *v,
                                               int y, bool exact = false) {
    const int b = m.rptr[y], en = m.rptr[y + 1];
    double q = 0.0;
    for (int j = b; j < en; j++) {
        const int ej = m.rent[j];
        const int g = ent_index(ej), a = ent_coef(ej);
        double d;
        if (a == 1) d = m.kk[y];
        else if (a > 1) d = m.kk[y] * (double)a * mypow(x[g], a - 1);
        else continue;
        for (int jj = b; jj < en; jj++) {
            const int eo = m.rent[jj];
            const int o = ent_index(eo);
            if (o != g) d = exact ? d * mypow(x[o], ent_coef(eo)) : d * x[o];
        }
        q = fma(d, v[g], q);
    }
    return q;
}

__device__ void jv_phase1(const Net &m, const double *x, const double *v, double *qr,
                          bool exact = false) {
    for (int y = threadIdx.x; y < m.r; y += kThreads) qr[y] = jv_reaction(m, x, v, y, exact);
}

__device__ __forceinline__ double jv_species(const Net &m, int i, const double *qr) {
    double acc = 0.0;
    const int e0 = m.sptr[i], e1 = m.sptr[i + 1];
    for (int e = e0; e < e1; e++) {
        const int ent = m.sent[e];
        acc = fma((double)ent_coef(ent), qr[ent_index(ent)], acc);
    }
    return acc;
}

// Vector-Jacobian products with the exact Jacobian of f (adjoint).
// Phase 1, per reaction j: g_j = sum_i S_ij v_i (net stoichiometry by
// reaction), t[q] = d prop_j / d x_{species(q)} * g_j for each reactant entry
// q of j, and, when theta is given, theta_j += h * prop_j(x) * g_j
// (d f / d log k_j = S_:j prop_j).  Phase 2, per species g:
// (J^T v)_g = sum of t[q] over the reactant entries q of species g.
struct AdjNet {
    const int *hrptr;  // [R+1] net stoichiometry by reaction
    const int *hrent;  // species * 256 + coefficient
    const int *asptr;  // [N+1] reactant entries by species
    const int *asent;  // reactant-entry indices q
};

__device__ void jtv_phase1(const Net &m, const AdjNet &a, const double *x, const double *v,
                           double *t, double *theta, double h) {
    for (int j = threadIdx.x; j < m.r; j += kThreads) {
        double g = 0.0;
        for (int e = a.hrptr[j]; e < a.hrptr[j + 1]; e++) {
            const int ent = a.hrent[e];
            g = fma((double)ent_coef(ent), v[ent_index(ent)], g);
        }
        const int b = m.rptr[j], en = m.rptr[j + 1];
        if (theta) {
            double prop = m.kk[j];
            for (int q = b; q < en; q++) prop *= mypow(x[ent_index(m.rent[q])], ent_coef(m.rent[q]));
            theta[j] += h * prop * g;
        }
        for (int q = b; q < en; q++) {
            const int eq = m.rent[q];
            const int sg = ent_index(eq), aq = ent_coef(eq);
            double d = aq > 0 ? m.kk[j] * (double)aq * mypow(x[sg], aq - 1) : 0.0;
            for (int q2 = b; q2 < en; q2++)
                if (q2 != q) d *= mypow(x[ent_index(m.rent[q2])], ent_coef(m.rent[q2]));
            t[q] = d * g;
        }
    }
}

__device__ __forceinline__ double jtv_species(const AdjNet &a, int g, const double *t) {
    double acc = 0.0;
    for (int e = a.asptr[g]; e < a.asptr[g + 1]; e++) acc += t[a.asent[e]];
    return acc;
}

// M = I - h*J(x) into M (row-major, leading dimension ld), J with the
// semantics of createJac + aggiorna_Jacobiano1 (kernels.cuh:205-271,393-402).
// Entry (i,g) accumulates, over the reactions of H row i in ascending order,
// temp = s*k [*a*x_g^(a-1)] * (each other reactant once).
// exact = true (adjoint): the exact derivative (other reactants enter with
// their stoichiometry) and rows i with mask[i] != 0 left as identity rows.
template <typename LT>
__device__ __noinline__ void assemble_newton_matrix(const Net &m, const double *x, double h, LT *M,
                                                    int ld, bool exact = false,
                                                    const double *mask = nullptr) {
    const int N = m.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int row = warp; row < N; row += kWarps) {
        LT *Mr = M + (int64_t)row * ld;
        for (int col = lane; col < ld; col += 32) Mr[col] = (row == col) ? LT(1) : LT(0);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += kThreads) {
        if (mask && mask[i] != 0.0) continue;
        const int e0 = m.sptr[i], e1 = m.sptr[i + 1];
        for (int e = e0; e < e1; e++) {
            const int y = ent_index(m.sent[e]);
            const int b = m.rptr[y], en = m.rptr[y + 1];
            for (int q = b; q < en; q++) {
                const int g = ent_index(m.rent[q]);
                // skip columns already produced by an earlier reaction of row i
                bool seen = false;
                for (int ep = e0; ep < e && !seen; ep++) {
                    const int yp = ent_index(m.sent[ep]);
                    for (int qp = m.rptr[yp]; qp < m.rptr[yp + 1]; qp++)
                        if (ent_index(m.rent[qp]) == g) { seen = true; break; }
                }
                if (seen) continue;
                double J = 0.0;
                for (int e2 = e; e2 < e1; e2++) {
                    const int ent2 = m.sent[e2];
                    const int y2 = ent_index(ent2), s2 = ent_coef(ent2);
                    const int b2 = m.rptr[y2], en2 = m.rptr[y2 + 1];
                    int a = 0;
                    bool has = false;
                    for (int q2 = b2; q2 < en2; q2++) {
                        const int ee = m.rent[q2];
                        if (ent_index(ee) == g) { a = ent_coef(ee); has = true; break; }
                    }
                    if (!has) continue;
                    double temp = 0.0;
                    if (a == 1) temp = temp + (double)s2 * m.kk[y2];
                    else if (a > 1)
                        temp = temp + (double)s2 * m.kk[y2] * (double)a * mypow(x[g], a - 1);
                    else continue;
                    for (int q2 = b2; q2 < en2; q2++) {
                        const int eo = m.rent[q2];
                        const int o = ent_index(eo);
                        if (o != g) temp = exact ? temp * mypow(x[o], ent_coef(eo)) : temp * x[o];
                    }
                    J = J + temp;
                }
                const double I = (i == g) ? 1.0 : 0.0;
                M[(int64_t)i * ld + g] = (LT)(I - h * J);
            }
        }
    }
    __syncthreads();
}

// Diagonal of M = I - h*J(x) in FP64: the entries assemble_newton_matrix
// writes on the diagonal (same Jacobian semantics), before the cast.
__device__ __noinline__ void newton_diag(const Net &m, const double *x, double h, double *out) {
    for (int i = threadIdx.x; i < m.n; i += kThreads) {
        const int e0 = m.sptr[i], e1 = m.sptr[i + 1];
        double J = 0.0;
        for (int e2 = e0; e2 < e1; e2++) {
            const int ent2 = m.sent[e2];
            const int y2 = ent_index(ent2), s2 = ent_coef(ent2);
            const int b2 = m.rptr[y2], en2 = m.rptr[y2 + 1];
            int a = 0;
            for (int q2 = b2; q2 < en2; q2++)
                if (ent_index(m.rent[q2]) == i) { a = ent_coef(m.rent[q2]); break; }
            if (a < 1) continue;
            double temp = 0.0;
            if (a == 1) temp = temp + (double)s2 * m.kk[y2];
            else temp = temp + (double)s2 * m.kk[y2] * (double)a * mypow(x[i], a - 1);
            for (int q2 = b2; q2 < en2; q2++) {
                const int o = ent_index(m.rent[q2]);
                if (o != i) temp = temp * x[o];
            }
            J = J + temp;
        }
        out[i] = 1.0 - h * J;
    }
}

// ------------------------------------------------------------------ LU

// Arg-max of |v| with the oracle's tie and NaN rules, combined over lanes,
// in the factor's own type (FP64 instructions are slow on this GPU, so the
// FP32 factorisation never touches the FP64 pipe here).
template <typename T>
struct PivT {
    T v;
    int i;
};
template <typename T>
__device__ __forceinline__ PivT<T> piv_better(PivT<T> a, PivT<T> b) {
    // larger |value| wins, ties to the smaller index; NaN values never win
    if (b.v > a.v || (b.v == a.v && b.i < a.i)) return b;
    return a;
}

// 8 consecutive LT from 16-byte aligned shared or global memory.
__device__ __forceinline__ void load8(const float *p, float *o) {
    const float4 a = reinterpret_cast<const float4 *>(p)[0];
    const float4 b = reinterpret_cast<const float4 *>(p)[1];
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
}
__device__ __forceinline__ void load8(const double *p, double *o) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const double2 v = reinterpret_cast<const double2 *>(p)[q];
        o[2 * q] = v.x;
        o[2 * q + 1] = v.y;
    }
}
__device__ __forceinline__ void load4(const float *p, float *o) {
    const float4 a = reinterpret_cast<const float4 *>(p)[0];
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
}
__device__ __forceinline__ void load4(const double *p, double *o) {
    const double2 a = reinterpret_cast<const double2 *>(p)[0];
    const double2 b = reinterpret_cast<const double2 *>(p)[1];
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}

// RM consecutive panel entries (RM = 8, 4 or 2; p aligned to RM elements).
template <int RM, typename T>
__device__ __forceinline__ void load_rows(const T *p, T *o) {
    if constexpr (RM == 8) {
        load8(p, o);
    } else if constexpr (RM == 4) {
        load4(p, o);
    } else {
        static_assert(RM == 2, "8, 4 or 2 rows per thread");
        o[0] = p[0];
        o[1] = p[1];
    }
}

__device__ __forceinline__ void store4(float *p, const float *v) {
    reinterpret_cast<float4 *>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void store4(double *p, const double *v) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
}

// In-place blocked right-looking LU with partial pivoting, N <= kThreads, on
// M (row-major, leading dimension ld) with implicit row interchanges: logical
// row i of P*A is physical row perm[i] of M, and no row is ever moved.
// Every element receives a = fma(-l, u, a) once per pivot in pivot order, as
// in the unblocked algorithm, so the factors equal the oracle's bit for bit.
//   panel: shared memory, column-major (lt), one row position per thread;
//          per pivot one barrier publishes the arg-max partials and one the
//          pivot row; thread jj moves the pivot row into place and eliminates
//          the displaced row, so no position has two writers;
//   U12:   unit-lower solve, one column per thread (L11 from lt);
//   trailing update: 128 x 128 tiles, thread (ty,tx) owns rows ty*8.. and
//          columns tx*4..; L21 is read from lt and U12 from a staged tile
//          (utile), both with 16-byte loads.
// Returns 0, or j+1 if the pivot of column j is exactly zero (uniform).
// One column tile of the LU's trailing update A22 -= L21 * U12, RM rows per
// thread (passes of 16*RM rows); every entry sums the same products in the
// same order whatever RM is.
template <typename LT, int RM>
__device__ __forceinline__ void lu_trailing(LT *M, int ld, int N, const int *perm, const LT *lt,
                                            int mp, const LT *utile, int j0, int pb, int c0,
                                            int m2, int tn0, int tx, int ty) {
    constexpr int PB = LuShape<LT>::PB, TN = 128, TM = kWarps * RM;
    for (int tm0 = 0; tm0 < m2; tm0 += TM) {
        const int rl = pb + tm0 + ty * RM;  // row relative to j0
        const int col0 = c0 + tn0 + tx * 4;
        LT acc[RM][4];
#pragma unroll
        for (int a = 0; a < RM; a++) {
            const int r = j0 + rl + a;
            if (r < N && col0 < ld) {
                load4(M + (int64_t)perm[r] * ld + col0, acc[a]);
            } else {
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = LT(0);
            }
        }
#pragma unroll 4
        for (int q = 0; q < PB; q++) {
            LT av[RM], bv[4];
            load_rows<RM>(lt + q * mp + rl, av);
            load4(utile + q * TN + tx * 4, bv);
#pragma unroll
            for (int a = 0; a < RM; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = lt_fma(-av[a], bv[b], acc[a][b]);
        }
#pragma unroll
        for (int a = 0; a < RM; a++) {
            const int r = j0 + rl + a;
            if (r < N) {
#pragma unroll
                for (int b = 0; b < 4; b++)
                    if (col0 + b < N) M[(int64_t)perm[r] * ld + col0 + b] = acc[a][b];
            }
        }
    }
}

// rm: rows per thread of the trailing update's tiles (8, 4 or 2; see
// lu_trailing); the factors do not depend on it (the autotuner picks it per
// network size).
template <typename LT>
__device__ __noinline__ int lu_factor(LT *M, int ld, int N, int *perm, LT *lt, LT *utile,
                                      LT *rowbuf, double *red, int *ired, long long *cyc,
                                      int rm = 8) {
    constexpr int PB = LuShape<LT>::PB;
    constexpr int TN = 128;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    LT *pivrow = rowbuf, *swaprow = rowbuf + PB;
    for (int i = tid; i < N; i += kThreads) perm[i] = i;
    __syncthreads();
    int fail = 0;
    long long c_a = clock64();
    for (int j0 = 0; j0 < N; j0 += PB) {
        const int pb = min(PB, N - j0);
        const int m = N - j0;
        // panel column-major in lt: lt[c*mp + r]; mp = 4 mod 32 keeps the
        // transposed writes conflict-free and rows 16-byte aligned
        const int mp = ((m + 31) & ~31) + 4;
        // thread tid owns panel position tid; its row of the panel lives in
        // registers while the panel is factored (pivot loop fully unrolled)
        LT row[PB];
        const bool own = tid < m;
        if (own) {
            const LT *src = M + (int64_t)perm[j0 + tid] * ld + j0;
            if (pb == PB) {
#pragma unroll
                for (int c = 0; c < PB; c += 4) load4(src + c, row + c);
            } else {
#pragma unroll
                for (int c = 0; c < PB; c++) row[c] = (c < pb) ? src[c] : LT(0);
            }
        } else {
#pragma unroll
            for (int c = 0; c < PB; c++) row[c] = LT(0);
        }
        PivT<LT> best{LT(-1), 1 << 30};
        if (own) {
            const LT v = fabs(row[0]);
            if (!isnan(v)) best = PivT<LT>{v, tid};
        }
        LT *redv = reinterpret_cast<LT *>(red);
#pragma unroll
        for (int jj = 0; jj < PB; jj++) {
            if (jj >= pb) break;
            for (int o = 16; o > 0; o >>= 1) {
                PivT<LT> other{__shfl_xor_sync(0xffffffffu, best.v, o),
                               __shfl_xor_sync(0xffffffffu, best.i, o)};
                best = piv_better(best, other);
            }
            if (lane == 0) {
                redv[warp] = best.v;
                ired[warp] = best.i;
            }
            // a NaN in the diagonal position keeps its own row (oracle rule)
            if (tid == jj) ired[kWarps] = isnan(row[jj]) ? 1 : 0;
            __syncthreads();
            // every warp combines the kWarps partials with shuffles (the order
            // of combination does not matter: piv_better is a total order)
            PivT<LT> all{LT(-1), 1 << 30};
            if (lane < kWarps) all = PivT<LT>{redv[lane], ired[lane]};
            for (int o = kWarps / 2; o > 0; o >>= 1) {
                PivT<LT> other{__shfl_xor_sync(0xffffffffu, all.v, o),
                               __shfl_xor_sync(0xffffffffu, all.i, o)};
                all = piv_better(all, other);
            }
            int p = __shfl_sync(0xffffffffu, all.i, 0);
            if (ired[kWarps] || p >= m) p = jj;
            if (tid == p) {
#pragma unroll
                for (int c = 0; c < PB; c++) pivrow[c] = row[c];
            }
            if (tid == jj && p != jj) {
#pragma unroll
                for (int c = 0; c < PB; c++) swaprow[c] = row[c];
                const int tmp = perm[j0 + jj];
                perm[j0 + jj] = perm[j0 + p];
                perm[j0 + p] = tmp;
            }
            __syncthreads();
            const LT d = pivrow[jj];
            const LT rd = LT(1) / d;
            if (d == LT(0)) {
                fail = j0 + jj + 1;
                break;
            }
            best = PivT<LT>{LT(-1), 1 << 30};
            if (tid == jj) {
                // the pivot row moves to position jj
                if (p != jj) {
#pragma unroll
                    for (int c = 0; c < PB; c++) row[c] = pivrow[c];
                }
            } else if (tid > jj && own) {
                // the displaced row jj goes to position p and is eliminated
                // there; every other position eliminates its own row
                if (tid == p) {
#pragma unroll
                    for (int c = 0; c < PB; c++) row[c] = swaprow[c];
                }
                // a zero multiplier needs no division: 0 * (1/d) is the same
                // signed zero as 0 / d, and most entries of M are zero
                const LT num = row[jj];
                const LT l = (num == LT(0)) ? num * rd : num / d;
                row[jj] = l;
#pragma unroll
                for (int c = jj + 1; c < PB; c++) row[c] = lt_fma(-l, pivrow[c], row[c]);
                if (jj + 1 < pb) {
                    const LT v = fabs(row[jj + 1]);
                    if (!isnan(v)) best = PivT<LT>{v, tid};
                }
            }
        }
        if (fail) break;
        long long c_b = clock64();
        if (tid == 0) cyc[0] += c_b - c_a;
        // panel back to its physical rows, into lt (column-major) for the
        // trailing update, and L11 row-major into utile for the U12 solve
        if (own) {
            LT *dst = M + (int64_t)perm[j0 + tid] * ld + j0;
            if (pb == PB) {
#pragma unroll
                for (int c = 0; c < PB; c += 4) store4(dst + c, row + c);
            } else {
#pragma unroll
                for (int c = 0; c < PB; c++)
                    if (c < pb) dst[c] = row[c];
            }
#pragma unroll
            for (int c = 0; c < PB; c++) lt[c * mp + tid] = row[c];
            if (tid < PB) {
#pragma unroll
                for (int c = 0; c < PB; c++) utile[tid * PB + c] = row[c];
            }
        }
        __syncthreads();
        // U12: unit-lower triangular solve on the panel's rows, one column per
        // thread
        for (int c = j0 + pb + tid; c < N; c += kThreads) {
            LT u[PB];
#pragma unroll
            for (int r = 0; r < PB; r++)
                u[r] = (r < pb) ? M[(int64_t)perm[j0 + r] * ld + c] : LT(0);
#pragma unroll
            for (int r = 1; r < PB; r++) {
                LT acc = u[r];
#pragma unroll
                for (int q4 = 0; q4 < r; q4 += 4) {
                    LT l4[4];
                    load4(utile + r * PB + q4, l4);
#pragma unroll
                    for (int q = q4; q < q4 + 4; q++)
                        if (q < r) acc = lt_fma(-l4[q - q4], u[q], acc);
                }
                u[r] = acc;
            }
#pragma unroll
            for (int r = 1; r < PB; r++)
                if (r < pb) M[(int64_t)perm[j0 + r] * ld + c] = u[r];
        }
        __syncthreads();
        c_a = clock64();
        if (tid == 0) cyc[1] += c_a - c_b;
        // trailing update A22 -= L21 * U12 (pb == PB whenever columns remain)
        const int c0 = j0 + pb;
        const int m2 = N - c0;
        if (m2 > 0) {
            const int tx = tid & 31, ty = tid >> 5;
            for (int tn0 = 0; tn0 < m2; tn0 += TN) {
                for (int idx = tid; idx < PB * TN; idx += kThreads) {
                    const int q = idx / TN, cc = idx - q * TN;
                    const int col = c0 + tn0 + cc;
                    utile[idx] = (col < N) ? M[(int64_t)perm[j0 + q] * ld + col] : LT(0);
                }
                __syncthreads();
                if (rm == 4) lu_trailing<LT, 4>(M, ld, N, perm, lt, mp, utile, j0, pb, c0, m2, tn0, tx, ty);
                else if (rm == 2) lu_trailing<LT, 2>(M, ld, N, perm, lt, mp, utile, j0, pb, c0, m2, tn0, tx, ty);
                else lu_trailing<LT, 8>(M, ld, N, perm, lt, mp, utile, j0, pb, c0, m2, tn0, tx, ty);
                __syncthreads();
            }
        }
        c_b = clock64();
        if (tid == 0) cyc[2] += c_b - c_a;
        c_a = c_b;
    }
    __syncthreads();
    return fail;
}

// Inverse of a 32 x 32 block by the whole CTA: Gauss-Jordan without pivoting
// (the rows arrive in pivot order) on [D | I].  Thread t owns row t / 16 and
// four of the 64 columns in registers; per pivot the pivot value, the scaled
// pivot row and the pivot column pass through shared memory (two buffers,
// alternating), two barriers per pivot.  D is read from Dsrc[r * ds + c]
// (rows/columns at or past nb are the identity), the inverse goes to
// Dinv[r * 32 + c].  xs: 2 * 97 T of scratch.  Returns false (uniformly) if
// a pivot is zero or not finite, or the inverse is not finite.
template <typename T>
__device__ bool cta_block_inverse(const T *Dsrc, int ds, int nb, T *Dinv, T *xs) {
    static_assert(kThreads == 512, "one thread per 4 of the 32 x 64 entries");
    const int t = threadIdx.x, r = t >> 4, c0 = (t & 15) * 4;
    T v[4];
#pragma unroll
    for (int b = 0; b < 4; b++) {
        const int c = c0 + b;
        if (c < 32) v[b] = (r < nb && c < nb) ? Dsrc[r * ds + c] : (r == c ? T(1) : T(0));
        else v[b] = (c - 32 == r) ? T(1) : T(0);
    }
    bool ok = true;
    for (int k = 0; k < 32; k++) {
        T *P = xs + (k & 1) * 97, *F = P + 64, *dd = P + 96;
        const int own = k - c0;
        if (own >= 0 && own < 4) {
            const T x = own == 0 ? v[0] : own == 1 ? v[1] : own == 2 ? v[2] : v[3];
            F[r] = x;
            if (r == k) *dd = x;
        }
        __syncthreads();
        const T d = *dd;
        ok = ok && d != T(0) && isfinite(d);
        if (r == k) {
            const T rd = T(1) / d;
#pragma unroll
            for (int b = 0; b < 4; b++) {
                v[b] = v[b] * rd;
                P[c0 + b] = v[b];
            }
        }
        __syncthreads();
        if (r != k) {
            const T f = F[r];
#pragma unroll
            for (int b = 0; b < 4; b++) v[b] = lt_fma(-f, P[c0 + b], v[b]);
        }
    }
    if (c0 >= 32) {
#pragma unroll
        for (int b = 0; b < 4; b++) {
            ok = ok && isfinite(v[b]);
            Dinv[r * 32 + (c0 - 32) + b] = v[b];
        }
    }
    return __syncthreads_and(ok) != 0;
}

// One column tile of the Gauss-Jordan update over all rows, RM rows per
// thread (passes of 16*RM rows): M[r, C] -= M[r, J] * B for rows that are
// not pivots, pivot rows take B.  Every entry sums the same products in the
// same order whatever RM is.
template <int RM>
__device__ __forceinline__ void gje_trailing(float *M, int ld, int N, const float *lt, int mp,
                                             const float *utile, const int *pos, int ty, int tx,
                                             int col0, bool inJ) {
    constexpr int PB = 32, TN = 128, TM = kWarps * RM;
    for (int tm0 = 0; tm0 < N; tm0 += TM) {
        const int rl = tm0 + ty * RM;
        float acc[RM][4];
#pragma unroll
        for (int a = 0; a < RM; a++) {
            const int r = rl + a;
            if (r < N && col0 < ld && !inJ) {
                load4(M + (int64_t)r * ld + col0, acc[a]);
            } else {
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = 0.f;
            }
        }
#pragma unroll 4
        for (int q = 0; q < PB; q++) {
            float av[RM], bv[4];
            load_rows<RM>(lt + q * mp + rl, av);
            load4(utile + q * TN + tx * 4, bv);
#pragma unroll
            for (int a = 0; a < RM; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = __fmaf_rn(-av[a], bv[b], acc[a][b]);
        }
#pragma unroll
        for (int a = 0; a < RM; a++) {
            const int r = rl + a;
            if (r < N && col0 < ld) {
                const int pr = pos[r];
                if (pr >= 0) load4(utile + pr * TN + tx * 4, acc[a]);
                store4(M + (int64_t)r * ld + col0, acc[a]);
            }
        }
    }
}

// FP32 form: in-place Gauss-Jordan inverse of M (row-major, N <= kThreads)
// with partial pivoting by rows, in kPB-column panels J:
//   pivot rows P_J: per column, the largest |value| among the rows that are
//     not yet pivots, after the panel's earlier columns are eliminated from
//     them (ties to the smaller row, NaN never wins); each candidate keeps
//     its row of the panel in registers;
//   D^-1 of the pivot block D = M[P_J, J] by warp 0 (shuffles);
//   every 128 x 128 tile:  M[i, C] -= M[i, J] * B[:, C]  (i not in P_J),
//     M[i, J] = -M[i, J] * D^-1,  M[P_J, :] = B,  with B = D^-1 M[P_J, C]
//     outside J and D^-1 inside J (M[:, J] is read from a snapshot in lt).
// perm[j] = pivot row of column j; the result X satisfies
// inv(M)[j][perm[k]] = X[perm[j]][k] (gje_apply).  pos: N ints of scratch.
// Returns 0, or j+1 if column j has no nonzero candidate.
// rm: rows per thread of the update tiles (8, 4 or 2; see gje_trailing).
__device__ __noinline__ int gje_factor(float *M, int ld, int N, int *perm, int *pos, float *lt,
                                       float *utile, float *dblk, float *rowbuf, double *red,
                                       int *ired, long long *cyc, int rm = 8) {
    constexpr int PB = 32, TN = 128;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int mp = ((N + 31) & ~31) + 4;  // lt: panel snapshot, column-major
    float *pivrow = rowbuf;
    float *redv = reinterpret_cast<float *>(red);
    for (int i = tid; i < N; i += kThreads) pos[i] = -1;  // -1 candidate, -2 used
    __syncthreads();
    int fail = 0;
    long long c_a = clock64();
    for (int j0 = 0; j0 < N; j0 += PB) {
        const int pb = min(PB, N - j0);
        float row[PB];
        const bool own = tid < N;
        if (own) {
            const float *src = M + (int64_t)tid * ld + j0;
            if (pb == PB) {
#pragma unroll
                for (int c = 0; c < PB; c += 4) load4(src + c, row + c);
            } else {
#pragma unroll
                for (int c = 0; c < PB; c++) row[c] = (c < pb) ? src[c] : 0.f;
            }
#pragma unroll
            for (int c = 0; c < PB; c++) lt[c * mp + tid] = row[c];
        }
        bool cand = own && pos[tid] == -1;
        PivT<float> best{-1.f, 1 << 30};
        if (cand) {
            const float v = fabsf(row[0]);
            if (!isnan(v)) best = PivT<float>{v, tid};
        }
#pragma unroll
        for (int jj = 0; jj < PB; jj++) {
            if (jj >= pb) break;
            for (int o = 16; o > 0; o >>= 1) {
                PivT<float> other{__shfl_xor_sync(0xffffffffu, best.v, o),
                                  __shfl_xor_sync(0xffffffffu, best.i, o)};
                best = piv_better(best, other);
            }
            if (lane == 0) {
                redv[warp] = best.v;
                ired[warp] = best.i;
            }
            __syncthreads();
            PivT<float> all{-1.f, 1 << 30};
            if (lane < kWarps) all = PivT<float>{redv[lane], ired[lane]};
            for (int o = kWarps / 2; o > 0; o >>= 1) {
                PivT<float> other{__shfl_xor_sync(0xffffffffu, all.v, o),
                                  __shfl_xor_sync(0xffffffffu, all.i, o)};
                all = piv_better(all, other);
            }
            const int p = __shfl_sync(0xffffffffu, all.i, 0);
            const float pv = __shfl_sync(0xffffffffu, all.v, 0);
            if (p >= N || !(pv > 0.f)) {  // uniform
                fail = j0 + jj + 1;
                break;
            }
            if (tid == p) {
#pragma unroll
                for (int c = 0; c < PB; c++) pivrow[c] = row[c];
                perm[j0 + jj] = p;
                pos[p] = jj;
                cand = false;
            }
            __syncthreads();
            best = PivT<float>{-1.f, 1 << 30};
            const float rd = 1.f / pivrow[jj];
            if (cand) {
                const float l = row[jj] * rd;
#pragma unroll
                for (int c = jj + 1; c < PB; c++) row[c] = __fmaf_rn(-l, pivrow[c], row[c]);
                if (jj + 1 < pb) {
                    const float v = fabsf(row[jj + 1]);
                    if (!isnan(v)) best = PivT<float>{v, tid};
                }
            }
        }
        if (fail) break;
        // D^-1 (D = M[P_J, J] with its original values) by the whole CTA; the
        // pivot rows' panel values are staged in utile, free until the B tiles
        for (int q = tid; q < PB * PB; q += kThreads) {
            const int r = q / PB, c = q - r * PB;
            utile[r * PB + c] = (r < pb && c < pb) ? M[(int64_t)perm[j0 + r] * ld + j0 + c] : 0.f;
        }
        __syncthreads();
        cta_block_inverse<float>(utile, PB, pb, dblk, utile + PB * PB);
        long long c_b = clock64();
        if (tid == 0) cyc[0] += c_b - c_a;
        // all rows and columns, 128 x 128 tiles
        const int tx = tid & 31, ty = tid >> 5;
        for (int tn0 = 0; tn0 < ld; tn0 += TN) {
            // B tile: stage the pivot rows' tile, then D^-1 times it (columns
            // outside J), D^-1 itself inside J
            for (int idx = tid; idx < PB * TN; idx += kThreads) {
                const int q = idx / TN, cc = idx - q * TN;
                const int col = tn0 + cc;
                utile[idx] = (q < pb && col < ld) ? M[(int64_t)perm[j0 + q] * ld + col] : 0.f;
            }
            __syncthreads();
            {
                const int cc = tid & (TN - 1), k0 = (tid >> 7) * 8;  // 128 columns x 4 groups of 8
                const int col = tn0 + cc;
                const bool inJ = col >= j0 && col < j0 + PB;
                float b[8];
#pragma unroll
                for (int kk = 0; kk < 8; kk++) {
                    const int k = k0 + kk;
                    float acc = 0.f;
                    if (inJ) {
                        acc = (k < pb && col - j0 < pb) ? dblk[k * PB + (col - j0)] : 0.f;
                    } else if (k < pb) {
#pragma unroll 8
                        for (int r = 0; r < PB; r++)
                            acc = __fmaf_rn(dblk[k * PB + r], utile[r * TN + cc], acc);
                    }
                    b[kk] = acc;
                }
                __syncthreads();
#pragma unroll
                for (int kk = 0; kk < 8; kk++) utile[(k0 + kk) * TN + cc] = b[kk];
            }
            __syncthreads();
            const int col0 = tn0 + tx * 4;
            const bool inJ = col0 >= j0 && col0 < j0 + PB;
            if (rm == 4) gje_trailing<4>(M, ld, N, lt, mp, utile, pos, ty, tx, col0, inJ);
            else if (rm == 2) gje_trailing<2>(M, ld, N, lt, mp, utile, pos, ty, tx, col0, inJ);
            else gje_trailing<8>(M, ld, N, lt, mp, utile, pos, ty, tx, col0, inJ);
            __syncthreads();
        }
        if (tid < pb) pos[perm[j0 + tid]] = -2;
        __syncthreads();
        c_a = clock64();
        if (tid == 0) cyc[2] += c_a - c_b;
    }
    __syncthreads();
    return fail;
}

// FP32 form: x = inv(M) b with the Gauss-Jordan result X in M: bvec holds
// b[perm[j]] on entry and x on exit; y = X * bvec (ybuf: N floats of
// scratch), then x[j] = y[perm[j]].  Each warp takes 4 rows at a time and
// issues all of their 16-byte loads (N <= 512: at most 4 per row and lane)
// before the first multiply, so a sweep waits for few L2 round trips.
__device__ __noinline__ void gje_apply(const float *M, int ld, int N, const int *perm,
                                       float *bvec, float *ybuf, bool gather = true) {
    constexpr int RW = 4, CH = kThreads / 128;  // rows per warp pass, 128-column chunks
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float b[CH][4];
#pragma unroll
    for (int ch = 0; ch < CH; ch++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int c = ch * 128 + lane * 4 + q;
            b[ch][q] = (c < N) ? bvec[c] : 0.f;
        }
    for (int i0 = warp * RW; i0 < N; i0 += kWarps * RW) {
        float4 a[RW][CH];
#pragma unroll
        for (int r = 0; r < RW; r++)
#pragma unroll
            for (int ch = 0; ch < CH; ch++) {
                const int c = ch * 128 + lane * 4;
                a[r][ch] = (i0 + r < N && c < N)
                               ? *reinterpret_cast<const float4 *>(M + (int64_t)(i0 + r) * ld + c)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        float acc[RW];
#pragma unroll
        for (int r = 0; r < RW; r++) {
            float s = 0.f;
#pragma unroll
            for (int ch = 0; ch < CH; ch++) {
                s = __fmaf_rn(a[r][ch].x, b[ch][0], s);
                s = __fmaf_rn(a[r][ch].y, b[ch][1], s);
                s = __fmaf_rn(a[r][ch].z, b[ch][2], s);
                s = __fmaf_rn(a[r][ch].w, b[ch][3], s);
            }
            acc[r] = s;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int r = 0; r < RW; r++) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
        if (lane < RW && i0 + lane < N) {
            float v = acc[0];
#pragma unroll
            for (int r = 1; r < RW; r++)
                if (lane == r) v = acc[r];
            ybuf[i0 + lane] = v;
        }
    }
    __syncthreads();
    if (!gather) return;  // the caller reads x[j] = ybuf[perm[j]] itself
    for (int j = threadIdx.x; j < N; j += kThreads) bvec[j] = ybuf[perm[j]];
    __syncthreads();
}

// Solve (P A) x = P b with the factors in M; b is in bvec (already permuted),
// overwritten by x.  Forward: ascending accumulation; backward: descending
// accumulation then one division (the oracle's order).  Used by the FP64
// form, whose results must equal the oracle's.
template <typename LT>
__device__ __noinline__ void lu_solve(const LT *M, int ld, int N, const int *perm, LT *bvec) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // forward substitution, unit lower
    for (int r0 = 0; r0 < N; r0 += 32) {
        const int nb = min(32, N - r0);
        if (warp == 0) {
            LT v = (lane < nb) ? bvec[r0 + lane] : LT(0);
            LT row[32];
#pragma unroll
            for (int q = 0; q < 32; q++)
                row[q] = (lane < nb && q < lane) ? M[(int64_t)perm[r0 + lane] * ld + r0 + q] : LT(0);
#pragma unroll
            for (int q = 0; q < 32; q++) {
                const LT bq = __shfl_sync(0xffffffffu, v, q);
                if (q < nb && lane > q && lane < nb) v = lt_fma(-row[q], bq, v);
            }
            if (lane < nb) bvec[r0 + lane] = v;
        }
        __syncthreads();
        for (int i = r0 + nb + tid; i < N; i += kThreads) {
            const LT *ri = M + (int64_t)perm[i] * ld + r0;
            LT seg[32];
#pragma unroll
            for (int q = 0; q < 32; q++) seg[q] = (q < nb) ? ri[q] : LT(0);
            LT acc = bvec[i];
#pragma unroll
            for (int q = 0; q < 32; q++)
                if (q < nb) acc = lt_fma(-seg[q], bvec[r0 + q], acc);
            bvec[i] = acc;
        }
        __syncthreads();
    }
    // backward substitution, upper
    const int nblk = (N + 31) / 32;
    for (int bk = nblk - 1; bk >= 0; bk--) {
        const int r0 = bk * 32;
        const int nb = min(32, N - r0);
        if (warp == 0) {
            LT v = (lane < nb) ? bvec[r0 + lane] : LT(0);
            LT row[32];
#pragma unroll
            for (int q = 0; q < 32; q++)
                row[q] = (lane < nb && q >= lane && q < nb) ? M[(int64_t)perm[r0 + lane] * ld + r0 + q]
                                                            : LT(1);
#pragma unroll
            for (int q = 31; q >= 0; q--) {
                if (q < nb) {
                    LT xq = v / row[q];  // meaningful on lane q only
                    xq = __shfl_sync(0xffffffffu, xq, q);
                    if (lane == q) v = xq;
                    else if (lane < q) v = lt_fma(-row[q], xq, v);
                }
            }
            if (lane < nb) bvec[r0 + lane] = v;
        }
        __syncthreads();
        for (int i = tid; i < r0; i += kThreads) {
            const LT *ri = M + (int64_t)perm[i] * ld + r0;
            LT seg[32];
#pragma unroll
            for (int q = 0; q < 32; q++) seg[q] = (q < nb) ? ri[q] : LT(0);
            LT acc = bvec[i];
#pragma unroll
            for (int q = 31; q >= 0; q--)
                if (q < nb) acc = lt_fma(-seg[q], bvec[r0 + q], acc);
            bvec[i] = acc;
        }
        __syncthreads();
    }
}

// FP32 form: inverses of the 32 x 32 diagonal blocks of L (unit lower) and U,
// dinv[b*2048 + i*32 + j] (L^-1) and dinv[b*2048 + 1024 + i*32 + j] (U^-1);
// rows/columns past N are identity.  One warp per block, lane j builds
// column j by substitution on the block rows held in registers.
__device__ __noinline__ void invert_diag_blocks(const float *M, int ld, int N, const int *perm,
                                                float *dinv) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nblk = (N + 31) / 32;
    for (int b = warp; b < nblk; b += kWarps) {
        const int r0 = b * 32;
        const int nb = min(32, N - r0);
        float row[32];  // row `lane` of the diagonal block (identity past nb)
#pragma unroll
        for (int k = 0; k < 32; k++)
            row[k] = (lane < nb && k < nb) ? M[(int64_t)perm[r0 + lane] * ld + r0 + k]
                                          : (lane == k ? 1.f : 0.f);
        float x[32];
        // L^-1 column `lane`: unit lower
#pragma unroll
        for (int i = 0; i < 32; i++) {
            float acc = (i == lane) ? 1.f : 0.f;
#pragma unroll
            for (int k = 0; k < i; k++)
                acc = __fmaf_rn(-__shfl_sync(0xffffffffu, row[k], i), x[k], acc);
            x[i] = acc;
        }
        float *Li = dinv + (int64_t)b * 2048;
#pragma unroll
        for (int i = 0; i < 32; i++) Li[i * 32 + lane] = x[i];
        // U^-1 column `lane`: upper
#pragma unroll
        for (int i = 31; i >= 0; i--) {
            float acc = (i == lane) ? 1.f : 0.f;
#pragma unroll
            for (int k = i + 1; k < 32; k++)
                acc = __fmaf_rn(-__shfl_sync(0xffffffffu, row[k], i), x[k], acc);
            x[i] = acc * (1.f / __shfl_sync(0xffffffffu, row[i], i));
        }
        float *Ui = Li + 1024;
#pragma unroll
        for (int i = 0; i < 32; i++) Ui[i * 32 + lane] = x[i];
    }
}

// 32 consecutive floats of row r starting at column c0 (c0 % 4 == 0), zero
// past the leading dimension.
__device__ __forceinline__ void load_seg32(const float *M, int ld, int r, int c0, float *seg) {
    const float4 *p = reinterpret_cast<const float4 *>(M + (int64_t)r * ld + c0);
#pragma unroll
    for (int q = 0; q < 8; q++) {
        float4 v = (c0 + 4 * q < ld) ? p[q] : make_float4(0.f, 0.f, 0.f, 0.f);
        seg[4 * q] = v.x;
        seg[4 * q + 1] = v.y;
        seg[4 * q + 2] = v.z;
        seg[4 * q + 3] = v.w;
    }
}

// FP32 form solve, N <= kThreads: thread t owns row t and keeps its running
// value in a register; warp w owns diagonal block w, whose inverse (from
// invert_diag_blocks) it holds in registers from the start.  Forward: at
// step b warp b applies L_bb^-1 and publishes the block's solution through
// a double-buffered shared array (xs, 64 floats); the rows below update with
// the segment of their row in block b, loaded one step ahead.  Backward:
// the same with U.  One barrier per block step.  bvec holds P*b on entry
// and x on exit.
__device__ __noinline__ void lu_solve_fast(const float *M, int ld, int N, const int *perm,
                                           const float *dinv, float *bvec, float *xs) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int nblk = (N + 31) / 32;
    const bool mine = tid < N;
    const int prow = mine ? perm[tid] : 0;
    float acc = mine ? bvec[tid] : 0.f;
    float inv[32], seg[32];
    // forward: unit lower
    if (w < nblk) {
        const float4 *ip = reinterpret_cast<const float4 *>(dinv + (int64_t)w * 2048 + lane * 32);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const float4 v = ip[q];
            inv[4 * q] = v.x; inv[4 * q + 1] = v.y; inv[4 * q + 2] = v.z; inv[4 * q + 3] = v.w;
        }
    }
    if (mine && w > 0) load_seg32(M, ld, prow, 0, seg);
    for (int b = 0; b < nblk; b++) {
        float *xb = xs + (b & 1) * 32;
        if (w == b) {
            float x = 0.f;
#pragma unroll
            for (int k = 0; k < 32; k++) x = __fmaf_rn(inv[k], __shfl_sync(0xffffffffu, acc, k), x);
            acc = x;
            xb[lane] = x;
        }
        __syncthreads();
        if (mine && w > b) {
            const int nb = min(32, N - b * 32);
#pragma unroll
            for (int k = 0; k < 32; k++)
                if (k < nb) acc = __fmaf_rn(-seg[k], xb[k], acc);
            if (b + 1 < w) load_seg32(M, ld, prow, (b + 1) * 32, seg);
        }
    }
    __syncthreads();
    // backward: upper
    if (w < nblk) {
        const float4 *ip =
            reinterpret_cast<const float4 *>(dinv + (int64_t)w * 2048 + 1024 + lane * 32);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const float4 v = ip[q];
            inv[4 * q] = v.x; inv[4 * q + 1] = v.y; inv[4 * q + 2] = v.z; inv[4 * q + 3] = v.w;
        }
    }
    if (mine && w < nblk - 1) load_seg32(M, ld, prow, (nblk - 1) * 32, seg);
    for (int b = nblk - 1; b >= 0; b--) {
        float *xb = xs + (b & 1) * 32;
        if (w == b) {
            float x = 0.f;
#pragma unroll
            for (int k = 0; k < 32; k++) x = __fmaf_rn(inv[k], __shfl_sync(0xffffffffu, acc, k), x);
            acc = x;
            xb[lane] = x;
        }
        __syncthreads();
        if (mine && w < b) {
            const int nb = min(32, N - b * 32);
#pragma unroll
            for (int k = 0; k < 32; k++)
                if (k < nb) acc = __fmaf_rn(-seg[k], xb[k], acc);
            if (b - 1 > w) load_seg32(M, ld, prow, (b - 1) * 32, seg);
        }
    }
    if (mine) bvec[tid] = acc;
    __syncthreads();
}

// Transposed solve with the same factors (adjoint): P A = L U, so
// A^T mu = b is U^T z = b (forward, blocks ascending), L^T w = z (backward),
// mu[perm[i]] = w[i] (done by the caller).  Diagonal blocks are applied as
// the transposes of the inverted blocks; the off-diagonal updates read rows
// of U (resp. L) of the current block, one column per thread.
__device__ __noinline__ void lu_solve_fast_T(const float *M, int ld, int N, const int *perm,
                                             const float *dinv, float *bvec) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nblk = (N + 31) / 32;
    for (int b = 0; b < nblk; b++) {
        const int r0 = b * 32;
        const int nb = min(32, N - r0);
        const int i = r0 + nb + tid;
        float seg[32];
        if (i < N) {
#pragma unroll
            for (int k = 0; k < 32; k++) seg[k] = (k < nb) ? M[(int64_t)perm[r0 + k] * ld + i] : 0.f;
        }
        if (warp == 0) {
            const float *Ui = dinv + (int64_t)b * 2048 + 1024;
            const float bi = (lane < nb) ? bvec[r0 + lane] : 0.f;
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < 32; k++)
                acc = __fmaf_rn(Ui[k * 32 + lane], __shfl_sync(0xffffffffu, bi, k), acc);
            if (lane < nb) bvec[r0 + lane] = acc;
        }
        __syncthreads();
        if (i < N) {
            float acc = bvec[i];
#pragma unroll
            for (int k = 0; k < 32; k++)
                if (k < nb) acc = __fmaf_rn(-seg[k], bvec[r0 + k], acc);
            bvec[i] = acc;
        }
        for (int i2 = i + kThreads; i2 < N; i2 += kThreads) {
            float acc = bvec[i2];
            for (int k = 0; k < nb; k++) acc = __fmaf_rn(-M[(int64_t)perm[r0 + k] * ld + i2], bvec[r0 + k], acc);
            bvec[i2] = acc;
        }
        __syncthreads();
    }
    for (int b = nblk - 1; b >= 0; b--) {
        const int r0 = b * 32;
        const int nb = min(32, N - r0);
        const int i = tid;
        float seg[32];
        if (i < r0) {
#pragma unroll
            for (int k = 0; k < 32; k++) seg[k] = (k < nb) ? M[(int64_t)perm[r0 + k] * ld + i] : 0.f;
        }
        if (warp == 0) {
            const float *Li = dinv + (int64_t)b * 2048;
            const float bi = (lane < nb) ? bvec[r0 + lane] : 0.f;
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < 32; k++)
                acc = __fmaf_rn(Li[k * 32 + lane], __shfl_sync(0xffffffffu, bi, k), acc);
            if (lane < nb) bvec[r0 + lane] = acc;
        }
        __syncthreads();
        if (i < r0) {
            float acc = bvec[i];
#pragma unroll
            for (int k = 0; k < 32; k++)
                if (k < nb) acc = __fmaf_rn(-seg[k], bvec[r0 + k], acc);
            bvec[i] = acc;
        }
        for (int i2 = i + kThreads; i2 < r0; i2 += kThreads) {
            float acc = bvec[i2];
            for (int k = 0; k < nb; k++) acc = __fmaf_rn(-M[(int64_t)perm[r0 + k] * ld + i2], bvec[r0 + k], acc);
            bvec[i2] = acc;
        }
        __syncthreads();
    }
}


// ------------------------------------------------ tuned factorisations
// Rows per thread of the trailing-update tiles, from bits 4-5 of an
// instance's flags (0: 8, 1: 4, 2: 2), as the batch's autotuner chose them.
__device__ __forceinline__ int tile_rows_of(int flags) {
    const int c = (flags >> 4) & 3;
    return c == 1 ? 4 : (c == 2 ? 2 : 8);
}

// ----------------------------------------------------------- integrator

struct Vecs {
    double *y1, *u, *k1, *k2, *k3, *k4, *k5, *k6, *fd, *tol;
};

// RKF45 stage stg (0..4) for species s with f = f(stage input)_s
// (kernels.cuh:68-143): the slope k_{stg+1} = f*dt (the feed for a fed
// species) and the next stage input u, in the reference's expression order.
__device__ __forceinline__ void rkf_stage(int stg, const Vecs &V, int s, double f, double dt) {
    double *k = stg == 0 ? V.k1 : stg == 1 ? V.k2 : stg == 2 ? V.k3 : stg == 3 ? V.k4 : V.k5;
    if (V.fd[s] != 0.0) {
        k[s] = V.fd[s];
        return;
    }
    k[s] = f * dt;
    switch (stg) {
    case 0: V.u[s] = V.y1[s] + V.k1[s] / 4.0; break;
    case 1: V.u[s] = V.y1[s] + (3.0 * V.k1[s]) / 32.0 + (9.0 * V.k2[s]) / 32.0; break;
    case 2:
        V.u[s] = V.y1[s] + (1932.0 * V.k1[s]) / 2197.0 - (7200.0 * V.k2[s]) / 2197.0 +
                 (7296.0 * V.k3[s]) / 2197.0;
        break;
    case 3:
        V.u[s] = V.y1[s] + (439.0 * V.k1[s]) / 216.0 - (8.0 * V.k2[s]) +
                 (3680.0 * V.k3[s]) / 513.0 - (845.0 * V.k4[s]) / 4104.0;
        break;
    default:
        V.u[s] = V.y1[s] - (8.0 * V.k1[s]) / 27.0 + (2.0 * V.k2[s]) -
                 (3544.0 * V.k3[s]) / 2565.0 + (1859.0 * V.k4[s]) / 4104.0 -
                 (11.0 * V.k5[s]) / 40.0;
        break;
    }
}

// Last stage for species s (kernels.cuh:144-199): k6, the 4th- and 5th-order
// solutions w1, w2 (w1 kept in k1 for an accept), the error R = |w1-w2|/dt,
// the accept test, and delta = 0.84 (atol/R)^(1/4); ok, dloc (min delta) and
// d0nan (species 0's delta is NaN) accumulate.
__device__ __forceinline__ void rkf_final(const Vecs &V, int s, double f, double dt,
                                          bool root_sqrt, bool &ok, double &dloc, bool &d0nan) {
    const double fdv = V.fd[s];
    double k6 = (fdv != 0.0) ? fdv : f * dt;
    V.k6[s] = k6;
    double w1, w2;
    if (fdv != 0.0) {
        w1 = fdv;
        w2 = fdv;
    } else {
        w1 = V.y1[s] + (25.0 * V.k1[s]) / 216.0 + (1408.0 * V.k3[s]) / 2565.0 +
             (2197.0 * V.k4[s]) / 4104.0 - V.k5[s] / 5.0;
        w2 = V.y1[s] + (16.0 * V.k1[s]) / 135.0 + (6656.0 * V.k3[s]) / 12825.0 +
             (28561.0 * V.k4[s]) / 56430.0 - (9.0 * V.k5[s] / 50.0) + (2.0 * k6) / 55.0;
    }
    V.k1[s] = w1;  // the 4th-order solution, kept on accept (u untouched)
    const double Rv = fabs(w1 - w2) / dt;
    const double q = V.tol[s] / Rv;
    const double delta = 0.84 * (root_sqrt ? sqrt(sqrt(q)) : pow(q, 0.25));
    if (!(Rv <= V.tol[s] && !isnan(Rv) && !isinf(Rv) && w1 > 0)) ok = false;
    if (s == 0) d0nan = isnan(delta);
    if (delta < dloc) dloc = delta;
}

#include "tc.cuh"
#include "wide.cuh"

// One instance, one CTA (kWide = false: the batched engine, everything in
// shared memory, per-CTA LU), or the leader CTA of the wide engine (kWide:
// vectors in global memory, linear algebra shared with the other CTAs
// through W; wlimit bounds every wait on them).
template <typename LT, bool kWide = false>
__device__ void integrate(const LaunchParams &P, int id, unsigned char *smem, double *red,
                          int *ired, int *mv, InstDesc &D, InstResult &st,
                          uint64_t deadline, const WideWs<LT> *W = nullptr,
                          uint64_t wlimit = 0) {
    constexpr int PB = LuShape<LT>::PB, TN = LuShape<LT>::TN;
    constexpr bool kMixed = std::is_same<LT, float>::value;
    const int tid = threadIdx.x;
    const long long c_start = clock64();
    if (tid == 0) {
        D = P.inst[id];
        st = InstResult{};
    }
    __syncthreads();
    const int N = D.n, R = D.r;
    const int *ia = P.iarena;
    const double *da = P.darena;
    Vecs V;
    double *kk, *pw, *qr;
    const int *rptr, *s_sptr, *s_sent, *s_rent;
    int *perm, *pos = nullptr;
    LT *bvec, *lt = nullptr, *utile = nullptr, *rowbuf = nullptr, *dblk = nullptr;
    int vstride;
    double *vbase;
    if constexpr (kWide) {
        vbase = W->vec;
        vstride = N;
        kk = const_cast<double *>(da + D.k);
        pw = W->pw;
        qr = W->qr;
        rptr = ia + D.rxn_ptr;
        s_sptr = ia + D.sp_ptr;
        s_sent = ia + D.sp_ent;
        s_rent = ia + D.rxn_ent;
        perm = W->piv;
        bvec = W->vin;
    } else {
        const SmemLayout L(P.nmax, P.rmax, P.amax, P.hmax, (int)sizeof(LT), PB, TN);
        vbase = reinterpret_cast<double *>(smem + L.vec);
        vstride = P.nmax;
        kk = reinterpret_cast<double *>(smem + L.kk);
        pw = reinterpret_cast<double *>(smem + L.pw);
        qr = reinterpret_cast<double *>(smem + L.qr);
        int *w_rptr = reinterpret_cast<int *>(smem + L.rptr);
        int *w_sptr = reinterpret_cast<int *>(smem + L.sptr);
        int *w_sent = reinterpret_cast<int *>(smem + L.sent);
        int *w_rent = reinterpret_cast<int *>(smem + L.rent);
        perm = reinterpret_cast<int *>(smem + L.perm);
        bvec = reinterpret_cast<LT *>(smem + L.bvec);
        lt = reinterpret_cast<LT *>(smem + L.lt);
        utile = reinterpret_cast<LT *>(smem + L.utile);
        rowbuf = reinterpret_cast<LT *>(smem + L.rowbuf);
        dblk = reinterpret_cast<LT *>(smem + L.dblk);
        pos = reinterpret_cast<int *>(smem + L.slot);
        for (int q = tid; q < D.nnz_a; q += kThreads) w_rent[q] = ia[D.rxn_ent + q];
        for (int q = tid; q < D.nnz_h; q += kThreads) w_sent[q] = ia[D.sp_ent + q];
        for (int q = tid; q <= N; q += kThreads) w_sptr[q] = ia[D.sp_ptr + q];
        for (int j = tid; j < R; j += kThreads) kk[j] = da[D.k + j];
        for (int j = tid; j <= R; j += kThreads) w_rptr[j] = ia[D.rxn_ptr + j];
        rptr = w_rptr;
        s_sptr = w_sptr;
        s_sent = w_sent;
        s_rent = w_rent;
    }
    V.y1 = vbase;
    V.u = vbase + 1 * vstride;
    V.k1 = vbase + 2 * vstride;
    V.k2 = vbase + 3 * vstride;
    V.k3 = vbase + 4 * vstride;
    V.k4 = vbase + 5 * vstride;
    V.k5 = vbase + 6 * vstride;
    V.k6 = vbase + 7 * vstride;
    V.fd = vbase + 8 * vstride;
    V.tol = vbase + 9 * vstride;

    Net m;
    m.n = N;
    m.r = R;
    m.nnz_a = D.nnz_a;
    m.rent = s_rent;
    m.sptr = s_sptr;
    m.sent = s_sent;
    m.rptr = rptr;
    m.kk = kk;

    for (int s = tid; s < N; s += kThreads) {
        V.y1[s] = da[D.x0 + s];
        V.u[s] = 0.0;  // the reference's stage vector is never written for fed species
        V.fd[s] = D.feed >= 0 ? da[D.feed + s] : 0.0;
        V.tol[s] = D.atol >= 0 ? da[D.atol + s] : 1e-12;
    }
    __syncthreads();

    const double *tv = da + D.t;
    const int *cs = D.cs >= 0 ? ia + D.cs : nullptr;
    double *out = P.out + D.out;
    LT *M = kWide ? nullptr
                  : reinterpret_cast<LT *>(P.workspace + (int64_t)blockIdx.x * P.ws_stride);
    const int ld = round_up4(N);
    // FP32 form: inverted diagonal blocks of the factors follow the matrix
    float *dinv = reinterpret_cast<float *>(M + (int64_t)N * ld);
    int *wflag = ired + kWarps + 1;  // wide engine: join results
    const int refine_max = P.refine_max > 0 ? P.refine_max : 8;
    const bool root_sqrt = (D.flags & 1) != 0;
    const int tile_rows = tile_rows_of(D.flags);
    long long c_mark = 0;

    int64_t outer = 0;  // every thread keeps the loop count (uniform control)
    // forward recording for the adjoint
    const bool rec = P.adj.desc != nullptr;
    AdjDesc AD{};
    if (rec) AD = P.adj.desc[id];
    int nsteps = 0, nstates = 0, rkf_run = 0;
    if (rec) {
        for (int s2 = tid; s2 < N; s2 += kThreads) P.adj.states[AD.states + s2] = V.y1[s2];
        nstates = 1;
    }
    int status = LASSIE_OK;
    int i = 0;
    double t1 = D.nt > 0 ? tv[0] : 0.0;
    double t = 0.0;
    double dt = D.rkf_step;
    double newDt = D.be_step;
    const int nt = D.nt, ncs = D.ncs;
    // mixed form: the factors in M stay valid across backward-Euler steps of
    // the same size; lu_rate is the worst refinement contraction per sweep
    // seen in the last solve that used them
    bool lu_valid = false, wide_abort = false;
    double lu_dt = 0.0, lu_rate = 1.0;

    while (i < nt) {
        if (D.max_steps > 0 && outer >= D.max_steps) {
            status = LASSIE_ERR_MAX_STEPS;
            break;
        }
        if (deadline && (outer & 63) == 0) {
            if (tid == 0) ired[0] = global_ns() > deadline;
            __syncthreads();
            const int expired = ired[0];
            __syncthreads();
            if (expired) {
                status = LASSIE_ERR_DEADLINE;
                break;
            }
        }
        outer++;
        // sampling (Simulation.cuh:674-690)
        if (fabs(t1 - t) < 1e-5) {
            for (int j = tid; j < ncs; j += kThreads)
                out[(int64_t)i * ncs + j] = V.y1[cs ? cs[j] : j];
            if (rec && tid == 0) P.adj.samp_step[AD.samp + i] = nsteps;
            i++;
            if (i >= nt) break;
            t1 = tv[i];
        }
        // ---- RKF45 attempt (Simulation.cuh:692-735, kernels.cuh:68-199)
        c_mark = clock64();
        bool ok = true;
        double dloc = INFINITY;
        bool d0nan = false;
        if constexpr (kWide) {
            // stages spread over the whole grid (fork-join tasks)
            wide_rkf_attempt<LT>(*W, m, V, dt, root_sqrt, pw, qr, wlimit, wflag, ok, dloc, d0nan,
                                 wide_abort);
        } else {
            for (int stg = 0; stg < 5; stg++) {
                rhs_rates(m, stg == 0 ? V.y1 : V.u, pw, qr);
                __syncthreads();
                for (int s = tid; s < N; s += kThreads)
                    rkf_stage(stg, V, s, rhs_species_r(m, s, pw, qr), dt);
                __syncthreads();
            }
            rhs_rates(m, V.u, pw, qr);
            __syncthreads();
            for (int s = tid; s < N; s += kThreads)
                rkf_final(V, s, rhs_species_r(m, s, pw, qr), dt, root_sqrt, ok, dloc, d0nan);
        }
        const int all_ok = __syncthreads_and(ok);
        if (tid == 0) st.cycles_rkf += clock64() - c_mark;
        const int dnan = __syncthreads_or(d0nan);
        double dmin = block_min_nonnan(dloc, red);
        if (dnan) dmin = NAN;  // thrust::min_element keeps a leading NaN
        if (all_ok) {
            // accept (Simulation.cuh:742-768)
            for (int s = tid; s < N; s += kThreads) V.y1[s] = V.k1[s];
            __syncthreads();
            if (rec) {
                if (nsteps >= AD.cap_steps || nstates >= AD.cap_states) {
                    status = LASSIE_ERR_RECORD_FULL;
                    break;
                }
                int slot = -1;
                if (++rkf_run >= P.adj.ckpt_every) {
                    slot = nstates++;
                    rkf_run = 0;
                    for (int s2 = tid; s2 < N; s2 += kThreads)
                        P.adj.states[AD.states + (int64_t)slot * N + s2] = V.y1[s2];
                }
                if (tid == 0) {
                    P.adj.rec_kind[AD.rec + nsteps] = 0;
                    P.adj.rec_dt[AD.rec + nsteps] = dt;
                    P.adj.rec_slot[AD.rec + nsteps] = slot;
                }
                nsteps++;
            }
            const double d_temp = dt * dmin;
            if ((t + d_temp) > t1) dt = fabs(t1 - t);
            else dt = d_temp;
            t = t + dt;
            if (tid == 0) st.rkf_accepts++;
            continue;
        }
        // reject (Simulation.cuh:769-921)
        const double dt_old = dt;
        dt = dt * dmin;
        if (!((dt < D.stiffness_tol) | isnan(dt) | isinf(dt) | (fabs(dt_old - dt) < 1e-3))) {
            if (tid == 0) st.rkf_retries++;
            continue;
        }
        dt = newDt;
        if ((t + dt) > t1) dt = fabs(t1 - t);
        double *yv = V.k2, *xr = V.k3, *dx = V.k4, *xf = V.k5, *res = V.k6, *mdiag = V.k1;
        for (int s = tid; s < N; s += kThreads) yv[s] = V.y1[s];
        __syncthreads();
        int64_t itN = 0;
        double errN = 1000;
        // reused: this step's solves use factors of an earlier step; soft:
        // they use reused factors, or (wide engine) a factorisation with an
        // earlier step's pivot order, so a solve that does not converge asks
        // for a fresh partial-pivoting factorisation
        bool luFail = false, reused = false, soft = false;
        // M = I - dt*J(x) assembled, its diagonal kept in FP64, factored; true
        // if the factorisation met an exactly zero pivot
        auto factor_at = [&](const double *x, bool fresh) -> bool {
            c_mark = clock64();
            bool fail;
            if constexpr (kWide) {
                if (tid == 0) st.lu_factorisations++;
                const int rc = wide_factor<LT>(*W, m, x, dt, fresh, mdiag, smem, red, ired,
                                               wlimit, wflag,
                                               reinterpret_cast<long long *>(&st.cycles_lu_panel));
                if (rc == 2) wide_abort = true;
                fail = rc == 1 || rc == 2;
                soft = rc == 3;
            } else {
                assemble_newton_matrix<LT>(m, x, dt, M, ld);
                for (int s2 = tid; s2 < N; s2 += kThreads)
                    mdiag[s2] = (double)M[(int64_t)s2 * ld + s2];
                if (tid == 0) st.cycles_matrix += clock64() - c_mark;
                if (tid == 0) st.lu_factorisations++;
                if constexpr (kMixed) {
                    // FP32: Gauss-Jordan inverse (each solve is a matrix-vector product)
                    fail = gje_factor(M, ld, N, perm, pos, lt, utile, dblk, rowbuf, red, ired,
                                      reinterpret_cast<long long *>(&st.cycles_lu_panel),
                                      tile_rows) != 0;
                } else {
                    fail = lu_factor<LT>(M, ld, N, perm, lt, utile, rowbuf, red, ired,
                                         reinterpret_cast<long long *>(&st.cycles_lu_panel),
                                         tile_rows) != 0;
                }
                soft = false;
            }
            if constexpr (kMixed) {
                lu_valid = !fail;
                lu_dt = dt;
                lu_rate = 0.0;
            }
            if (tid == 0) st.cycles_lu += clock64() - c_mark;
            return fail;
        };
        if (tid == 0) st.be_steps++;
        bool expired = false;
        // mixed form: a step that reused an earlier step's factors and ends
        // with negative or non-finite species is solved once more from y1
        // with fresh factors before the reference's revert applies (stale
        // factors converge in norm but can leave species far below the others
        // inexact); fresh_only forces the fresh factorisation
        bool fresh_only = false, step_reused = false;
        for (int pass = 0; pass < 2; pass++) {
        if (pass > 0) {
            for (int s = tid; s < N; s += kThreads) yv[s] = V.y1[s];
            __syncthreads();
            itN = 0;
            errN = 1000;
            luFail = false;
            reused = false;
            soft = false;
            fresh_only = true;
            lu_valid = false;
        }
        step_reused = false;
        while ((itN < D.newton_iter) & (errN > D.newton_tol)) {
            if (wide_abort) break;
            if (deadline && (itN & 63) == 63) {
                if (tid == 0) ired[0] = global_ns() > deadline;
                __syncthreads();
                expired = ired[0] != 0;
                __syncthreads();
                if (expired) break;
            }
            // x = f(y_v); x = -(y_v - y1 - h*x)   (kernels.cuh:289-300)
            if constexpr (kWide) {
                if (!wide_newton_rhs<LT>(*W, m, V, dt, itN == 0, wlimit, wflag)) {
                    wide_abort = true;
                    break;
                }
            } else {
                rhs_rates(m, yv, pw, qr);
                __syncthreads();
                for (int s = tid; s < N; s += kThreads) {
                    const double f = rhs_species_r(m, s, pw, qr);
                    xr[s] = -(yv[s] - V.y1[s] - dt * f);
                    if (itN == 0) xf[s] = yv[s];
                }
                __syncthreads();
            }
            if (itN == 0) {
                reused = false;
                if constexpr (kMixed)
                    reused = !fresh_only && P.lu_reuse && lu_valid && dt == lu_dt &&
                             lu_rate <= kReuseRate;
                if (reused) {
                    step_reused = true;
                    // factors of an earlier step precondition this step's
                    // refinement; the diagonal is this step's
                    c_mark = clock64();
                    newton_diag(m, yv, dt, mdiag);
                    __syncthreads();
                    if (tid == 0) st.cycles_matrix += clock64() - c_mark;
                    soft = true;
                } else {
                    luFail = factor_at(yv, false);
                }
            }
            if (luFail) {
                // Simulation.cuh:869-875, kernels.cuh:512-521
                for (int s = tid; s < N; s += kThreads)
                    if (bad_value(yv[s])) yv[s] = V.y1[s];
                __syncthreads();
                newDt = dt * 0.1;
                if (tid == 0) st.lu_failures++;
                break;
            }
            c_mark = clock64();
            if constexpr (!kMixed) {
                for (int s = tid; s < N; s += kThreads) bvec[s] = (LT)xr[perm[s]];
                __syncthreads();
                if constexpr (kWide) {
                    if (!wide_apply<LT>(*W, smem, wlimit, wflag)) wide_abort = true;
                } else {
                    lu_solve<LT>(M, ld, N, perm, bvec);
                }
                for (int s = tid; s < N; s += kThreads) dx[s] = (double)bvec[s];
                __syncthreads();
            } else {
                // FP32 solves, FP64 residuals: dx converges to the FP64 solve.
                // Each residual is scaled by a power of two to unit max norm
                // before the FP32 solve; rows whose scaled residual is below
                // the FP32 normal range (species far below the others) get an
                // FP64 diagonal correction instead, so that they keep their
                // sign and magnitude as in the FP64 solve.
                for (int attempt = 0; attempt < 3; attempt++) {
                    for (int s = tid; s < N; s += kThreads) {
                        dx[s] = 0.0;
                        res[s] = xr[s];
                    }
                    long long rlb = 0;
                    for (int s = tid; s < N; s += kThreads) rlb = max(rlb, absbits_nonan(res[s]));
                    double rmax = block_max(__longlong_as_double(rlb), red);
                    double prev = INFINITY, rate = 0.0;
                    bool converged = false;
                    for (int sweep = 0; sweep < refine_max; sweep++) {
                        if (rmax == 0.0) {  // exact
                            converged = true;
                            break;
                        }
                        // a non-finite residual is solved unscaled, so that
                        // inf/NaN reach the update as in the FP64 solve
                        const bool finite = isfinite(rmax);
                        const int e = finite ? ilogb(rmax) : 0;
                        const double sc = ldexp(1.0, -e), isc = ldexp(1.0, e);
                        // |res| * sc < 2^-126  <=>  |res| < 2^(e-126): bit-pattern bound
                        const int le = e - 126;
                        const long long lost_lim =
                            le >= -1022 ? (long long)(le + 1023) << 52
                                        : (le >= -1074 ? 1LL << (le + 1074) : 0LL);
                        double cmax, xmax;
                        if constexpr (kWide) {
                            // scaling, matrix-vector product and update on the grid
                            const long long c_tri = clock64();
                            if (!wide_solve_update<LT>(*W, V, sc, isc, lost_lim,
                                                       reinterpret_cast<LT *>(smem), wlimit,
                                                       wflag, cmax, xmax))
                                wide_abort = true;
                            if (tid == 0) st.cycles_solve_tri += clock64() - c_tri;
                            if (wide_abort) break;
                        } else {
                        for (int s = tid; s < N; s += kThreads)
                            bvec[s] = (LT)(res[perm[s]] * sc);
                        __syncthreads();
                        const long long c_tri = clock64();
                        gje_apply(reinterpret_cast<const float *>(M), ld, N, perm,
                                  reinterpret_cast<float *>(bvec), reinterpret_cast<float *>(lt),
                                  false);
                        if (tid == 0) st.cycles_solve_tri += clock64() - c_tri;
                        long long cmb = 0, xmb = 0;
                        for (int s = tid; s < N; s += kThreads) {
                            double c = (double)reinterpret_cast<const float *>(lt)[perm[s]] * isc;
                            // the part of this row's right-hand side that the
                            // FP32 cast lost (below the FP32 normal range),
                            // applied through the diagonal
                            if ((__double_as_longlong(res[s]) & 0x7fffffffffffffffLL) < lost_lim) {
                                const double rs = res[s] * sc;
                                if (fabs(mdiag[s]) >= 0.5)
                                    c += (rs - (double)(float)rs) * isc / mdiag[s];
                            }
                            const double nx = dx[s] + c;
                            dx[s] = nx;
                            cmb = max(cmb, absbits_nonan(c));
                            xmb = max(xmb, absbits_nonan(nx));
                        }
                        cmax = __longlong_as_double(cmb);
                        xmax = __longlong_as_double(xmb);
                        block_max2(cmax, xmax, red);
                        }
                        if (tid == 0) st.refine_sweeps++;
                        if (sweep > 0) rate = fmax(rate, cmax / prev);
                        // stop when this correction, or the next one predicted
                        // from the contraction so far, is below FP64 resolution
                        // of dx.  Fresh factors contract geometrically (their
                        // error is rounding noise): the last ratio predicts the
                        // next one.  Reused factors precondition another
                        // matrix, whose iteration need not contract evenly: the
                        // prediction takes the worst ratio of the solve and
                        // waits for three corrections.  (A test on the state's
                        // last bits instead -- stop when no species of y + dx
                        // moves -- was measured and dropped: species many
                        // orders below the others cannot be resolved through
                        // the FP32 inverse, extra sweeps only scatter their
                        // sign, and the batch took three times the FP64 form's
                        // negative-species reverts.)
                        const double r_est = soft ? rate : cmax / prev;
                        const bool small_next =
                            sweep >= (soft ? 2 : 1) && !(cmax * r_est > 1e-16 * xmax);
                        const bool done = !(cmax > 1e-15 * xmax) || small_next;
                        if (!finite || done) {
                            converged = true;
                            break;
                        }
                        // stagnation, the sweep limit, or reused factors that
                        // contract too slowly: not converged
                        if (!(cmax < 0.5 * prev) || sweep + 1 == refine_max ||
                            (soft && sweep > 0 && !(cmax <= kBailRate * prev)))
                            break;
                        prev = cmax;
                        // res = xr - (dx - h*J(xf)*dx)
                        if constexpr (kWide) {
                            if (!wide_residual<LT>(*W, m, V, dt, wlimit, wflag, rmax))
                                wide_abort = true;
                            if (wide_abort) break;
                        } else {
                        jv_phase1(m, xf, dx, qr);
                        __syncthreads();
                        rlb = 0;
                        for (int s = tid; s < N; s += kThreads) {
                            const double jv = jv_species(m, s, qr);
                            const double r = xr[s] - (dx[s] - dt * jv);
                            res[s] = r;
                            rlb = max(rlb, absbits_nonan(r));
                        }
                        rmax = block_max(__longlong_as_double(rlb), red);
                        }
                    }
                    lu_rate = rate;
                    if (converged || !soft || wide_abort) break;
                    // the reused factors do not converge: factor this step's
                    // matrix (Jacobian at the step's frozen point) and solve
                    // again -- in the wide engine first with the earlier pivot
                    // order, then with a fresh pivot search if that fails too
                    const bool fresh = !reused;
                    reused = false;
                    luFail = factor_at(xf, fresh);
                    if (luFail) break;
                }
                if (luFail) {
                    // as above: the step's own matrix failed to factor
                    for (int s = tid; s < N; s += kThreads)
                        if (bad_value(yv[s])) yv[s] = V.y1[s];
                    __syncthreads();
                    newDt = dt * 0.1;
                    if (tid == 0) st.lu_failures++;
                    break;
                }
            }
            if (tid == 0) st.cycles_solve += clock64() - c_mark;
            // y_v += dx; dx = y_v - y_v_old (kernels.cuh:462-477); ||dx|| with
            // FP32-rounded squares (Simulation.cuh:58-64, 883-890)
            double sq = 0.0;
            for (int s = tid; s < N; s += kThreads) {
                const double old = yv[s];
                const double nv = (V.fd[s] == 0) ? yv[s] + dx[s] : V.fd[s];
                yv[s] = nv;
                const double d = nv - old;
                dx[s] = d;
                sq = sq + (double)(float)(d * d);
            }
            errN = sqrt(block_sum(sq, red));
            itN = itN + 1;
            if (tid == 0) st.newton_iters++;
        }
        if (!kMixed || pass > 0 || !step_reused || luFail || expired || wide_abort) break;
        bool stale_bad = false;
        for (int s = tid; s < N; s += kThreads) stale_bad |= bad_value(yv[s]);
        if (!__syncthreads_or(stale_bad)) break;
        }
        bool reverted = false;
        if (!luFail) {
            // Simulation.cuh:894-909
            bool anybad = false;
            for (int s = tid; s < N; s += kThreads) anybad |= bad_value(yv[s]);
            if (__syncthreads_or(anybad)) {
                reverted = true;
                for (int s = tid; s < N; s += kThreads)
                    if (bad_value(yv[s])) yv[s] = V.y1[s];
                newDt = dt * 0.1;
                if (tid == 0) st.nan_reverts++;
            }
        }
        __syncthreads();
        if (expired || wide_abort) {
            status = LASSIE_ERR_DEADLINE;
            break;
        }
        if (rec) {
            if (nsteps >= AD.cap_steps || nstates >= AD.cap_states) {
                status = LASSIE_ERR_RECORD_FULL;
                break;
            }
            const int slot = nstates++;
            rkf_run = 0;
            for (int s2 = tid; s2 < N; s2 += kThreads)
                P.adj.states[AD.states + (int64_t)slot * N + s2] = yv[s2];
            if (tid == 0) {
                P.adj.rec_kind[AD.rec + nsteps] = luFail ? 2 : (reverted ? 3 : 1);
                P.adj.rec_dt[AD.rec + nsteps] = dt;
                P.adj.rec_slot[AD.rec + nsteps] = slot;
            }
            nsteps++;
        }
        double *tmp = V.y1;
        V.y1 = V.k2;
        V.k2 = tmp;
        t = t + dt;
    }
    if (rec && tid == 0) P.adj.nsteps[id] = nsteps;
    if constexpr (kWide) wide_exit<LT>(*W);
    __syncthreads();
    if (tid == 0) {
        st.outer_iters = outer;
        st.t_final = t;
        st.dt_be_final = newDt;
        st.status = status;
        st.cycles_total = clock64() - c_start;
        P.res[id] = st;
    }
    __syncthreads();
}

#include "bdf.cuh"

template <typename LT>
__global__ void __launch_bounds__(kThreads, 1) compat_kernel(LaunchParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[2 * kWarps + 1];
    __shared__ int ired[kWarps + 2 + LuShape<LT>::PB];
    __shared__ int mv[4 * LuShape<LT>::PB];
    __shared__ InstDesc D;
    __shared__ InstResult st;
    __shared__ int next;
    __shared__ uint64_t start;
    if (threadIdx.x == 0) start = global_ns();
    __syncthreads();
    const uint64_t deadline = P.deadline_ns ? start + P.deadline_ns : 0;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(P.queue, 1);
        __syncthreads();
        const int q = next;
        __syncthreads();
        if (q >= P.n_inst) break;
        if (P.controller == LASSIE_CTRL_BDF) {
            bdf_integrate<LT>(P, P.order[q], smem, red, ired, D, st, deadline);
            continue;
        }
        integrate<LT>(P, P.order[q], smem, red, ired, mv, D, st, deadline);
    }
}

// ------------------------------------------------------------- adjoint

// Fehlberg coefficients of the stages (kernels.cuh:79-143) and of the
// 4th-order solution kept on acceptance (kernels.cuh:172).
__constant__ double kRkA[6][5] = {
    {0, 0, 0, 0, 0},
    {1.0 / 4.0, 0, 0, 0, 0},
    {3.0 / 32.0, 9.0 / 32.0, 0, 0, 0},
    {1932.0 / 2197.0, -7200.0 / 2197.0, 7296.0 / 2197.0, 0, 0},
    {439.0 / 216.0, -8.0, 3680.0 / 513.0, -845.0 / 4104.0, 0},
    {-8.0 / 27.0, 2.0, -3544.0 / 2565.0, 1859.0 / 4104.0, -11.0 / 40.0}};
__constant__ double kRkB[5] = {25.0 / 216.0, 0.0, 1408.0 / 2565.0, 2197.0 / 4104.0, -1.0 / 5.0};

// Stage inputs Y[0..4] and slopes K[0..4] of an RKF45 step of size dt from y
// (Y[0] may alias y), with the forward attempt's exact arithmetic, so a
// recomputed step equals the forward one bit for bit; fed species take the
// feed as slope and 0 as later stage input.  w (optional) receives the
// 4th-order solution.
__device__ void rkf_stages(const Net &m, const double *y, double dt, const double *fd,
                           double *const *Y, double *const *K, double *pw, double *w) {
    const int N = m.n, tid = threadIdx.x;
    if (Y[0] != y) {
        for (int s = tid; s < N; s += kThreads) Y[0][s] = y[s];
    }
    for (int s = tid; s < N; s += kThreads)
        for (int i = 1; i < 5; i++) Y[i][s] = 0.0;
    __syncthreads();
    for (int st = 0; st < 5; st++) {
        rhs_phase1(m, Y[st], pw);
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) {
            const double f = rhs_species(m, s, pw);
            if (fd[s] != 0.0) {
                K[st][s] = fd[s];
                continue;
            }
            K[st][s] = f * dt;
            const double y0 = y[s];
            const double *k1 = K[0], *k2 = K[1], *k3 = K[2], *k4 = K[3], *k5 = K[4];
            if (st == 0) Y[1][s] = y0 + k1[s] / 4.0;
            else if (st == 1) Y[2][s] = y0 + (3.0 * k1[s]) / 32.0 + (9.0 * k2[s]) / 32.0;
            else if (st == 2)
                Y[3][s] = y0 + (1932.0 * k1[s]) / 2197.0 - (7200.0 * k2[s]) / 2197.0 +
                          (7296.0 * k3[s]) / 2197.0;
            else if (st == 3)
                Y[4][s] = y0 + (439.0 * k1[s]) / 216.0 - (8.0 * k2[s]) +
                          (3680.0 * k3[s]) / 513.0 - (845.0 * k4[s]) / 4104.0;
            else if (w)
                w[s] = y0 + (25.0 * k1[s]) / 216.0 + (1408.0 * k3[s]) / 2565.0 +
                       (2197.0 * k4[s]) / 4104.0 - k5[s] / 5.0;
        }
        __syncthreads();
    }
    if (w) {
        for (int s = tid; s < N; s += kThreads)
            if (fd[s] != 0.0) w[s] = fd[s];
        __syncthreads();
    }
}

struct AdjSmem {
    int64_t vec, kk, pw, tq, theta, rptr, sptr, sent, rent, hrptr, hrent, asptr, asent, perm,
        slot, bvec, lt, utile, rowbuf, total;
    __host__ __device__ AdjSmem(int nmax, int rmax, int amax, int hmax) {
        auto al = [](int64_t v) { return (v + 15) & ~int64_t(15); };
        const int PB = LuShape<float>::PB;
        int64_t o = 0;
        vec = o;    o = al(o + int64_t(16) * nmax * 8);
        kk = o;     o = al(o + int64_t(rmax) * 8);
        pw = o;     o = al(o + int64_t(amax > 0 ? amax : 1) * 8);
        tq = o;     o = al(o + int64_t(amax > 0 ? amax : 1) * 8);
        theta = o;  o = al(o + int64_t(rmax) * 8);
        rptr = o;   o = al(o + int64_t(rmax + 1) * 4);
        sptr = o;   o = al(o + int64_t(nmax + 1) * 4);
        sent = o;   o = al(o + int64_t(hmax > 0 ? hmax : 1) * 4);
        rent = o;   o = al(o + int64_t(amax > 0 ? amax : 1) * 4);
        hrptr = o;  o = al(o + int64_t(rmax + 1) * 4);
        hrent = o;  o = al(o + int64_t(hmax > 0 ? hmax : 1) * 4);
        asptr = o;  o = al(o + int64_t(nmax + 1) * 4);
        asent = o;  o = al(o + int64_t(amax > 0 ? amax : 1) * 4);
        perm = o;   o = al(o + int64_t(nmax) * 4);
        slot = o;   o = al(o + int64_t(nmax) * 4);
        bvec = o;   o = al(o + int64_t(nmax) * 4);
        lt = o;     o = al(o + (int64_t(PB) * (((nmax + 31) & ~31) + 4) + 160) * 4);
        utile = o;  o = al(o + int64_t(PB) * 128 * 4);
        rowbuf = o; o = al(o + int64_t(2 * PB) * 4);
        total = o;
    }
};

// Backward pass of one instance: the discrete adjoint of its recorded step
// sequence for L = sum over samples and sampled species of (y - target)^2.
// Accepted RKF45 steps: reverse stage recursion with J^T products at the
// recomputed stage inputs.  Backward-Euler steps y' = y + h f(y') (taken as
// exactly solved): (I - h J(y'))^T mu = lambda with an FP32 LU of the exact
// Jacobian and FP64 refinement; lambda <- mu.  d L / d log k accumulates
// h * prop_j * (S^T kbar)_j at every stage and step.
__device__ void adjoint_instance(const LaunchParams &P, int id, unsigned char *smem, double *red,
                                 int *ired, int *mv, InstDesc &D, double *cyc_dummy) {
    const int tid = threadIdx.x;
    if (tid == 0) D = P.inst[id];
    __syncthreads();
    const AdjDesc AD = P.adj.desc[id];
    const int N = D.n, R = D.r;
    const AdjSmem L(P.nmax, P.rmax, P.amax, P.hmax);
    double *vb = reinterpret_cast<double *>(smem + L.vec);
    double *lam = vb, *lnew = vb + P.nmax, *kbar = vb + 2 * P.nmax, *fd = vb + 3 * P.nmax;
    double *Y[5], *Yb[5], *Kst[5];
    for (int i = 0; i < 5; i++) Y[i] = vb + (4 + i) * P.nmax;
    for (int i = 1; i < 5; i++) Yb[i] = vb + (8 + i) * P.nmax;  // slots 9..12
    Yb[0] = nullptr;
    // slopes alias the adjoint stage vectors Yb (not live while stages are built)
    Kst[0] = vb + 13 * P.nmax;
    Kst[1] = vb + 14 * P.nmax;
    Kst[2] = vb + 15 * P.nmax;
    Kst[3] = Yb[1];
    Kst[4] = Yb[2];
    double *kk = reinterpret_cast<double *>(smem + L.kk);
    double *pw = reinterpret_cast<double *>(smem + L.pw);
    double *tq = reinterpret_cast<double *>(smem + L.tq);
    double *theta = reinterpret_cast<double *>(smem + L.theta);
    int *rptr = reinterpret_cast<int *>(smem + L.rptr);
    int *s_sptr = reinterpret_cast<int *>(smem + L.sptr);
    int *s_sent = reinterpret_cast<int *>(smem + L.sent);
    int *s_rent = reinterpret_cast<int *>(smem + L.rent);
    int *s_hrptr = reinterpret_cast<int *>(smem + L.hrptr);
    int *s_hrent = reinterpret_cast<int *>(smem + L.hrent);
    int *s_asptr = reinterpret_cast<int *>(smem + L.asptr);
    int *s_asent = reinterpret_cast<int *>(smem + L.asent);
    int *perm = reinterpret_cast<int *>(smem + L.perm);
    float *bvec = reinterpret_cast<float *>(smem + L.bvec);
    float *lt = reinterpret_cast<float *>(smem + L.lt);
    float *utile = reinterpret_cast<float *>(smem + L.utile);
    float *rowbuf = reinterpret_cast<float *>(smem + L.rowbuf);
    const int *ia = P.iarena;
    const double *da = P.darena;
    for (int q = tid; q < D.nnz_a; q += kThreads) s_rent[q] = ia[D.rxn_ent + q];
    for (int q = tid; q < D.nnz_h; q += kThreads) {
        s_sent[q] = ia[D.sp_ent + q];
        s_hrent[q] = ia[D.hr_ent + q];
    }
    for (int q = tid; q <= N; q += kThreads) {
        s_sptr[q] = ia[D.sp_ptr + q];
        s_asptr[q] = ia[D.as_ptr + q];
    }
    for (int q = tid; q < D.nnz_a; q += kThreads) s_asent[q] = ia[D.as_ent + q];
    for (int j = tid; j <= R; j += kThreads) {
        rptr[j] = ia[D.rxn_ptr + j];
        s_hrptr[j] = ia[D.hr_ptr + j];
    }
    for (int j = tid; j < R; j += kThreads) {
        kk[j] = da[D.k + j];
        theta[j] = 0.0;
    }
    for (int s = tid; s < N; s += kThreads) {
        fd[s] = D.feed >= 0 ? da[D.feed + s] : 0.0;
        lam[s] = 0.0;
    }
    __syncthreads();
    Net m;
    m.n = N;
    m.r = R;
    m.nnz_a = D.nnz_a;
    m.rent = s_rent;
    m.sptr = s_sptr;
    m.sent = s_sent;
    m.rptr = rptr;
    m.kk = kk;
    AdjNet an{s_hrptr, s_hrent, s_asptr, s_asent};

    const int *cs = D.cs >= 0 ? ia + D.cs : nullptr;
    const int ncs = D.ncs;
    const double *target = P.adj.target + D.out;
    const int *samp = P.adj.samp_step + AD.samp;
    const int *rk = P.adj.rec_kind + AD.rec;
    const double *rdt = P.adj.rec_dt + AD.rec;
    const int *rslot = P.adj.rec_slot + AD.rec;
    const double *states = P.adj.states + AD.states;
    double *buf = P.adj.scratch + (int64_t)blockIdx.x * P.adj.scratch_stride;
    float *M = reinterpret_cast<float *>(P.workspace + (int64_t)blockIdx.x * P.ws_stride);
    const int ld = round_up4(N);
    float *dinv = M + (int64_t)N * ld;
    const int ns = P.adj.nsteps[id];
    int ip = D.nt - 1;
    // samples taken at state index `si`: lambda += 2 (y - target) on sampled species
    auto add_samples = [&](int si, const double *y) {
        while (ip >= 0 && samp[ip] == si) {
            for (int j = tid; j < ncs; j += kThreads) {
                const int sp = cs ? cs[j] : j;
                lam[sp] += 2.0 * (y[sp] - target[(int64_t)ip * ncs + j]);
            }
            __syncthreads();
            ip--;
        }
    };
    while (ip >= 0 && samp[ip] > ns) ip--;  // (not expected) samples past the record
    int n = ns - 1;
    while (n >= 0) {
        int p = n;
        while (p > 0 && rslot[p - 1] < 0) p--;
        const int sp0 = (p == 0) ? 0 : rslot[p - 1];
        for (int s = tid; s < N; s += kThreads) buf[s] = states[(int64_t)sp0 * N + s];
        __syncthreads();
        for (int q = p; q <= n; q++) {
            double *yo = buf + (int64_t)(q - p + 1) * N;
            if (rslot[q] >= 0) {
                for (int s = tid; s < N; s += kThreads) yo[s] = states[(int64_t)rslot[q] * N + s];
                __syncthreads();
            } else {
                rkf_stages(m, buf + (int64_t)(q - p) * N, rdt[q], fd, Y, Kst, pw, yo);
            }
        }
        for (int q = n; q >= p; q--) {
            const double *yin = buf + (int64_t)(q - p) * N;
            const double *yout = buf + (int64_t)(q - p + 1) * N;
            add_samples(q + 1, yout);
            const int kind = rk[q];
            const double h = rdt[q];
            if (kind == 0) {
                rkf_stages(m, yin, h, fd, Y, Kst, pw, nullptr);
                for (int s = tid; s < N; s += kThreads) lnew[s] = (fd[s] != 0.0) ? 0.0 : lam[s];
                __syncthreads();
                for (int i = 4; i >= 0; i--) {
                    for (int s = tid; s < N; s += kThreads) {
                        double kb = 0.0;
                        if (fd[s] == 0.0) {
                            kb = kRkB[i] * lam[s];
                            for (int mm = i + 1; mm < 5; mm++) kb += kRkA[mm][i] * Yb[mm][s];
                        }
                        kbar[s] = kb;
                    }
                    __syncthreads();
                    jtv_phase1(m, an, Y[i], kbar, tq, theta, h);
                    __syncthreads();
                    for (int s = tid; s < N; s += kThreads) {
                        double yb = h * jtv_species(an, s, tq);
                        if (i >= 1 && fd[s] != 0.0) yb = 0.0;
                        if (i >= 1) Yb[i][s] = yb;
                        lnew[s] += yb;
                    }
                    __syncthreads();
                }
                for (int s = tid; s < N; s += kThreads) lam[s] = lnew[s];
                __syncthreads();
            } else if (kind == 1) {
                // (I - h D J(y'))^T mu = lambda, D masks fed rows
                double *mu = Y[0], *res = Y[1], *mdiag = Y[2], *vm = Y[3];
                assemble_newton_matrix<float>(m, yout, h, M, ld, true, fd);
                for (int s = tid; s < N; s += kThreads) mdiag[s] = (double)M[(int64_t)s * ld + s];
                const int fail = lu_factor<float>(M, ld, N, perm, lt, utile, rowbuf, red, ired,
                                                  reinterpret_cast<long long *>(cyc_dummy));
                if (fail == 0) {
                    invert_diag_blocks(M, ld, N, perm, dinv);
                    __syncthreads();
                    double rloc = 0.0;
                    for (int s = tid; s < N; s += kThreads) {
                        mu[s] = 0.0;
                        res[s] = lam[s];
                        rloc = fmax(rloc, fabs(lam[s]));
                    }
                    double rmax = block_max(rloc, red);
                    double prev = INFINITY;
                    for (int sweep = 0; sweep < 12; sweep++) {
                        if (rmax == 0.0) break;
                        const bool finite = isfinite(rmax);
                        const int e = finite ? ilogb(rmax) : 0;
                        const double sc = ldexp(1.0, -e), isc = ldexp(1.0, e);
                        for (int s = tid; s < N; s += kThreads) bvec[s] = (float)(res[s] * sc);
                        __syncthreads();
                        lu_solve_fast_T(M, ld, N, perm, dinv, bvec);
                        double cmax = 0.0, xmax = 0.0;
                        for (int i2 = tid; i2 < N; i2 += kThreads) {
                            const int s = perm[i2];
                            double c = (double)bvec[i2] * isc;
                            const double rs = res[s] * sc;
                            if (fabs(rs) < 0x1p-126 && fabs(mdiag[s]) >= 0.5)
                                c += (rs - (double)(float)rs) * isc / mdiag[s];
                            const double nx = mu[s] + c;
                            mu[s] = nx;
                            cmax = fmax(cmax, fabs(c));
                            xmax = fmax(xmax, fabs(nx));
                        }
                        cmax = block_max(cmax, red);
                        xmax = block_max(xmax, red);
                        const bool small_next = sweep > 0 && !(cmax * (cmax / prev) > 1e-16 * xmax);
                        if (!finite || !(cmax > 1e-15 * xmax) || !(cmax < 0.5 * prev) || small_next)
                            break;
                        prev = cmax;
                        // res = lambda - (mu - h J^T (D mu))
                        for (int s = tid; s < N; s += kThreads) vm[s] = (fd[s] != 0.0) ? 0.0 : mu[s];
                        __syncthreads();
                        jtv_phase1(m, an, yout, vm, tq, nullptr, h);
                        __syncthreads();
                        rloc = 0.0;
                        for (int s = tid; s < N; s += kThreads) {
                            const double r = lam[s] - (mu[s] - h * jtv_species(an, s, tq));
                            res[s] = r;
                            rloc = fmax(rloc, fabs(r));
                        }
                        rmax = block_max(rloc, red);
                    }
                    for (int s = tid; s < N; s += kThreads) vm[s] = (fd[s] != 0.0) ? 0.0 : mu[s];
                    __syncthreads();
                    jtv_phase1(m, an, yout, vm, tq, theta, h);  // d/dlog k contributions
                    __syncthreads();
                    for (int s = tid; s < N; s += kThreads) lam[s] = vm[s];
                    __syncthreads();
                }
            }
            // kinds 2 and 3 (state unchanged / reverted species): identity
        }
        n = p - 1;
        if (n < 0) add_samples(0, buf);
    }
    if (ns == 0) {
        for (int s = tid; s < N; s += kThreads) buf[s] = states[s];
        __syncthreads();
        add_samples(0, buf);
    }
    double *g = P.adj.grad + AD.grad;
    for (int j = tid; j < R; j += kThreads) g[j] = theta[j];
    for (int s = tid; s < N; s += kThreads) g[R + s] = lam[s];
    __syncthreads();
}

__global__ void __launch_bounds__(kThreads, 1) adjoint_kernel(LaunchParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[2 * kWarps + 1];
    __shared__ int ired[kWarps + 2 + LuShape<float>::PB];
    __shared__ int mv[4 * LuShape<float>::PB];
    __shared__ InstDesc D;
    __shared__ double cyc[4];
    __shared__ int next;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(P.queue, 1);
        __syncthreads();
        const int q = next;
        __syncthreads();
        if (q >= P.n_inst) break;
        adjoint_instance(P, P.order[q], smem, red, ired, mv, D, cyc);
    }
}

int64_t adjoint_smem_bytes(int nmax, int rmax, int amax, int hmax) {
    return AdjSmem(nmax, rmax, amax, hmax).total;
}

cudaError_t adjoint_launch(const LaunchParams &P, int grid, int64_t smem, cudaStream_t stream) {
    cudaError_t e = cudaFuncSetAttribute(adjoint_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    adjoint_kernel<<<grid, kThreads, smem, stream>>>(P);
    return cudaGetLastError();
}

// ------------------------------------------------------------- launch

int64_t compat_smem_bytes(int nmax, int rmax, int amax, int hmax, int precision,
                          int controller) {
    if (controller == LASSIE_CTRL_BDF)
        return precision == LASSIE_PREC_FP64
                   ? SmemLayout(nmax, rmax, amax, hmax, 8, LuShape<double>::PB,
                                LuShape<double>::TN, kBdfVecs)
                         .total
                   : SmemLayout(nmax, rmax, amax, hmax, 4, LuShape<float>::PB,
                                LuShape<float>::TN, kBdfVecs)
                         .total;
    if (precision == LASSIE_PREC_FP64)
        return SmemLayout(nmax, rmax, amax, hmax, 8, LuShape<double>::PB, LuShape<double>::TN)
            .total;
    return SmemLayout(nmax, rmax, amax, hmax, 4, LuShape<float>::PB, LuShape<float>::TN).total;
}

cudaError_t compat_configure(int precision, int64_t smem) {
    if (precision == LASSIE_PREC_FP64)
        return cudaFuncSetAttribute(compat_kernel<double>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaFuncSetAttribute(compat_kernel<float>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t compat_launch(const LaunchParams &P, int grid, int64_t smem, cudaStream_t stream) {
    if (P.precision == LASSIE_PREC_FP64)
        compat_kernel<double><<<grid, kThreads, smem, stream>>>(P);
    else
        compat_kernel<float><<<grid, kThreads, smem, stream>>>(P);
    return cudaGetLastError();
}

// ------------------------------------------------------- wide engine

// One instance (P.inst[0]) over the whole GPU: CTA 0 integrates, the others
// serve its linear-algebra tasks.  Launched cooperatively (all CTAs resident).
template <typename LT>
__global__ void __launch_bounds__(kThreads, 1) wide_kernel(LaunchParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[2 * kWarps + 1];
    __shared__ int ired[kWarps + 2 + LuShape<LT>::PB];
    __shared__ int mv[4 * LuShape<LT>::PB];
    __shared__ InstDesc D;
    __shared__ InstResult st;
    __shared__ uint64_t start;
    if (threadIdx.x == 0) start = global_ns();
    __syncthreads();
    const uint64_t deadline = P.deadline_ns ? start + P.deadline_ns : 0;
    // every wait on another CTA ends at the launch deadline (if any) or after
    // kWideStallNs without progress
    const uint64_t wlimit = deadline;
    const InstDesc &D0 = P.inst[0];
    const int N = D0.n;
    WideWs<LT> W = wide_ws<LT>(P.workspace, N, D0.r, D0.nnz_a);
    // tensor-core rank updates: each CTA holds kTcN TMEM columns and an
    // mbarrier for the whole launch
    __shared__ uint64_t tc_bar;
    __shared__ uint32_t tc_slot, tc_phase;
    const bool tc = std::is_same<LT, float>::value && P.tensor_cores != 0;
    if (tc) {
        if (threadIdx.x < 32) tc_alloc(&tc_slot, kTcN);
        if (threadIdx.x == 0) {
            tc_mbar_init(&tc_bar);
            tc_phase = 0;
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        W.tc_on = P.tensor_cores == 2 ? 2 : 1;
        W.tc_bar = &tc_bar;
        W.tc_phase = &tc_phase;
        W.tc_tmem = tc_slot;
    }
    if (blockIdx.x == 0) {
        integrate<LT, true>(P, 0, smem, red, ired, mv, D, st, deadline, &W, wlimit);
    } else {
        Net m;
        m.n = N;
        m.r = D0.r;
        m.nnz_a = D0.nnz_a;
        m.rent = P.iarena + D0.rxn_ent;
        m.sptr = P.iarena + D0.sp_ptr;
        m.sent = P.iarena + D0.sp_ent;
        m.rptr = P.iarena + D0.rxn_ptr;
        m.kk = P.darena + D0.k;
        // the leader's mdiag is its vector k1 (third of the ten)
        wide_worker<LT>(W, m, W.vec + 2 * (int64_t)N, smem, wlimit);
    }
    if (tc) {
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (threadIdx.x < 32) tc_dealloc(W.tc_tmem, kTcN);
    }
}

int64_t wide_workspace_bytes(int N, int R, int nnz_a, int precision) {
    return WideLayout(N, R, nnz_a, precision == LASSIE_PREC_FP64 ? 8 : 4).total;
}

int64_t wide_flags_offset(int N, int R, int nnz_a, int precision) {
    return WideLayout(N, R, nnz_a, precision == LASSIE_PREC_FP64 ? 8 : 4).flags;
}

int64_t wide_dynamic_smem(int N, int precision) {
    return wide_smem_bytes(N, precision == LASSIE_PREC_FP64 ? 8 : 4);
}

// Configures the kernel and returns the number of CTAs of one cooperative
// launch (one per SM), or 0 if a CTA does not fit.
int wide_configure(int precision, int64_t smem, int sm_count) {
    const void *f = precision == LASSIE_PREC_FP64 ? (const void *)wide_kernel<double>
                                                  : (const void *)wide_kernel<float>;
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, kThreads, (size_t)smem) !=
            cudaSuccess ||
        per_sm < 1)
        return 0;
    return sm_count < kWideMaxGrid ? sm_count : kWideMaxGrid;
}

// The caller clears the control block and the pivot-order flag first.
cudaError_t wide_launch(const LaunchParams &P, int grid, int64_t smem, cudaStream_t stream) {
    LaunchParams Pc = P;
    void *args[] = {&Pc};
    const void *f = P.precision == LASSIE_PREC_FP64 ? (const void *)wide_kernel<double>
                                                    : (const void *)wide_kernel<float>;
    return cudaLaunchCooperativeKernel(f, grid, kThreads, args, (size_t)smem, stream);
}

// ------------------------------------------------ tensor-core self-test

// D = A * B (A: 128 x 32, B: 32 x kTcN, D: 128 x kTcN, row-major FP32) through
// tc_tile_product (kBf16: tc_tile_product_bf16) on one CTA; status[0] = 1 on
// success, 2 if the MMA wait ran out.
template <bool kBf16>
__global__ void __launch_bounds__(kThreads, 1) tc_selftest_kernel(const float *A, const float *B,
                                                                  float *D, int *status) {
    extern __shared__ __align__(16) unsigned char smem[];
    float *sAh = reinterpret_cast<float *>(smem);
    float *sAl = sAh + kTcM * kTcK;
    float *sBh = sAl + kTcM * kTcK;
    float *sBl = sBh + kTcN * kTcK;
    uint16_t *sA16 = reinterpret_cast<uint16_t *>(smem), *sB16 = sA16 + kTcM * kTcK;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sBl + kTcN * kTcK);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x;
    if (tid < 32) tc_alloc(slot, kTcN);
    if (tid == 0) tc_mbar_init(bar);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    for (int q = tid; q < kTcM * kTcK; q += kThreads) {
        const int r = q / kTcK, k = q - r * kTcK;
        const float x = A[q];
        if constexpr (kBf16) {
            sA16[tc_off16(r, k) / 2] = bf16_bits(x);
        } else {
            const float hi = tf32_hi(x);
            const int o = tc_off(r, k) / 4;
            sAh[o] = hi;
            sAl[o] = x - hi;
        }
    }
    for (int q = tid; q < kTcN * kTcK; q += kThreads) {
        const int n = q / kTcK, k = q - n * kTcK;
        const float x = B[k * kTcN + n];
        if constexpr (kBf16) {
            sB16[tc_off16(n, k) / 2] = bf16_bits(x);
        } else {
            const float hi = tf32_hi(x);
            const int o = tc_off(n, k) / 4;
            sBh[o] = hi;
            sBl[o] = x - hi;
        }
    }
    tc_proxy_fence();
    __syncthreads();
    uint32_t phase = 0;
    float out[32];
    bool ok;
    if constexpr (kBf16) ok = tc_tile_product_bf16(sA16, sB16, bar, tmem, phase, out);
    else ok = tc_tile_product(sAh, sAl, sBh, sBl, bar, tmem, phase, out);
    if (ok) {
        const int w = tid >> 5, row = (w & 3) * 32 + (tid & 31), c0 = (w >> 2) * 32;
        for (int i = 0; i < 32; i++) D[row * kTcN + c0 + i] = out[i];
    }
    __syncthreads();
    if (tid < 32) tc_dealloc(tmem, kTcN);
    if (tid == 0) status[0] = ok ? 1 : 2;
}

template <bool kBf16>
static int tc_selftest_launch(const float *dA, const float *dB, float *dD, int *dstatus,
                              void *stream) {
    const int smem = kTcSmemBytes;
    if (cudaFuncSetAttribute(tc_selftest_kernel<kBf16>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return LASSIE_ERR_CUDA;
    tc_selftest_kernel<kBf16><<<1, kThreads, smem, (cudaStream_t)stream>>>(dA, dB, dD, dstatus);
    return cudaGetLastError() == cudaSuccess ? LASSIE_OK : LASSIE_ERR_CUDA;
}

extern "C" int lassie_tc_selftest(const float *dA, const float *dB, float *dD, int *dstatus,
                                  void *stream) {
    return tc_selftest_launch<false>(dA, dB, dD, dstatus, stream);
}

extern "C" int lassie_tc_selftest_bf16(const float *dA, const float *dB, float *dD, int *dstatus,
                                       void *stream) {
    return tc_selftest_launch<true>(dA, dB, dD, dstatus, stream);
}

// ------------------------------------------ single-evaluation kernels

// dx = f(x) for a batch of parameterisations of one network: one warp per
// instance (no CTA barrier on the data path).  The network structure is
// staged once per CTA; each warp copies its instance's x into its own
// shared-memory slice with 16-byte loads, forms the reaction rates (k read
// coalesced), then the species sums in the oracle's order (rhs_species), and
// stores dx.  On GB300 the FP64 pipe (about two operations per clock per SM),
// not HBM, bounds this kernel: one product per reactant and one sum per
// net-stoichiometry entry against 24 bytes per species.  So the kernel keeps
// that pipe's instruction count at the useful work:
// - lanes take reactions and species in the host's order of their trip
//   counts (rord, sord), so the 32 lanes of a warp run loops of equal length;
// - a species sum starts from its first term rather than 0.0 + term.  The
//   two differ only in the sign of an all-zero sum (0.0 + -0.0 is +0.0, and
//   no other partial sum can be -0.0 in round-to-nearest), which the final
//   line restores.
constexpr int kRhsThreads = 256;
constexpr int kRhsWarps = kRhsThreads / 32;

__device__ __forceinline__ void warp_copy_f64(double *dst, const double *src, int n) {
    const int lane = threadIdx.x & 31;
    if ((((uintptr_t)src) & 15) == 0 && (n & 1) == 0) {
        const double2 *s2 = reinterpret_cast<const double2 *>(src);
        double2 *d2 = reinterpret_cast<double2 *>(dst);
        for (int i = lane; i < n / 2; i += 32) d2[i] = __ldcs(s2 + i);
    } else {
        for (int i = lane; i < n; i += 32) dst[i] = __ldcs(src + i);
    }
}

// Net-stoichiometry term c * k * prod(x^a) of entry `ent` when |c| != 1 (the
// oracle's per-entry product order).
__device__ __forceinline__ double rhs_term_scaled(int y, int c, const int *rptr, const int *rent,
                                                  const double *kb, const double *xs) {
    double v = (double)c * __ldg(kb + y);
    for (int q = rptr[y]; q < rptr[y + 1]; q++) {
        const int eq = rent[q];
        v = v * mypow(xs[ent_index(eq)], ent_coef(eq));
    }
    return v;
}

__device__ __forceinline__ double neg_bits(double v) {
    return __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ull);
}

// k_y * x_a^ea * x_b^eb ... in reactant order (rhs_rates' product)
__device__ __forceinline__ double rhs_rate(int y, const int *rptr, const int *rent,
                                           const double *kb, const double *xs) {
    double r = __ldg(kb + y);
    for (int q = rptr[y]; q < rptr[y + 1]; q++) {
        const int e = rent[q];
        r = r * mypow(xs[ent_index(e)], ent_coef(e));
    }
    return r;
}

// dx_s from the rates: the entries of H row s in ascending order.  acc - r
// is acc + (-r) in IEEE arithmetic: one addition per entry, and a sign flip
// (integer) for a leading -r; the sum starts from its first term, and the
// sign of an all-zero sum is restored at the end.
__device__ __forceinline__ double rhs_species_sum(int s, const int *sptr, const int *sent,
                                                  const int *rptr, const int *rent,
                                                  const double *rate, const double *kb,
                                                  const double *xs) {
    const int e0 = sptr[s], e1 = sptr[s + 1];
    if (e0 == e1) return 0.0;
    double acc;
    {
        const int ent = sent[e0];
        const int y = ent_index(ent), c = ent_coef(ent);
        acc = c == 1 ? rate[y]
                     : (c == -1 ? neg_bits(rate[y]) : rhs_term_scaled(y, c, rptr, rent, kb, xs));
    }
    for (int e = e0 + 1; e < e1; e++) {
        const int ent = sent[e];
        const int y = ent_index(ent), c = ent_coef(ent);
        if (c == 1) acc = acc + rate[y];
        else if (c == -1) acc = acc - rate[y];
        else acc = acc + rhs_term_scaled(y, c, rptr, rent, kb, xs);
    }
    if (__double_as_longlong(acc) == (long long)0x8000000000000000ull) acc = 0.0;
    return acc;
}

__global__ void __launch_bounds__(kRhsThreads) rhs_batch_kernel(
    int n_inst, int N, int R, int nnz_a, int nnz_h, const int *__restrict__ rptr_g,
    const int *__restrict__ rent_g, const int *__restrict__ sptr_g, const int *__restrict__ sent_g,
    const int *__restrict__ order_g, const double *__restrict__ k, const double *__restrict__ x,
    double *__restrict__ dx) {
    extern __shared__ __align__(16) unsigned char smem[];
    int *rptr = reinterpret_cast<int *>(smem);
    int *sptr = rptr + (R + 1);
    int *rent = sptr + (N + 1);
    int *sent = rent + (nnz_a > 0 ? nnz_a : 1);
    int *rord = sent + (nnz_h > 0 ? nnz_h : 1);
    int *sord = rord + R;
    const int64_t ints = (int64_t)(R + 1) + (N + 1) + (nnz_a > 0 ? nnz_a : 1) +
                         (nnz_h > 0 ? nnz_h : 1) + R + N;
    double *wbase = reinterpret_cast<double *>(smem + ((ints * 4 + 15) & ~int64_t(15)));
    const int per_warp = ((N + 1) & ~1) + ((R + 1) & ~1);
    for (int j = threadIdx.x; j <= R; j += kRhsThreads) rptr[j] = rptr_g[j];
    for (int j = threadIdx.x; j <= N; j += kRhsThreads) sptr[j] = sptr_g[j];
    for (int j = threadIdx.x; j < nnz_a; j += kRhsThreads) rent[j] = rent_g[j];
    for (int j = threadIdx.x; j < nnz_h; j += kRhsThreads) sent[j] = sent_g[j];
    for (int j = threadIdx.x; j < R + N; j += kRhsThreads) rord[j] = order_g[j];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double *xs = wbase + (int64_t)warp * per_warp;
    double *rate = xs + ((N + 1) & ~1);
    for (int b = blockIdx.x * kRhsWarps + warp; b < n_inst; b += gridDim.x * kRhsWarps) {
        warp_copy_f64(xs, x + (int64_t)b * N, N);
        __syncwarp();
        const double *kb = k + (int64_t)b * R;
        // reaction products once per reaction (rhs_rates), then the species
        // sums (rhs_species_r): bit-identical to the per-entry products
        for (int t = lane; t < R; t += 32) {
            const int y = rord[t];
            rate[y] = rhs_rate(y, rptr, rent, kb, xs);
        }
        __syncwarp();
        double *db = dx + (int64_t)b * N;
        for (int t = lane; t < N; t += 32) {
            const int s = sord[t];
            db[s] = rhs_species_sum(s, sptr, sent, rptr, rent, rate, kb, xs);
        }
        __syncwarp();
    }
}


// The same RHS for networks whose x and rates do not fit once per warp: one
// CTA per parameterisation, x and the rates in shared memory, the structure
// read through L1/L2.  Same operations in the same order as rhs_batch_kernel.
__global__ void __launch_bounds__(kRhsThreads) rhs_batch_cta_kernel(
    int n_inst, int N, int R, const int *__restrict__ rptr, const int *__restrict__ rent,
    const int *__restrict__ sptr, const int *__restrict__ sent, const int *__restrict__ order,
    const double *__restrict__ k, const double *__restrict__ x, double *__restrict__ dx) {
    extern __shared__ __align__(16) unsigned char smem[];
    double *xs = reinterpret_cast<double *>(smem);
    double *rate = xs + N;
    const int *rord = order, *sord = order + R;
    for (int b = blockIdx.x; b < n_inst; b += gridDim.x) {
        __syncthreads();  // the previous instance is done with xs/rate
        for (int s = threadIdx.x; s < N; s += kRhsThreads) xs[s] = __ldcs(x + (int64_t)b * N + s);
        __syncthreads();
        const double *kb = k + (int64_t)b * R;
        for (int t = threadIdx.x; t < R; t += kRhsThreads) {
            const int y = __ldg(rord + t);
            rate[y] = rhs_rate(y, rptr, rent, kb, xs);
        }
        __syncthreads();
        double *db = dx + (int64_t)b * N;
        for (int t = threadIdx.x; t < N; t += kRhsThreads) {
            const int s = __ldg(sord + t);
            db[s] = rhs_species_sum(s, sptr, sent, rptr, rent, rate, kb, xs);
        }
    }
}

cudaError_t rhs_batch_launch(int n_inst, int N, int R, int nnz_a, int nnz_h, const int *rptr,
                             const int *rent, const int *sptr, const int *sent, const int *order,
                             const double *k, const double *x, double *dx, int sm_count,
                             cudaStream_t stream) {
    const int64_t ints = (int64_t)(R + 1) + (N + 1) + (nnz_a > 0 ? nnz_a : 1) +
                         (nnz_h > 0 ? nnz_h : 1) + R + N;
    const int64_t per_warp = ((N + 1) & ~1) + ((R + 1) & ~1);
    const int64_t smem = ((ints * 4 + 15) & ~int64_t(15)) + per_warp * 8 * kRhsWarps;
    if (smem > 200 * 1024) {
        // large network: one CTA per parameterisation
        const int64_t smem1 = int64_t(N + R) * 8;
        if (smem1 > 200 * 1024) return cudaErrorInvalidValue;
        cudaError_t e = cudaFuncSetAttribute(rhs_batch_cta_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
        if (e != cudaSuccess) return e;
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rhs_batch_cta_kernel, kRhsThreads,
                                                          (size_t)smem1);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        const int grid = (int)std::min<int64_t>(n_inst, (int64_t)sm_count * per_sm);
        rhs_batch_cta_kernel<<<grid, kRhsThreads, smem1, stream>>>(n_inst, N, R, rptr, rent, sptr,
                                                                   sent, order, k, x, dx);
        return cudaGetLastError();
    }
    cudaError_t e = cudaFuncSetAttribute(rhs_batch_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rhs_batch_kernel, kRhsThreads,
                                                      (size_t)smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const int64_t want = ((int64_t)n_inst + kRhsWarps - 1) / kRhsWarps;
    const int grid = (int)std::min<int64_t>(want, (int64_t)sm_count * per_sm);
    rhs_batch_kernel<<<grid, kRhsThreads, smem, stream>>>(n_inst, N, R, nnz_a, nnz_h, rptr, rent,
                                                          sptr, sent, order, k, x, dx);
    return cudaGetLastError();
}

// M = I - h*J(x) in FP64 for one instance (one CTA).
__global__ void __launch_bounds__(kThreads) newton_matrix_kernel(
    int N, int R, int nnz_a, const int *__restrict__ rptr_g, const int *__restrict__ rent,
    const int *__restrict__ sptr, const int *__restrict__ sent, const double *__restrict__ k,
    const double *__restrict__ x, double h, double *M) {
    extern __shared__ __align__(16) unsigned char smem[];
    double *xs = reinterpret_cast<double *>(smem);
    double *kk = xs + N;
    int *rptr = reinterpret_cast<int *>(kk + R);
    for (int j = threadIdx.x; j <= R; j += kThreads) rptr[j] = rptr_g[j];
    for (int s = threadIdx.x; s < N; s += kThreads) xs[s] = x[s];
    for (int j = threadIdx.x; j < R; j += kThreads) kk[j] = k[j];
    __syncthreads();
    Net m;
    m.n = N;
    m.r = R;
    m.nnz_a = nnz_a;
    m.rent = rent;
    m.sptr = sptr;
    m.sent = sent;
    m.rptr = rptr;
    m.kk = kk;
    assemble_newton_matrix<double>(m, xs, h, M, N);
}

cudaError_t newton_matrix_launch(int N, int R, int nnz_a, const int *rptr, const int *rent,
                                 const int *sptr, const int *sent, const double *k,
                                 const double *x, double h, double *M, cudaStream_t stream) {
    const int64_t smem = int64_t(N + R) * 8 + int64_t(R + 1) * 4;
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(newton_matrix_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    newton_matrix_kernel<<<1, kThreads, smem, stream>>>(N, R, nnz_a, rptr, rent, sptr, sent, k,
                                                       x, h, M);
    return cudaGetLastError();
}

// M_b = I - h*J(x_b) for a batch of parameterisations of one network, dense
// row-major, FP64 or FP32 (the matrix the mixed form factors).  The output is
// n_inst*N*N elements against (N+R) doubles read per instance, so the kernel
// is bound by HBM writes.  Each CTA stages its instance's x and k
// in shared memory.  Work units are (instance, chunk of kJacChunk rows): the
// warps write the chunk's identity/zero rows with 16-byte streaming stores,
// then all threads of the CTA compute the chunk's structural nonzeros (one
// per thread) and patch them while those lines are still in L2.  The nonzero pattern comes
// from the host: jptr/jcol/jrow (columns ascending in each row) and, per
// nonzero (i,g), the reactions of H row i in ascending order that have g
// among their reactants (tptr/tent: reaction and net coefficient, then the
// reactant coefficient of g).  Each contributes createJac's term
// (kernels.cuh:219-271): s*k [*a*x_g^(a-1)] * (each other reactant once), so
// the entries are the ones assemble_newton_matrix writes, bit for bit.
constexpr int kJacThreads = 256;
constexpr int kJacWarps = kJacThreads / 32;
constexpr int kJacChunk = 64;

template <typename OT>
__device__ __forceinline__ void warp_identity_row(OT *row, int N, int diag) {
    constexpr int V = 16 / (int)sizeof(OT);
    const int lane = threadIdx.x & 31;
    int head = (int)((((uintptr_t)0 - (uintptr_t)row) & 15) / sizeof(OT));
    if (head > N) head = N;
    for (int c = lane; c < head; c += 32) __stcs(row + c, c == diag ? OT(1) : OT(0));
    const int nv = (N - head) / V;
    OT *body = row + head;
    const int dv = diag - head;  // diagonal position inside the body
    for (int v = lane; v < nv; v += 32) {
        const int c0 = v * V;
        if constexpr (V == 2) {
            double2 w = make_double2(c0 == dv ? 1.0 : 0.0, c0 + 1 == dv ? 1.0 : 0.0);
            __stcs(reinterpret_cast<double2 *>(body) + v, w);
        } else {
            float4 w = make_float4(c0 == dv ? 1.f : 0.f, c0 + 1 == dv ? 1.f : 0.f,
                                   c0 + 2 == dv ? 1.f : 0.f, c0 + 3 == dv ? 1.f : 0.f);
            __stcs(reinterpret_cast<float4 *>(body) + v, w);
        }
    }
    for (int c = head + nv * V + lane; c < N; c += 32) __stcs(row + c, c == diag ? OT(1) : OT(0));
}

struct JacPattern {
    const int *jptr, *jcol, *jrow, *tptr;
    const int2 *tent;  // (make_ent(reaction, net coefficient), coefficient of g)
};

// createJac's entry (i,g) without the identity, same operations in the same
// order as assemble_newton_matrix (non-exact form).
__device__ __forceinline__ double jac_entry(const int *__restrict__ rptr,
                                            const int *__restrict__ rent, const JacPattern &P,
                                            const double *kk, const double *x, int p, int g) {
    double J = 0.0;
    for (int t = __ldg(P.tptr + p), te = __ldg(P.tptr + p + 1); t < te; t++) {
        const int2 tt = __ldg(P.tent + t);
        const int y2 = ent_index(tt.x), s2 = ent_coef(tt.x), a = tt.y;
        double temp = 0.0;
        if (a == 1) temp = temp + (double)s2 * kk[y2];
        else temp = temp + (double)s2 * kk[y2] * (double)a * mypow(x[g], a - 1);
        for (int q2 = __ldg(rptr + y2), en2 = __ldg(rptr + y2 + 1); q2 < en2; q2++) {
            const int o = ent_index(__ldg(rent + q2));
            if (o != g) temp = temp * x[o];
        }
        J = J + temp;
    }
    return J;
}

template <typename OT>
__global__ void __launch_bounds__(kJacThreads) newton_batch_kernel(
    int n_inst, int N, int R, const int *__restrict__ rptr, const int *__restrict__ rent,
    JacPattern P, const double *__restrict__ k, const double *__restrict__ x, double h,
    OT *__restrict__ M) {
    extern __shared__ __align__(16) unsigned char smem[];
    double *xs = reinterpret_cast<double *>(smem);
    double *kk = xs + N;
    const int warp = threadIdx.x >> 5;
    // work units (instance, chunk of rows); each CTA takes a contiguous range
    // of them, so it restages x and k only when the instance changes
    const int nchunk = (N + kJacChunk - 1) / kJacChunk;
    const int64_t units = (int64_t)n_inst * nchunk;
    const int64_t u0 = units * blockIdx.x / gridDim.x, u1 = units * (blockIdx.x + 1) / gridDim.x;
    int staged = -1;
    for (int64_t u = u0; u < u1; u++) {
        const int b = (int)(u / nchunk), r0 = (int)(u % nchunk) * kJacChunk;
        const int r1 = min(N, r0 + kJacChunk);
        if (b != staged) {  // uniform across the CTA
            __syncthreads();  // the previous instance's patches are done with xs/kk
            for (int s = threadIdx.x; s < N; s += kJacThreads) xs[s] = __ldcs(x + (int64_t)b * N + s);
            for (int j = threadIdx.x; j < R; j += kJacThreads) kk[j] = __ldcs(k + (int64_t)b * R + j);
            staged = b;
        }
        OT *Mb = M + (int64_t)b * N * N;
        for (int i = r0 + warp; i < r1; i += kJacWarps)
            warp_identity_row<OT>(Mb + (int64_t)i * N, N, i);
        __syncthreads();  // rows written, xs/kk staged
        for (int p = __ldg(P.jptr + r0) + threadIdx.x, pe = __ldg(P.jptr + r1); p < pe;
             p += kJacThreads) {
            const int i = __ldg(P.jrow + p), g = __ldg(P.jcol + p);
            const double J = jac_entry(rptr, rent, P, kk, xs, p, g);
            const double I = (i == g) ? 1.0 : 0.0;
            Mb[(int64_t)i * N + g] = (OT)(I - h * J);
        }
    }
}

cudaError_t newton_batch_launch(int n_inst, int N, int R, const int *rptr, const int *rent,
                                const int *jac, int64_t nnz, const double *k, const double *x,
                                double h, void *M, bool fp32, int sm_count, cudaStream_t stream) {
    const int64_t smem = int64_t(N + R) * 8;
    if (smem > 160 * 1024) return cudaErrorInvalidValue;
    // jac = [jptr N+1 | jcol nnz | jrow nnz | tptr nnz+1 | pad to 8 bytes | tent]
    JacPattern P;
    P.jptr = jac;
    P.jcol = P.jptr + N + 1;
    P.jrow = P.jcol + nnz;
    P.tptr = P.jrow + nnz;
    const int64_t ints = (int64_t)N + 1 + 2 * nnz + nnz + 1;
    P.tent = reinterpret_cast<const int2 *>(jac + ((ints + 1) & ~int64_t(1)));
    auto launch = [&](auto kern, auto *out) -> cudaError_t {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kJacThreads, (size_t)smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        const int64_t units = (int64_t)n_inst * ((N + kJacChunk - 1) / kJacChunk);
        const int grid = (int)std::min<int64_t>(units, (int64_t)sm_count * per_sm);
        kern<<<grid, kJacThreads, smem, stream>>>(n_inst, N, R, rptr, rent, P, k, x, h, out);
        return cudaGetLastError();
    };
    if (fp32) return launch(newton_batch_kernel<float>, static_cast<float *>(M));
    return launch(newton_batch_kernel<double>, static_cast<double *>(M));
}

// Factor + solve one dense system with the engine's LU (tests).
template <typename LT>
__global__ void __launch_bounds__(kThreads, 1) lu_solve_kernel(int N, LT *A, int ld,
                                                               const double *b, double *x,
                                                               int *info) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int PB = LuShape<LT>::PB;
    __shared__ double red[2 * kWarps + 1];
    __shared__ int ired[kWarps + 2 + PB];
    const SmemLayout L(N, 1, 1, 1, (int)sizeof(LT), PB, 128);
    int *perm = reinterpret_cast<int *>(smem + L.perm);
    LT *bvec = reinterpret_cast<LT *>(smem + L.bvec);
    LT *lt = reinterpret_cast<LT *>(smem + L.lt);
    LT *utile = reinterpret_cast<LT *>(smem + L.utile);
    LT *rowbuf = reinterpret_cast<LT *>(smem + L.rowbuf);
    __shared__ long long cyc[3];
    if (threadIdx.x == 0) cyc[0] = cyc[1] = cyc[2] = 0;
    const int fail = lu_factor<LT>(A, ld, N, perm, lt, utile, rowbuf, red, ired, cyc);
    if (threadIdx.x == 0) *info = fail;
    if (fail) return;
    for (int s = threadIdx.x; s < N; s += kThreads) bvec[s] = (LT)b[perm[s]];
    __syncthreads();
    if constexpr (std::is_same<LT, float>::value) {
        float *dinv = A + (int64_t)N * ld;
        invert_diag_blocks(A, ld, N, perm, dinv);
        __syncthreads();
        lu_solve_fast(A, ld, N, perm, dinv, bvec, reinterpret_cast<float *>(rowbuf));
    } else {
        lu_solve<LT>(A, ld, N, perm, bvec);
    }
    for (int s = threadIdx.x; s < N; s += kThreads) x[s] = (double)bvec[s];
}

// Autotuner probe: every CTA factors the same diagonally dominant N x N
// test matrix `reps` times in its own workspace slot, with rm rows per
// thread in the trailing update (the per-CTA LU in FP64, the Gauss-Jordan
// inverse in FP32) -- the work and the contention of a batch of such
// networks.  *fails counts factorisations that met a zero pivot (none do).
template <typename LT>
__global__ void __launch_bounds__(kThreads, 1) tune_factor_kernel(int N, int rm, int reps,
                                                                  unsigned char *ws,
                                                                  int64_t ws_stride, int *fails) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int PB = LuShape<LT>::PB;
    __shared__ double red[2 * kWarps + 1];
    __shared__ int ired[kWarps + 2 + PB];
    __shared__ long long cyc[3];
    const SmemLayout L(N, 1, 1, 1, (int)sizeof(LT), PB, 128);
    int *perm = reinterpret_cast<int *>(smem + L.perm);
    int *pos = reinterpret_cast<int *>(smem + L.slot);
    LT *lt = reinterpret_cast<LT *>(smem + L.lt);
    LT *utile = reinterpret_cast<LT *>(smem + L.utile);
    LT *rowbuf = reinterpret_cast<LT *>(smem + L.rowbuf);
    LT *dblk = reinterpret_cast<LT *>(smem + L.dblk);
    const int ld = round_up4(N);
    LT *M = reinterpret_cast<LT *>(ws + (int64_t)blockIdx.x * ws_stride);
    if (threadIdx.x == 0) cyc[0] = cyc[1] = cyc[2] = 0;
    for (int r = 0; r < reps; r++) {
        for (int q = threadIdx.x; q < N * ld; q += kThreads) {
            const int i = q / ld, j = q - i * ld;
            uint32_t h = (uint32_t)q * 2654435761u;
            h ^= h >> 15;
            h *= 2246822519u;
            h ^= h >> 13;
            const float v = ((float)(h & 0xffffu) * (1.0f / 65536.0f) - 0.5f) * 0.02f;
            M[q] = (LT)(j >= N ? 0.0f : (i == j ? 1.0f + v : v));
        }
        __syncthreads();
        int f;
        if constexpr (std::is_same<LT, float>::value)
            f = gje_factor(M, ld, N, perm, pos, lt, utile, dblk, rowbuf, red, ired, cyc, rm);
        else
            f = lu_factor<LT>(M, ld, N, perm, lt, utile, rowbuf, red, ired, cyc, rm);
        if (threadIdx.x == 0 && f) atomicAdd(fails, 1);
        __syncthreads();
    }
}

int64_t tune_factor_smem(int N, int precision) {
    return precision == LASSIE_PREC_FP64
               ? SmemLayout(N, 1, 1, 1, 8, LuShape<double>::PB, 128).total
               : SmemLayout(N, 1, 1, 1, 4, LuShape<float>::PB, 128).total;
}

cudaError_t tune_factor_launch(int precision, int N, int rm, int reps, void *ws,
                               int64_t ws_stride, int grid, int *fails, cudaStream_t stream) {
    const int64_t smem = tune_factor_smem(N, precision);
    cudaError_t e;
    if (precision == LASSIE_PREC_FP64) {
        e = cudaFuncSetAttribute(tune_factor_kernel<double>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        tune_factor_kernel<double><<<grid, kThreads, smem, stream>>>(
            N, rm, reps, (unsigned char *)ws, ws_stride, fails);
    } else {
        e = cudaFuncSetAttribute(tune_factor_kernel<float>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        tune_factor_kernel<float><<<grid, kThreads, smem, stream>>>(
            N, rm, reps, (unsigned char *)ws, ws_stride, fails);
    }
    return cudaGetLastError();
}

int64_t lu_solve_smem(int N, int precision) {
    if (precision == LASSIE_PREC_FP64)
        return SmemLayout(N, 1, 1, 1, 8, LuShape<double>::PB, 128).total;
    return SmemLayout(N, 1, 1, 1, 4, LuShape<float>::PB, 128).total;
}

cudaError_t lu_solve_launch(int N, void *A, int ld, const double *b, double *x, int *info,
                            int precision, cudaStream_t stream) {
    const int64_t smem = lu_solve_smem(N, precision);
    if (smem > 220 * 1024) return cudaErrorInvalidValue;
    cudaError_t e;
    if (precision == LASSIE_PREC_FP64) {
        e = cudaFuncSetAttribute(lu_solve_kernel<double>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        lu_solve_kernel<double><<<1, kThreads, smem, stream>>>(N, (double *)A, ld, b, x, info);
    } else {
        e = cudaFuncSetAttribute(lu_solve_kernel<float>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        lu_solve_kernel<float><<<1, kThreads, smem, stream>>>(N, (float *)A, ld, b, x, info);
    }
    return cudaGetLastError();
}

}  // namespace lassie
