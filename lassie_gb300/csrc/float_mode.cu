// The reference's single-precision mode (`-p float`, Simulation<float>,
// simulator.cu:289-294): LASSIE's loop with the state, the rate constants,
// the stage vectors, the step sizes and the Newton matrix in float, and
// double temporaries exactly where C++ promotion puts them in the reference
// kernels (kernels.cuh:5-199, 205-300, 393-402, 462-535): the RHS sums each
// reaction term in double and rounds the running sum to float after every
// term; the RKF45 combinations are evaluated in double from float stages
// and stored as float; the step-size factor is 0.84 * pow(atol/R, 0.25f)
// with float operands.
//
// This file is compiled with the reference's own device flags
// (--use_fast_math: flush-to-zero, fast float division and pow, and FMA
// contraction), and its kernels write every expression with the reference's
// types and order, so that the compiler treats them alike; the scalar loop
// logic that the reference runs on the host in float (Simulation.cuh:
// 737-790) uses round-to-nearest intrinsics, which are never contracted.
// The dense solve is a float LU with partial pivoting in place of
// cuSOLVER's Sgetrf/Sgetrs (Simulation.cuh:1280-1326), and the Newton norm
// sums its float squares in a fixed block order in place of thrust's.
//
// One CTA integrates one instance at a time (work queue, largest first);
// networks of at most kThreads species.  Not a fast path: it exists so that
// `-p float` computes what the reference computes.
#include <cmath>
#include <cstdint>

#include <cuda_runtime.h>

#include "common.cuh"
#include "lassie_gb300.h"

namespace lassie {
namespace {

__device__ __forceinline__ uint64_t fm_now() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// myPow<float> (kernels.cuh:52-63): the product in float, returned as double
__device__ __forceinline__ double fm_pow(float base, int ex) {
    float potenza = 1.0;
    while (ex > 0) {
        potenza = potenza * base;
        ex--;
    }
    return potenza;
}

struct FNet {
    int n, r;
    const int *rptr, *rent, *sptr, *sent;
    const float *c;
};

// generate_ode<float> for species i (kernels.cuh:5-50)
__device__ float fm_rhs(const FNet &m, int i, const float *y0) {
    float y1 = 0;
    for (int e = m.sptr[i]; e < m.sptr[i + 1]; e++) {
        const int ent = m.sent[e];
        const int y = ent_index(ent);
        const int signum = ent_coef(ent);
        const int start_moni = m.rptr[y], end_moni = m.rptr[y + 1];
        double temp = 0;
        if (end_moni > start_moni) {
            for (int j = start_moni; j < end_moni; j++) {
                const int re = m.rent[j];
                if (j == start_moni)
                    temp += signum * m.c[y] * fm_pow(y0[ent_index(re)], ent_coef(re));
                else
                    temp *= fm_pow(y0[ent_index(re)], ent_coef(re));
            }
            y1 = y1 + temp;
        } else {
            y1 = y1 + signum * m.c[y];
        }
    }
    return y1;
}

// createJac_<float> entry (index2, gid) (kernels.cuh:219-271)
__device__ float fm_jac(const FNet &m, int index2, int gid, const float *y0) {
    float y1 = 0;
    for (int e = m.sptr[index2]; e < m.sptr[index2 + 1]; e++) {
        const int ent = m.sent[e];
        const int y = ent_index(ent);
        const int signum = ent_coef(ent);
        const int start_moni = m.rptr[y], end_moni = m.rptr[y + 1];
        double temp = 0;
        for (int j = start_moni; j < end_moni; j++) {
            const int re = m.rent[j];
            const int sp = ent_index(re), st = ent_coef(re);
            if ((st == 1) & (sp == gid)) {
                temp = temp + signum * m.c[y];
                for (int jj = start_moni; jj < end_moni; jj++)
                    if (ent_index(m.rent[jj]) != gid) temp = temp * y0[ent_index(m.rent[jj])];
            } else if ((st > 1) & (sp == gid)) {
                temp = temp + signum * m.c[y] * st * fm_pow(y0[sp], st - 1);
                for (int jj = start_moni; jj < end_moni; jj++)
                    if (ent_index(m.rent[jj]) != gid) temp = temp * y0[ent_index(m.rent[jj])];
            }
        }
        y1 = y1 + temp;
    }
    return y1;
}

constexpr int kW = kThreads / 32;

// minimum of doubles, a leading NaN kept (thrust::min_element over the
// deltas converted to double, Simulation.cuh:754-756)
__device__ double fm_block_min(double v, bool nan0, double *red, int *flag) {
    const double big = INFINITY;
    double x = isnan(v) ? big : v;
    for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = x;
    if (threadIdx.x == 0) *flag = nan0 ? 1 : 0;
    __syncthreads();
    double s = l < kW ? red[l] : big;
    for (int o = kW / 2; o > 0; o >>= 1) s = fmin(s, __shfl_xor_sync(0xffffffffu, s, o));
    s = __shfl_sync(0xffffffffu, s, 0);
    return *flag ? (double)NAN : s;
}

// float sum in a fixed order (the reference's thrust reduction of the
// float squares, Simulation.cuh:883-890)
__device__ float fm_block_sum(float v, float *red) {
    for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    float s = l < kW ? red[l] : 0.0f;
    for (int o = kW / 2; o > 0; o >>= 1) s = __fadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
    return __shfl_sync(0xffffffffu, s, 0);
}

// In-place LU with partial pivoting of the row-major n x n float matrix A
// (stride ld): pivot = largest |value| (first on ties), row swaps recorded
// in piv; 0, or j + 1 when column j has only zeros.
__device__ int fm_lu(float *A, int ld, int n, int *piv, float *redv, int *redi) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int j = 0; j < n; j++) {
        float best = -1.0f;
        int bi = n;
        for (int i = j + tid; i < n; i += kThreads) {
            const float v = fabsf(A[(int64_t)i * ld + j]);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        __syncthreads();
        if (lane == 0) {
            redv[w] = best;
            redi[w] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            float b = -1.0f;
            int p = n;
            for (int q = 0; q < kW; q++)
                if (redv[q] > b || (redv[q] == b && redi[q] < p)) {
                    b = redv[q];
                    p = redi[q];
                }
            piv[j] = p;
            redi[kW] = (p >= n || !(b > 0.0f)) ? 1 : 0;
        }
        __syncthreads();
        if (redi[kW]) return j + 1;
        const int p = piv[j];
        if (p != j)
            for (int c = tid; c < n; c += kThreads) {
                const float t = A[(int64_t)j * ld + c];
                A[(int64_t)j * ld + c] = A[(int64_t)p * ld + c];
                A[(int64_t)p * ld + c] = t;
            }
        __syncthreads();
        const float d = A[(int64_t)j * ld + j];
        for (int i = j + 1 + tid; i < n; i += kThreads) A[(int64_t)i * ld + j] /= d;
        __syncthreads();
        const int m = n - j - 1;
        for (int q = tid; q < m * m; q += kThreads) {
            const int i = j + 1 + q / m, c = j + 1 + q % m;
            A[(int64_t)i * ld + c] -= A[(int64_t)i * ld + j] * A[(int64_t)j * ld + c];
        }
        __syncthreads();
    }
    return 0;
}

// b <- A^-1 b with the factors of fm_lu (one thread: row interchanges,
// forward and backward substitution)
__device__ void fm_lu_solve(const float *A, int ld, int n, const int *piv, float *b) {
    if (threadIdx.x == 0) {
        for (int j = 0; j < n; j++) {
            const int p = piv[j];
            if (p != j) {
                const float t = b[j];
                b[j] = b[p];
                b[p] = t;
            }
        }
        for (int i = 0; i < n; i++) {
            float acc = b[i];
            for (int j = 0; j < i; j++) acc -= A[(int64_t)i * ld + j] * b[j];
            b[i] = acc;
        }
        for (int i = n - 1; i >= 0; i--) {
            float acc = b[i];
            for (int j = i + 1; j < n; j++) acc -= A[(int64_t)i * ld + j] * b[j];
            b[i] = acc / A[(int64_t)i * ld + i];
        }
    }
    __syncthreads();
}

__device__ __forceinline__ bool fm_bad(float v) { return isnan(v) || isinf(v) || v < 0; }

// float vectors of one instance in shared memory, in this order
constexpr int kFVecs = 16;

__device__ void fm_integrate(const LaunchParams &P, int id, unsigned char *smem, double *redd,
                             float *redf, int *redi, InstDesc &D, InstResult &st, uint64_t deadline) {
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
    // shared memory: kFVecs float vectors of nmax, rate constants, structure
    float *vb = reinterpret_cast<float *>(smem);
    const int vs = P.nmax;
    float *y1 = vb, *u = vb + vs, *k1 = vb + 2 * vs, *k2 = vb + 3 * vs, *k3 = vb + 4 * vs,
          *k4 = vb + 5 * vs, *k5 = vb + 6 * vs, *k6 = vb + 7 * vs, *w1 = vb + 8 * vs,
          *w2 = vb + 9 * vs, *delta = vb + 10 * vs, *feed = vb + 11 * vs, *tol = vb + 12 * vs,
          *yv = vb + 13 * vs, *x = vb + 14 * vs, *xJ = vb + 15 * vs;
    float *c = vb + kFVecs * vs;
    int *rptr = reinterpret_cast<int *>(c + P.rmax);
    int *sptr = rptr + P.rmax + 1;
    int *rent = sptr + P.nmax + 1;
    int *sent = rent + (P.amax > 0 ? P.amax : 1);
    int *piv = sent + (P.hmax > 0 ? P.hmax : 1);
    for (int q = tid; q <= R; q += kThreads) rptr[q] = ia[D.rxn_ptr + q];
    for (int q = tid; q <= N; q += kThreads) sptr[q] = ia[D.sp_ptr + q];
    for (int q = tid; q < D.nnz_a; q += kThreads) rent[q] = ia[D.rxn_ent + q];
    for (int q = tid; q < D.nnz_h; q += kThreads) sent[q] = ia[D.sp_ent + q];
    // Reader.h:47,64: strtod, then the conversion to T = float
    for (int j = tid; j < R; j += kThreads) c[j] = (float)da[D.k + j];
    for (int s = tid; s < N; s += kThreads) {
        y1[s] = (float)da[D.x0 + s];
        u[s] = 0.0f;
        feed[s] = D.feed >= 0 ? (float)da[D.feed + s] : 0.0f;
        tol[s] = D.atol >= 0 ? (float)da[D.atol + s] : (float)1e-12;
    }
    __syncthreads();
    FNet m{N, R, rptr, rent, sptr, sent, c};
    float *Mx = reinterpret_cast<float *>(P.workspace + (int64_t)blockIdx.x * P.ws_stride);
    const int ld = round_up4(N);
    const double *tv = da + D.t;
    const int *cs = D.cs >= 0 ? ia + D.cs : nullptr;
    double *out = P.out + D.out;
    const int nt = D.nt, ncs = D.ncs;
    // Simulation.cuh:632-672, T = float
    const float dt_rkf = (float)D.rkf_step, dt_ei = (float)D.be_step;
    const float tollN = (float)D.newton_tol, isStiff = (float)D.stiffness_tol;
    const int iterN = (int)D.newton_iter;
    int i = 0;
    float t1 = nt > 0 ? (float)tv[0] : 0.0f;
    float t = 0;
    float dt = dt_rkf;
    float newDtBDF = dt_ei;
    int status = LASSIE_OK;
    int64_t outer = 0;
    while (i < nt) {
        if (D.max_steps > 0 && outer >= D.max_steps) {
            status = LASSIE_ERR_MAX_STEPS;
            break;
        }
        if (deadline && (outer & 63) == 0) {
            if (tid == 0) redi[0] = fm_now() > deadline;
            __syncthreads();
            const int exp = redi[0];
            __syncthreads();
            if (exp) {
                status = LASSIE_ERR_DEADLINE;
                break;
            }
        }
        outer++;
        if (fabs(__fsub_rn(t1, t)) < 1e-5) {
            for (int j = tid; j < ncs; j += kThreads) out[(int64_t)i * ncs + j] = y1[cs ? cs[j] : j];
            i++;
            if (i >= nt) break;
            t1 = (float)tv[i];
        }
        // RKF45 stages (kernels.cuh:68-182)
        for (int s = tid; s < N; s += kThreads) k1[s] = fm_rhs(m, s, y1);
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) {
            if (feed[s] != 0.0) k1[s] = feed[s];
            else {
                k1[s] = k1[s] * dt;
                u[s] = y1[s] + k1[s] / 4.0;
            }
        }
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) k2[s] = fm_rhs(m, s, u);
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) {
            if (feed[s] != 0.0) k2[s] = feed[s];
            else {
                k2[s] = k2[s] * dt;
                u[s] = y1[s] + (3.0 * k1[s]) / 32.0 + (9.0 * k2[s]) / 32.0;
            }
        }
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) k3[s] = fm_rhs(m, s, u);
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) {
            if (feed[s] != 0.0) k3[s] = feed[s];
            else {
                k3[s] = k3[s] * dt;
                u[s] = y1[s] + (1932.0 * k1[s]) / 2197.0 - (7200.0 * k2[s]) / 2197.0 +
                       (7296.0 * k3[s]) / 2197.0;
            }
        }
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) k4[s] = fm_rhs(m, s, u);
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) {
            if (feed[s] != 0.0) k4[s] = feed[s];
            else {
                k4[s] = k4[s] * dt;
                u[s] = y1[s] + (439.0 * k1[s]) / 216.0 - (8.0 * k2[s]) + (3680.0 * k3[s]) / 513.0 -
                       (845.0 * k4[s]) / 4104.0;
            }
        }
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) k5[s] = fm_rhs(m, s, u);
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) {
            if (feed[s] != 0.0) k5[s] = feed[s];
            else {
                k5[s] = k5[s] * dt;
                u[s] = y1[s] - (8.0 * k1[s]) / 27.0 + (2.0 * k2[s]) - (3544.0 * k3[s]) / 2565.0 +
                       (1859.0 * k4[s]) / 4104.0 - (11.0 * k5[s]) / 40.0;
            }
        }
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) k6[s] = fm_rhs(m, s, u);
        __syncthreads();
        int okc = 1;
        bool nan0 = false;
        double dloc = INFINITY;
        for (int s = tid; s < N; s += kThreads) {
            if (feed[s] != 0.0) k6[s] = feed[s];
            else k6[s] = k6[s] * dt;
            // rk_Fehlberg_agg (kernels.cuh:155-182)
            if (feed[s] != 0.0) {
                w1[s] = feed[s];
                w2[s] = feed[s];
            } else {
                w1[s] = y1[s] + (25.0 * k1[s]) / 216.0 + (1408.0 * k3[s]) / 2565.0 +
                        (2197.0 * k4[s]) / 4104.0 - k5[s] / 5.0;
                w2[s] = y1[s] + (16.0 * k1[s]) / 135.0 + (6656.0 * k3[s]) / 12825.0 +
                        (28561.0 * k4[s]) / 56430.0 - (9.0 * k5[s] / 50.0) + (2.0 * k6[s]) / 55.0;
            }
            // calculate_delta (kernels.cuh:184-199)
            const float R_ = std::fabs(w1[s] - w2[s]) / dt;
            const float ex = 0.25;
            delta[s] = 0.84 * std::pow(tol[s] / R_, ex);
            if (!(R_ <= tol[s] && !isnan(R_) && !isinf(R_) && w1[s] > 0)) okc = 0;
            const double dd = (double)delta[s];
            if (s == 0 && isnan(dd)) nan0 = true;
            if (!isnan(dd)) dloc = fmin(dloc, dd);
        }
        const int all_ok = __syncthreads_and(okc);
        const int anynan0 = __syncthreads_or(nan0);
        const double dmin = fm_block_min(dloc, anynan0 != 0, redd, redi);
        if (all_ok) {
            // Simulation.cuh:742-768 (host code, float)
            for (int s = tid; s < N; s += kThreads) y1[s] = w1[s];
            __syncthreads();
            float d_temp = (float)dmin;
            d_temp = __fmul_rn(dt, d_temp);
            if (__fadd_rn(t, d_temp) > t1) dt = fabsf(__fsub_rn(t1, t));
            else dt = d_temp;
            t = __fadd_rn(t, dt);
            if (tid == 0) st.rkf_accepts++;
            continue;
        }
        // Simulation.cuh:769-921
        {
            const float d_temp = (float)dmin;
            const float dt_old = dt;
            dt = __fmul_rn(dt, d_temp);
            if (!((dt < isStiff) | isnan(dt) | isinf(dt) | (fabsf(__fsub_rn(dt_old, dt)) < 1e-3))) {
                if (tid == 0) st.rkf_retries++;
                continue;
            }
        }
        dt = newDtBDF;
        if (__fadd_rn(t, dt) > t1) dt = fabsf(__fsub_rn(t1, t));
        for (int s = tid; s < N; s += kThreads) yv[s] = y1[s];
        __syncthreads();
        if (tid == 0) st.be_steps++;
        int itN = 0;
        float errN = 1000;
        bool luFail = false;
        while ((itN < iterN) & (errN > tollN)) {
            if (deadline && (itN & 63) == 63) {
                if (tid == 0) redi[0] = fm_now() > deadline;
                __syncthreads();
                const int exp = redi[0];
                __syncthreads();
                if (exp) {
                    status = LASSIE_ERR_DEADLINE;
                    break;
                }
            }
            for (int s = tid; s < N; s += kThreads) x[s] = fm_rhs(m, s, yv);
            __syncthreads();
            // calculate_nonLinear1th (kernels.cuh:289-300)
            for (int s = tid; s < N; s += kThreads) x[s] = -(yv[s] - y1[s] - dt * x[s]);
            __syncthreads();
            if (itN == 0) {
                // createJac + aggiorna_Jacobiano1 (kernels.cuh:205-271, 393-402);
                // Mx[row * ld + col] = I - dt * J(row, col)
                for (int q = tid; q < N * N; q += kThreads) {
                    const int row = q / N, col = q - row * N;
                    const float J = fm_jac(m, row, col, yv);
                    const float I = row == col ? 1.0f : 0.0f;
                    Mx[(int64_t)row * ld + col] = I - dt * J;
                }
                __syncthreads();
                if (tid == 0) st.lu_factorisations++;
                if (fm_lu(Mx, ld, N, piv, redf, redi) != 0) luFail = true;
            }
            if (luFail) {
                // Simulation.cuh:869-875, kernels.cuh:512-521
                for (int s = tid; s < N; s += kThreads)
                    if (fm_bad(yv[s])) yv[s] = y1[s];
                __syncthreads();
                newDtBDF = __fmul_rn(dt, 0.1f);
                if (tid == 0) st.lu_failures++;
                break;
            }
            for (int s = tid; s < N; s += kThreads) xJ[s] = x[s];
            __syncthreads();
            fm_lu_solve(Mx, ld, N, piv, xJ);
            // aggiorna_Newton (kernels.cuh:462-477), square functor and sum
            float sq = 0.0f;
            for (int s = tid; s < N; s += kThreads) {
                const float old = yv[s];
                if (feed[s] == 0) yv[s] = yv[s] + xJ[s];
                else yv[s] = feed[s];
                xJ[s] = yv[s] - old;
                sq = __fadd_rn(sq, __fmul_rn(xJ[s], xJ[s]));
            }
            errN = __fsqrt_rn(fm_block_sum(sq, redf));
            itN = itN + 1;
            if (tid == 0) st.newton_iters++;
        }
        if (status != LASSIE_OK) break;
        if (!luFail) {
            // Simulation.cuh:894-909
            bool anybad = false;
            for (int s = tid; s < N; s += kThreads) anybad |= fm_bad(yv[s]);
            if (__syncthreads_or(anybad)) {
                for (int s = tid; s < N; s += kThreads)
                    if (fm_bad(yv[s])) yv[s] = y1[s];
                newDtBDF = __fmul_rn(dt, 0.1f);
                if (tid == 0) st.nan_reverts++;
            }
        }
        __syncthreads();
        for (int s = tid; s < N; s += kThreads) y1[s] = yv[s];
        __syncthreads();
        t = __fadd_rn(t, dt);
    }
    __syncthreads();
    if (tid == 0) {
        st.outer_iters = outer;
        st.t_final = t;
        st.dt_be_final = newDtBDF;
        st.status = status;
        st.cycles_total = clock64() - c_start;
        P.res[id] = st;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kThreads, 1) float_kernel(LaunchParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double redd[kW];
    __shared__ float redf[kW];
    __shared__ int redi[kW + 1];
    __shared__ InstDesc D;
    __shared__ InstResult st;
    __shared__ int next;
    __shared__ uint64_t start;
    if (threadIdx.x == 0) start = fm_now();
    __syncthreads();
    const uint64_t deadline = P.deadline_ns ? start + P.deadline_ns : 0;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(P.queue, 1);
        __syncthreads();
        const int q = next;
        __syncthreads();
        if (q >= P.n_inst) break;
        fm_integrate(P, P.order[q], smem, redd, redf, redi, D, st, deadline);
    }
}

}  // namespace

int64_t float_smem_bytes(int nmax, int rmax, int amax, int hmax) {
    return (int64_t)kFVecs * nmax * 4 + (int64_t)rmax * 4 + (int64_t)(rmax + 1) * 4 +
           (int64_t)(nmax + 1) * 4 + (int64_t)(amax > 0 ? amax : 1) * 4 +
           (int64_t)(hmax > 0 ? hmax : 1) * 4 + (int64_t)nmax * 4 + 64;
}

cudaError_t float_configure(int64_t smem) {
    return cudaFuncSetAttribute(float_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
}

cudaError_t float_launch(const LaunchParams &P, int grid, int64_t smem, cudaStream_t stream) {
    float_kernel<<<grid, kThreads, smem, stream>>>(P);
    return cudaGetLastError();
}

}  // namespace lassie
