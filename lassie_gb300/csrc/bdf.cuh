// Standard controller: variable-order (1..5), quasi-constant-step BDF in
// backward-difference form with rtol/atol error control, one CTA per
// instance inside compat_kernel<double> (Shampine & Reichelt, "The MATLAB
// ODE Suite", SIAM J. Sci. Comput. 18, 1997, with kappa = 0).
//
// LASSIE itself only runs backward Euler with a fixed step; its sources also
// carry BDF2-6 correctors for a constant step that nothing calls
// (calculate_nonLinear2th..6th, kernels.cuh:302-390, and the Newton matrices
// aggiorna_Jacobiano2..6, kernels.cuh:405-457).  At a constant step h and
// order k the corrector here is that classical BDFk formula, with BDF5's
// denominator 137 (the reference writes 147, BDF6's), and the Newton matrix
// is I - beta_k h J with beta_k = 1 / (1 + 1/2 + ... + 1/k).  What this adds
// is the error control, the step and order selection, and the interpolation
// of the history when the step changes.
//
// Per attempt (order q, differences D[0..q+2] of the accepted solutions):
//   y0  = D[0] + D[1] + ... + D[q]                 prediction
//   psi = (g_1 D[1] + ... + g_q D[q]) / g_q,       g_j = 1 + 1/2 + ... + 1/j
//   d   solves d - c f(y0 + d) + psi = 0,  c = h / g_q, by at most 4
//       modified Newton iterations on I - c J (J exact, from the last point
//       where it was evaluated)
//   err = d / (q + 1), RMS norm weighted by atol + rtol |y0 + d|
// accepted: D[q+2] = d - D[q+1], D[q+1] = d, D[i] += D[i+1] for i = q..0;
// samples in (t, t + h] come from the degree-q interpolant; after q + 1
// steps of one size, the order moves to whichever of q-1, q, q+1 allows the
// largest step.  Step changes rescale D (D <- (R(f) U)^T D).  Step factors
// are rounded down to multiples of 2^-10, so that a last-bit difference of
// pow() between platforms does not change h.  The CPU oracle follows the
// same operation order, and the norms sum in block_sum's order, so the FP64
// form (FP64 LU) reproduces the oracle bit for bit.  The mixed form
// (LT = float) uses an FP32 Gauss-Jordan inverse of I - cJ as the modified
// Newton iteration matrix: the corrections are applied to FP64 residuals,
// so the converged step solves the same FP64 equations to the Newton
// tolerance, with possibly more iterations.
//
// Included by compat_engine.cu after the RHS, Jacobian, LU and reduction
// helpers (namespace lassie).

constexpr int kBdfMaxOrder = 5;
constexpr int kBdfNewtonMaxIter = 4;
constexpr int kBdfFallback = 4;  // Newton failures in a row before FP64 factors (mixed)
constexpr int kBdfVecs = kBdfMaxOrder + 3 + 12;  // differences + work vectors
constexpr double kBdfMinFactor = 0.2, kBdfMaxFactor = 10.0;
constexpr double kBdfEps = 2.220446049250313e-16;  // 2^-52

__device__ __forceinline__ double bdf_quantize(double f) { return floor(f * 1024.0) / 1024.0; }

// the next double above a finite t (C's nextafter(t, +inf))
__device__ __forceinline__ double bdf_next_up(double t) {
    const long long b = __double_as_longlong(t);
    if (t == 0.0) return __longlong_as_double(1LL);
    return __longlong_as_double(t > 0.0 ? b + 1 : b - 1);
}

// sqrt(mean((v / scale)^2)) over the CTA
__device__ __forceinline__ double bdf_rms(const double *v, const double *scale, int N,
                                          double *red) {
    double part = 0.0;
    for (int s = threadIdx.x; s < N; s += kThreads) {
        const double q = v[s] / scale[s];
        part = part + q * q;
    }
    return sqrt(block_sum(part, red) / (double)N);
}

// D[0..q] <- RU^T D[0..q], RU = R(factor) R(1), R(f)[i][j] = prod_{r=1..i}
// (r - 1 - f j) / r for j >= 1, R[0][j] = 1, R[i>0][0] = 0.
// The (q+1) x (q+1) matrix RU is formed once, by thread 0 (FP64 is slow on
// this GPU: 512 threads forming it redundantly cost tens of microseconds),
// and read by every thread from shared memory.
__device__ __noinline__ void bdf_change_d(double *Dd, int vstride, int N, int q, double factor) {
    __shared__ double RU[kBdfMaxOrder + 1][kBdfMaxOrder + 1];
    if (threadIdx.x == 0) {
        double R[kBdfMaxOrder + 1][kBdfMaxOrder + 1], U[kBdfMaxOrder + 1][kBdfMaxOrder + 1];
#pragma unroll 1
        for (int pass = 0; pass < 2; pass++) {
            const double f = pass == 0 ? factor : 1.0;
            double (*M)[kBdfMaxOrder + 1] = pass == 0 ? R : U;
            for (int j = 0; j <= q; j++) M[0][j] = 1.0;
            for (int i = 1; i <= q; i++)
                for (int j = 0; j <= q; j++) {
                    const double mij =
                        j == 0 ? 0.0 : ((double)(i - 1) - f * (double)j) / (double)i;
                    M[i][j] = M[i - 1][j] * mij;
                }
        }
        for (int i = 0; i <= q; i++)
            for (int j = 0; j <= q; j++) {
                double a = 0.0;
                for (int l = 0; l <= q; l++) a = a + R[i][l] * U[l][j];
                RU[i][j] = a;
            }
    }
    __syncthreads();
    for (int s = threadIdx.x; s < N; s += kThreads) {
        double nv[kBdfMaxOrder + 1];
        for (int j = 0; j <= q; j++) {
            double a = 0.0;
            for (int i = 0; i <= q; i++) a = a + RU[i][j] * Dd[(int64_t)i * vstride + s];
            nv[j] = a;
        }
        for (int j = 0; j <= q; j++) Dd[(int64_t)j * vstride + s] = nv[j];
    }
    __syncthreads();
}

template <typename LT>
__device__ __noinline__ void bdf_integrate(const LaunchParams &P, int id, unsigned char *smem, double *red,
                              int *ired, InstDesc &D, InstResult &st, uint64_t deadline) {
    constexpr bool kMixed = std::is_same<LT, float>::value;
    constexpr int PB = LuShape<LT>::PB, TN = LuShape<LT>::TN;
    __shared__ double s_bcast[1];  // a scalar formed by thread 0 for all
    __shared__ int s_ibcast;
    const int tid = threadIdx.x;
    if (tid == 0) {
        D = P.inst[id];
        st = InstResult{};
    }
    __syncthreads();
    const int N = D.n, R = D.r;
    const int *ia = P.iarena;
    const double *da = P.darena;
    const SmemLayout L(P.nmax, P.rmax, P.amax, P.hmax, (int)sizeof(LT), PB, TN, kBdfVecs);
    double *vbase = reinterpret_cast<double *>(smem + L.vec);
    const int vstride = P.nmax;
    double *kk = reinterpret_cast<double *>(smem + L.kk);
    double *pw = reinterpret_cast<double *>(smem + L.pw);
    double *qr = reinterpret_cast<double *>(smem + L.qr);
    int *w_rptr = reinterpret_cast<int *>(smem + L.rptr);
    int *w_sptr = reinterpret_cast<int *>(smem + L.sptr);
    int *w_sent = reinterpret_cast<int *>(smem + L.sent);
    int *w_rent = reinterpret_cast<int *>(smem + L.rent);
    int *perm = reinterpret_cast<int *>(smem + L.perm);
    LT *bvec = reinterpret_cast<LT *>(smem + L.bvec);
    LT *lt = reinterpret_cast<LT *>(smem + L.lt);
    LT *utile = reinterpret_cast<LT *>(smem + L.utile);
    LT *rowbuf = reinterpret_cast<LT *>(smem + L.rowbuf);
    LT *dblk = reinterpret_cast<LT *>(smem + L.dblk);
    int *pos = reinterpret_cast<int *>(smem + L.slot);
    for (int q = tid; q < D.nnz_a; q += kThreads) w_rent[q] = ia[D.rxn_ent + q];
    for (int q = tid; q < D.nnz_h; q += kThreads) w_sent[q] = ia[D.sp_ent + q];
    for (int q = tid; q <= N; q += kThreads) w_sptr[q] = ia[D.sp_ptr + q];
    for (int j = tid; j < R; j += kThreads) kk[j] = da[D.k + j];
    for (int j = tid; j <= R; j += kThreads) w_rptr[j] = ia[D.rxn_ptr + j];
    Net m;
    m.n = N;
    m.r = R;
    m.nnz_a = D.nnz_a;
    m.rent = w_rent;
    m.sptr = w_sptr;
    m.sent = w_sent;
    m.rptr = w_rptr;
    m.kk = kk;

    constexpr int Q = kBdfMaxOrder + 3;
    double *Dd = vbase;  // Q difference vectors
    double *ypred = vbase + (int64_t)Q * vstride;
    double *psi = ypred + vstride, *dv = psi + vstride, *ynew = dv + vstride;
    double *f = ynew + vstride, *dy = f + vstride, *scale = dy + vstride;
    double *atolv = scale + vstride, *aux = atolv + vstride, *xj = aux + vstride;
    double *fedv = xj + vstride, *res = fedv + vstride;

    const double rtol = P.rtol;
    for (int s = tid; s < N; s += kThreads) {
        const double fd = D.feed >= 0 ? da[D.feed + s] : 0.0;
        fedv[s] = fd;
        atolv[s] = D.atol >= 0 ? da[D.atol + s] : P.atol;
        xj[s] = fd != 0.0 ? fd : da[D.x0 + s];
        for (int j = 0; j < Q; j++) Dd[(int64_t)j * vstride + s] = 0.0;
    }
    __syncthreads();

    const double *tv = da + D.t;
    const int *cs = D.cs >= 0 ? ia + D.cs : nullptr;
    const int ncs = D.ncs, nt = D.nt;
    double *out = P.out + D.out;
    LT *M = reinterpret_cast<LT *>(P.workspace + (int64_t)blockIdx.x * P.ws_stride);
    const int ld = round_up4(N);
    long long cyc[3] = {0, 0, 0};
    long long c_mark = 0;
    const long long c_start = clock64();

    double gamma[kBdfMaxOrder + 2], econst[kBdfMaxOrder + 2];
    gamma[0] = 0.0;
    for (int j = 1; j <= kBdfMaxOrder + 1; j++) gamma[j] = gamma[j - 1] + 1.0 / (double)j;
    for (int j = 0; j <= kBdfMaxOrder + 1; j++) econst[j] = 1.0 / (double)(j + 1);
    const double newton_tol = fmax(10.0 * kBdfEps / rtol, fmin(0.03, sqrt(rtol)));
    const int max_order = P.max_order >= 1 && P.max_order <= kBdfMaxOrder ? P.max_order
                                                                            : kBdfMaxOrder;

    // f(x) with fed species held (zero slope); x in smem, result in fo
    auto rhs = [&](const double *x, double *fo) {
        rhs_rates(m, x, pw, qr);
        __syncthreads();
        for (int s = tid; s < N; s += kThreads)
            fo[s] = fedv[s] != 0.0 ? 0.0 : rhs_species_r(m, s, pw, qr);
        __syncthreads();
    };

    // nt >= 1 below (no samples: nothing to integrate)
    double tc = nt > 0 ? tv[0] : 0.0;
    const double t_end = nt > 0 ? tv[nt - 1] : 0.0;
    int isample = 0;
    while (isample < nt && tv[isample] <= tc) {
        for (int c = tid; c < ncs; c += kThreads)
            out[(int64_t)isample * ncs + c] = xj[cs ? cs[c] : c];
        isample++;
    }
    int status = LASSIE_OK;
    int q = 1;
    // mixed form: a Newton failure on FP32 factors retries the step on FP64
    // factors at the same size; after kBdfFallback FP32 failures without an
    // FP32 success in between, the instance factors in FP64 for the rest of
    // its integration (the workspace has FP64 room; the FP32 panel buffers
    // are as large as the FP64 ones, the solve vector is res)
    bool fp64_lu = !kMixed;
    int fail_run = 0, fp64_left = 0;
    double h = 0.0;
    int64_t attempts = 0, rhs_evals = 0, jac_evals = 0;
    if (isample < nt) {
        // y = x0 (fed species at their feed) is in xj; f0 in f
        rhs(xj, f);
        rhs_evals++;
        if (P.first_step > 0.0) {
            h = P.first_step;
        } else {
            // initial step (Hairer, Norsett & Wanner, II.4, order 1)
            for (int s = tid; s < N; s += kThreads) scale[s] = atolv[s] + fabs(xj[s]) * rtol;
            __syncthreads();
            const double d0 = bdf_rms(xj, scale, N, red), d1 = bdf_rms(f, scale, N, red);
            double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
            h0 = fmin(h0, t_end - tc);
            for (int s = tid; s < N; s += kThreads) ynew[s] = xj[s] + h0 * f[s];
            __syncthreads();
            rhs(ynew, dy);
            rhs_evals++;
            for (int s = tid; s < N; s += kThreads) aux[s] = dy[s] - f[s];
            __syncthreads();
            const double d2 = bdf_rms(aux, scale, N, red) / h0;
            const double h1 = (d1 <= 1e-15 && d2 <= 1e-15) ? fmax(1e-6, h0 * 1e-3)
                                                           : sqrt(0.01 / fmax(d1, d2));
            h = fmin(fmin(100.0 * h0, h1), t_end - tc);
        }
        if (P.max_step > 0.0 && h > P.max_step) h = P.max_step;
        for (int s = tid; s < N; s += kThreads) {
            Dd[s] = xj[s];
            Dd[vstride + s] = h * f[s];
        }
        __syncthreads();
        // J is evaluated at xj (here the start); it counts as current only
        // within the step that evaluated it
        jac_evals++;
        bool jac_current = false, lu_valid = false;
        int n_equal = 0;
        while (isample < nt && status == LASSIE_OK) {
            bool accepted = false;
            int n_iter = 0;
            double err_norm = 0.0;
            while (!accepted) {
                if (D.max_steps > 0 && attempts >= D.max_steps) {
                    status = LASSIE_ERR_MAX_STEPS;
                    break;
                }
                if (deadline && (attempts & 63) == 63) {
                    if (tid == 0) ired[0] = global_ns() > deadline;
                    __syncthreads();
                    const bool expired = ired[0] != 0;
                    __syncthreads();
                    if (expired) {
                        status = LASSIE_ERR_DEADLINE;
                        break;
                    }
                }
                attempts++;
                const double min_step = 10.0 * (bdf_next_up(tc) - tc);
                if (P.max_step > 0.0 && h > P.max_step) {
                    bdf_change_d(Dd, vstride, N, q, P.max_step / h);
                    h = P.max_step;
                    n_equal = 0;
                    lu_valid = false;
                }
                if (h < min_step) {
                    status = LASSIE_ERR_STEP_TOO_SMALL;
                    break;
                }
                double t_new = tc + h;
                if (t_new > t_end) {
                    t_new = t_end;
                    bdf_change_d(Dd, vstride, N, q, (t_end - tc) / h);
                    h = t_end - tc;
                    n_equal = 0;
                    lu_valid = false;
                }
                for (int s = tid; s < N; s += kThreads) {
                    double a = Dd[s];
                    for (int j = 1; j <= q; j++) a = a + Dd[(int64_t)j * vstride + s];
                    ypred[s] = a;
                    scale[s] = atolv[s] + rtol * fabs(a);
                    double p = 0.0;
                    for (int j = 1; j <= q; j++) p = p + gamma[j] * Dd[(int64_t)j * vstride + s];
                    psi[s] = p / gamma[q];
                }
                __syncthreads();
                const double c = h / gamma[q];
                bool converged = false;
                for (;;) {
                    if (!lu_valid) {
                        c_mark = clock64();
                        assemble_newton_matrix<LT>(m, xj, c, M, ld, true, fedv);
                        if (tid == 0) st.cycles_matrix += clock64() - c_mark;
                        c_mark = clock64();
                        int fail;
                        if constexpr (kMixed) {
                            if (fp64_lu) {
                                double *Md = reinterpret_cast<double *>(M);
                                assemble_newton_matrix<double>(m, xj, c, Md, ld, true, fedv);
                                fail = lu_factor<double>(Md, ld, N, perm,
                                                         reinterpret_cast<double *>(lt),
                                                         reinterpret_cast<double *>(utile),
                                                         reinterpret_cast<double *>(rowbuf), red,
                                                         ired, cyc);
                            } else {
                                fail = gje_factor(M, ld, N, perm, pos, lt, utile, dblk, rowbuf,
                                                  red, ired, cyc);
                            }
                        } else {
                            fail = lu_factor<LT>(M, ld, N, perm, lt, utile, rowbuf, red, ired, cyc);
                        }
                        if (tid == 0) {
                            st.cycles_lu += clock64() - c_mark;
                            st.lu_factorisations++;
                        }
                        lu_valid = fail == 0;
                    }
                    converged = false;
                    n_iter = 0;
                    if (lu_valid) {
                        // modified Newton from the prediction
                        for (int s = tid; s < N; s += kThreads) {
                            ynew[s] = ypred[s];
                            dv[s] = 0.0;
                        }
                        __syncthreads();
                        double dy_old = -1.0;
                        for (int it = 0; it < kBdfNewtonMaxIter; it++) {
                            rhs(ynew, f);
                            rhs_evals++;
                            int bad = 0;
                            for (int s = tid; s < N; s += kThreads) bad |= !isfinite(f[s]);
                            if (__syncthreads_or(bad)) break;
                            c_mark = clock64();
                            if (kMixed && !fp64_lu) {
                                // dy solves (I - cJ) dy = r in FP64 by
                                // refinement with the FP32 inverse X:
                                // dy += X res, res = r - (dy - c J dy) with
                                // the exact J at xj, matrix-free; each res
                                // is scaled by a power of two to unit max
                                // norm for the FP32 cast
                                long long rb = 0;
                                for (int s = tid; s < N; s += kThreads) {
                                    const double r = c * f[s] - psi[s] - dv[s];
                                    aux[s] = r;
                                    res[s] = r;
                                    dy[s] = 0.0;
                                    rb = max(rb, absbits_nonan(r));
                                }
                                double rmax = block_max(__longlong_as_double(rb), red);
                                const double r0max = rmax;
                                const int sweeps = P.refine_max > 0 ? P.refine_max : 8;
                                for (int sw = 0; sw < sweeps; sw++) {
                                    if (!(rmax > 0.0) || !isfinite(rmax)) break;
                                    const int e = ilogb(rmax);
                                    const double sc = ldexp(1.0, -e), isc = ldexp(1.0, e);
                                    for (int s = tid; s < N; s += kThreads)
                                        bvec[s] = (LT)(res[perm[s]] * sc);
                                    __syncthreads();
                                    gje_apply(reinterpret_cast<const float *>(M), ld, N, perm,
                                              reinterpret_cast<float *>(bvec),
                                              reinterpret_cast<float *>(lt), false);
                                    for (int s = tid; s < N; s += kThreads)
                                        dy[s] = dy[s] + (double)reinterpret_cast<const float *>(lt)[perm[s]] * isc;
                                    __syncthreads();
                                    if (tid == 0) st.refine_sweeps++;
                                    // res = r - (dy - c J dy)
                                    jv_phase1(m, xj, dy, qr, true);
                                    __syncthreads();
                                    long long nb = 0;
                                    for (int s = tid; s < N; s += kThreads) {
                                        const double jv = fedv[s] != 0.0 ? 0.0 : jv_species(m, s, qr);
                                        const double rr = aux[s] - (dy[s] - c * jv);
                                        res[s] = rr;
                                        nb = max(nb, absbits_nonan(rr));
                                    }
                                    const double nmax = block_max(__longlong_as_double(nb), red);
                                    const bool done = nmax <= r0max * 0x1p-50 || nmax > 0.5 * rmax;
                                    rmax = nmax;
                                    if (done) break;
                                }
                            } else {
                                // FP64 LU (the FP64 form, or the mixed form's
                                // fallback with res as the solve vector)
                                double *Md = reinterpret_cast<double *>(M);
                                double *bv = kMixed ? res : reinterpret_cast<double *>(bvec);
                                for (int s = tid; s < N; s += kThreads) {
                                    const int ps = perm[s];
                                    bv[s] = c * f[ps] - psi[ps] - dv[ps];
                                }
                                __syncthreads();
                                lu_solve<double>(Md, ld, N, perm, bv);
                                for (int s = tid; s < N; s += kThreads) dy[s] = bv[s];
                                __syncthreads();
                            }
                            if (tid == 0) {
                                st.cycles_solve += clock64() - c_mark;
                                st.newton_iters++;
                            }
                            n_iter = it + 1;
                            const double dyn = bdf_rms(dy, scale, N, red);
                            double rate = -1.0;
                            if (dy_old >= 0.0) rate = dyn / dy_old;
                            if (rate >= 0.0) {
                                double rp = 1.0;
                                for (int r = 0; r < kBdfNewtonMaxIter - it; r++) rp = rp * rate;
                                if (rate >= 1.0 || rp / (1.0 - rate) * dyn > newton_tol) break;
                            }
                            for (int s = tid; s < N; s += kThreads) {
                                ynew[s] = ynew[s] + dy[s];
                                dv[s] = dv[s] + dy[s];
                            }
                            __syncthreads();
                            if (dyn == 0.0 ||
                                (rate >= 0.0 && rate / (1.0 - rate) * dyn < newton_tol)) {
                                converged = true;
                                break;
                            }
                            dy_old = dyn;
                        }
                    }
                    if (converged || jac_current) break;
                    // a fresh Jacobian at the prediction
                    for (int s = tid; s < N; s += kThreads) xj[s] = ypred[s];
                    __syncthreads();
                    jac_evals++;
                    jac_current = true;
                    lu_valid = false;
                }
                if (!converged) {
                    if (tid == 0) st.lu_failures++;
                    if (kMixed && !fp64_lu) {
                        // the FP32 inverse may be what failed: the same step
                        // once more on FP64 factors before the step shrinks;
                        // after kBdfFallback such failures without an FP32
                        // success in between, a longer FP64 stretch
                        fp64_lu = true;
                        if (++fail_run >= kBdfFallback) {
                            fp64_left = 1 << 30;  // FP64 factors from here on
                            if (tid == 0) st.nan_reverts++;  // counts the switch
                        } else {
                            fp64_left = 1;
                        }
                        lu_valid = false;
                        continue;
                    }
                    bdf_change_d(Dd, vstride, N, q, 0.5);
                    h = h * 0.5;
                    n_equal = 0;
                    lu_valid = false;
                    continue;
                }
                const double safety = 0.9 * (double)(2 * kBdfNewtonMaxIter + 1) /
                                      (double)(2 * kBdfNewtonMaxIter + n_iter);
                for (int s = tid; s < N; s += kThreads) {
                    scale[s] = atolv[s] + rtol * fabs(ynew[s]);
                    aux[s] = econst[q] * dv[s];
                }
                __syncthreads();
                err_norm = bdf_rms(aux, scale, N, red);
                if (err_norm > 1.0) {
                    // Newton converged: the factors stay until the next
                    // refactoring (modified Newton with the previous c)
                    if (tid == 0) {
                        st.rkf_retries++;
                        // one thread forms the factor (FP64 pow), all read it
                        double f0 = safety * pow(err_norm, -1.0 / (double)(q + 1));
                        s_bcast[0] = bdf_quantize(fmax(kBdfMinFactor, f0));
                    }
                    __syncthreads();
                    const double fct = s_bcast[0];
                    bdf_change_d(Dd, vstride, N, q, fct);
                    h = h * fct;
                    n_equal = 0;
                    continue;
                }
                accepted = true;
                if (!fp64_lu) fail_run = 0;
                if (kMixed && fp64_lu && --fp64_left <= 0) {
                    fp64_lu = false;  // back to FP32 factors at the next factorisation
                    lu_valid = false;
                }
                if (tid == 0) st.be_steps++;
                n_equal++;
                tc = t_new;
                jac_current = false;
                for (int s = tid; s < N; s += kThreads) {
                    Dd[(int64_t)(q + 2) * vstride + s] = dv[s] - Dd[(int64_t)(q + 1) * vstride + s];
                    Dd[(int64_t)(q + 1) * vstride + s] = dv[s];
                    for (int i = q; i >= 0; i--)
                        Dd[(int64_t)i * vstride + s] =
                            Dd[(int64_t)i * vstride + s] + Dd[(int64_t)(i + 1) * vstride + s];
                }
                __syncthreads();
                // samples in (t_old, tc] from the step's degree-q interpolant
                while (isample < nt && tv[isample] <= tc) {
                    const double ts = tv[isample];
                    double pj[kBdfMaxOrder + 1];
                    double p = 1.0;
                    for (int j = 0; j < q; j++) {
                        p = p * ((ts - (tc - h * (double)j)) / (h * (double)(1 + j)));
                        pj[j] = p;
                    }
                    for (int c2 = tid; c2 < ncs; c2 += kThreads) {
                        const int s = cs ? cs[c2] : c2;
                        double a = Dd[s];
                        if (ts != tc)
                            for (int j = 1; j <= q; j++) a = a + Dd[(int64_t)j * vstride + s] * pj[j - 1];
                        out[(int64_t)isample * ncs + c2] = a;
                    }
                    isample++;
                }
                if (n_equal < q + 1) break;
                // order and step for the next step
                double e_m = INFINITY, e_p = INFINITY;
                if (q > 1) {
                    for (int s = tid; s < N; s += kThreads)
                        aux[s] = econst[q - 1] * Dd[(int64_t)q * vstride + s];
                    __syncthreads();
                    e_m = bdf_rms(aux, scale, N, red);
                }
                if (q < max_order) {
                    for (int s = tid; s < N; s += kThreads)
                        aux[s] = econst[q + 1] * Dd[(int64_t)(q + 2) * vstride + s];
                    __syncthreads();
                    e_p = bdf_rms(aux, scale, N, red);
                }
                // one thread forms the candidate factors (FP64 pow), all read
                // the choice
                if (tid == 0) {
                    const double en[3] = {e_m, err_norm, e_p};
                    double fq[3];
                    for (int i = 0; i < 3; i++) {
                        fq[i] = en[i] == 0.0 ? INFINITY
                                             : (isinf(en[i]) ? 0.0
                                                             : pow(en[i], -1.0 / (double)(q + i)));
                        fq[i] = bdf_quantize(fmin(kBdfMaxFactor, safety * fq[i]));
                    }
                    int best = 0;
                    for (int i = 1; i < 3; i++)
                        if (fq[i] > fq[best]) best = i;
                    s_bcast[0] = fq[best];
                    s_ibcast = best;
                }
                __syncthreads();
                const int best = s_ibcast;
                const double fbest = s_bcast[0];
                __syncthreads();
                q += best - 1;
                h = h * fbest;
                bdf_change_d(Dd, vstride, N, q, fbest);
                n_equal = 0;
                lu_valid = false;
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        st.outer_iters = attempts;
        st.cycles_total = clock64() - c_start;
        st.t_final = tc;
        st.dt_be_final = h;
        st.jac_evals = jac_evals;
        st.rhs_evals = rhs_evals;
        st.order_final = q;
        st.status = status;
        P.res[id] = st;
    }
    __syncthreads();
}
