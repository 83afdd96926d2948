// Single-instance engine for networks above kThreads species: the whole GPU
// integrates one instance.  Included by compat_engine.cu inside its
// namespace (uses its helpers).
//
// One cooperative launch, one CTA per SM.  CTA 0 (the leader) runs the same
// integrator as the batched engine (integrate<LT, true>) with its vectors in
// global memory; the dense linear algebra is spread over all CTAs through a
// fork-join on a control block in global memory: the leader publishes a
// task and bumps a generation counter, every CTA does its share, the
// workers count themselves done, the leader waits for the count.
//
// The Newton matrix M = I - h*J is inverted in place by blocked Gauss-Jordan
// elimination with partial pivoting (row pivots, kWPB-column panels): per
// panel, the pivot block D (rows p_j0.., columns J) is inverted by the leader,
// and all CTAs form PR = D^-1 * M[P_J, C] from the leader's copy of the pivot
// rows and apply
//     M[i, C] -= M[i, J] * PR[:, C]   (i not a pivot row, C not in J)
//     M[i, J]  = -M[i, J] * D^-1,   M[P_J, C] = PR,   M[P_J, J] = D^-1.
// The panels of one kWSP-column super-panel S restrict C to S's columns;
// the other columns then take the same step for all of S at once (rank
// kWSP, see the super-panel section below).
// The result X satisfies inv(M)[j][p_k] = X[p_j][k], so a solve is
//     x[j] = (X * r[p])[p_j]:   one dense matrix-vector product,
// where the LU's two triangular solves would be 2N/32 dependent block steps.
// Pivot rows of the last fresh factorisation are reused (no pivot search)
// while the pivot blocks stay invertible; the integrator's refinement checks
// every solve and asks for fresh pivots when one does not converge.
#pragma once

constexpr int kWPB = 32;   // Gauss-Jordan panel width
constexpr int kWT = 128;   // rank-update tile: kWT rows x kWT columns per CTA pass
// Super-panel: kWSP columns (kWSP / kWPB panels) are eliminated within
// their own columns first; the rest of the matrix then takes one rank-kWSP
// update instead of kWSP / kWPB rank-kWPB ones, so it is read and written
// once per kWSP columns.  One column tile wide.
constexpr int kWSP = 128;
static_assert(kWSP == kWT && kWSP % kWPB == 0, "a super-panel is one column tile");

enum WideTask : int { kTaskExit = 0, kTaskAssemble = 1, kTaskUpdate = 3,
                      kTaskMatvec = 4, kTaskRates = 5, kTaskRkf = 6, kTaskRkfFinal = 7,
                      kTaskSolve = 8, kTaskSolveUpdate = 9, kTaskJv = 10, kTaskResidual = 11,
                      kTaskNewtonRhs = 12, kTaskPivotLevel = 13, kTaskPanelS = 14,
                      kTaskUpdateS = 15 };

// Most CTAs of one wide launch (per-CTA partial results of the RKF45 error).
constexpr int kWideMaxGrid = 256;

// Control block (global memory), zeroed before the launch.
struct WideCtl {
    unsigned int gen;   // task generation, bumped by the leader
    unsigned int done;  // CTAs other than the leader done with the current task
    int abort;          // a wait ran out of time
    int task;
    int j0, pb;         // current panel
    int pad0, pad1;     // pivot level: candidates, source list; panel/update: super-panel start
    double h;           // step of the matrix being assembled (RKF45: the step)
    const double *x;    // state the Jacobian (or the RHS) is evaluated at
    Vecs vecs;          // the leader's current RKF45 vectors (and Newton aliases)
    int root_sqrt;      // RKF45 step factor: sqrt(sqrt()) instead of pow
    double sc, isc;     // refinement: residual scale and its inverse
    long long lost;     // refinement: bit-pattern bound of the FP32-lost residuals
};

// Workspace of the wide engine, carved from one allocation (WideLayout).
template <typename LT>
struct WideWs {
    WideCtl *ctl;
    double *vec;      // 10 FP64 N-vectors (the batched engine's shared-memory set)
    double *pw;       // [nnz_a] reactant powers
    double *qr;       // [R] per-reaction scratch
    LT *A;            // N x ld, row-major; after factorisation the in-place inverse
    int *piv;         // [N] pivot row of each column
    int *pos;         // [N] position of a row among the current panel's pivots, or -1
    int *used;        // [N] 1 once a row has been a pivot (fresh pivot search)
    LT *PN;           // [kWPB][N] scratch; its first 2N ints are the pivot candidate lists
    int *cand;        // [2][N] candidate rows of the pivot search (two lists, alternating)
    LT *Dinv;         // [kWPB][kWPB]
    LT *SNAP;         // [kWPB][kWSP] the panel's pivot rows in the super-panel's tile
    LT *AJS;          // [N][kWSP] super-panel columns before its panels
    LT *PRS;          // [kWSP][ld] DS^-1 * M[P_S, :] (DS: the super-panel's pivot block)
    LT *vin, *vout;   // [N] matrix-vector product input (gathered) and output
    int *flags;       // [0]: pivot order valid (set by the leader)
    long long *part;  // [2][kWideMaxGrid]: per-CTA RKF45 accept flag, min delta bits
    int N, ld;
    // this CTA's tensor-core state (rank updates on tcgen05 when tc_on)
    int tc_on;
    uint64_t *tc_bar;     // mbarrier (shared)
    uint32_t *tc_phase;   // its parity (shared)
    uint32_t tc_tmem;     // kTcN TMEM columns
};

struct WideLayout {
    int64_t ctl, vec, pw, qr, A, piv, pos, used, PN, Dinv, SNAP, AJS, PRS, vin, vout, flags, part,
        total;
    __host__ __device__ static int64_t al(int64_t v) { return (v + 255) & ~int64_t(255); }
    __host__ __device__ WideLayout(int N, int R, int nnz_a, int lt) {
        const int64_t ld = (N + 3) & ~3;
        int64_t o = 0;
        ctl = o;   o = al(o + 256);
        vec = o;   o = al(o + int64_t(10) * N * 8);
        pw = o;    o = al(o + int64_t(nnz_a > 0 ? nnz_a : 1) * 8);
        qr = o;    o = al(o + int64_t(R > 0 ? R : 1) * 8);
        A = o;     o = al(o + int64_t(N) * ld * lt);
        piv = o;   o = al(o + int64_t(N) * 4);
        pos = o;   o = al(o + int64_t(N) * 4);
        used = o;  o = al(o + int64_t(N) * 4);
        PN = o;    o = al(o + int64_t(kWPB) * N * lt);
        Dinv = o;  o = al(o + int64_t(kWPB) * kWPB * lt);
        SNAP = o;  o = al(o + int64_t(kWPB) * kWSP * lt);
        AJS = o;   o = al(o + int64_t(N) * kWSP * lt);
        PRS = o;   o = al(o + int64_t(kWSP) * ld * lt);
        vin = o;   o = al(o + int64_t(N) * lt);
        vout = o;  o = al(o + int64_t(N) * lt);
        flags = o; o = al(o + 16);
        part = o;  o = al(o + int64_t(2) * kWideMaxGrid * 8);
        total = o;
    }
};

template <typename LT>
__device__ WideWs<LT> wide_ws(unsigned char *base, int N, int R, int nnz_a) {
    const WideLayout L(N, R, nnz_a, (int)sizeof(LT));
    WideWs<LT> W;
    W.ctl = reinterpret_cast<WideCtl *>(base + L.ctl);
    W.vec = reinterpret_cast<double *>(base + L.vec);
    W.pw = reinterpret_cast<double *>(base + L.pw);
    W.qr = reinterpret_cast<double *>(base + L.qr);
    W.A = reinterpret_cast<LT *>(base + L.A);
    W.piv = reinterpret_cast<int *>(base + L.piv);
    W.pos = reinterpret_cast<int *>(base + L.pos);
    W.used = reinterpret_cast<int *>(base + L.used);
    W.PN = reinterpret_cast<LT *>(base + L.PN);
    W.cand = reinterpret_cast<int *>(base + L.PN);
    W.Dinv = reinterpret_cast<LT *>(base + L.Dinv);
    W.SNAP = reinterpret_cast<LT *>(base + L.SNAP);
    W.AJS = reinterpret_cast<LT *>(base + L.AJS);
    W.PRS = reinterpret_cast<LT *>(base + L.PRS);
    W.vin = reinterpret_cast<LT *>(base + L.vin);
    W.vout = reinterpret_cast<LT *>(base + L.vout);
    W.flags = reinterpret_cast<int *>(base + L.flags);
    W.part = reinterpret_cast<long long *>(base + L.part);
    W.N = N;
    W.ld = (N + 3) & ~3;
    W.tc_on = 0;
    W.tc_bar = nullptr;
    W.tc_phase = nullptr;
    W.tc_tmem = 0;
    return W;
}

// Pivot search: candidate rows one CTA chooses from at once (their panel
// values in shared memory), and the rows per group of a tournament level.
__host__ __device__ constexpr int tour_max(int lt) { return lt == 4 ? 1024 : 512; }
constexpr int kTourGroup = 128;
__host__ __device__ constexpr int64_t tour_smem_bytes(int lt) {
    return int64_t(tour_max(lt)) * (kWPB + 1) * lt + int64_t(tour_max(lt)) * 4 +
           int64_t(2) * kWarps * (lt + 4);
}

// Dynamic shared memory of the wide kernel: the rank-update tiles, the
// matrix-vector input or the pivot search's candidates, whichever is
// largest, plus the pivot-block inverse.
__host__ __device__ inline int64_t wide_smem_bytes(int N, int lt) {
    int64_t tiles = (int64_t(kWPB) * (kWT + 4) + int64_t(kWPB) * kWT) * lt;
    // tensor-core operands: two split-TF32 sets (staging overlaps the MMAs)
    if (lt == 4 && tiles < 2 * 4 * kWT * kWPB * 4) tiles = 2 * 4 * kWT * kWPB * 4;
    const int64_t vin = int64_t((N + 3) & ~3) * lt;
    int64_t big = tiles > vin ? tiles : vin;
    if (big < tour_smem_bytes(lt)) big = tour_smem_bytes(lt);
    const int64_t ds = int64_t(kWSP) * kWSP * lt + kWSP * 4;  // task_panel_s
    if (big < ds) big = ds;
    return big + int64_t(kWPB) * kWPB * lt;
}

// ---------------------------------------------------------------- sync

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_acquire_i(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// A wait on another CTA that sees no progress for this long gives up (tasks
// take milliseconds; the leader's longest serial phase, a fresh pivot
// search, tens of milliseconds).
constexpr uint64_t kWideStallNs = 60ull * 1000000000ull;

// Thread 0 waits until *p >= target; false if the control block's abort flag
// is set, the wait sees no progress for kWideStallNs, or the wall clock
// passes `limit` (the launch deadline, 0 = none); it then sets the abort flag.
__device__ bool wide_wait(const unsigned *p, unsigned target, WideCtl *ctl, uint64_t limit) {
    unsigned spins = 0;
    const uint64_t t0 = global_ns();
    while (ld_acquire(p) < target) {
        if ((++spins & 63) == 0) {
            if (ld_acquire_i(&ctl->abort)) return false;
            const uint64_t now = global_ns();
            if ((limit && now > limit) || now - t0 > kWideStallNs) {
                atomicExch(&ctl->abort, 1);
                return false;
            }
        }
        __nanosleep(32);
    }
    return true;
}

// *p += 1 with release semantics at GPU scope: the CTA's writes before the
// caller's last barrier are visible to whoever acquires the new value.
__device__ __forceinline__ void red_release_add1(unsigned *p) {
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(p) : "memory");
}

// ---------------------------------------------------------------- tasks

// Rows of M = I - h*J(x) (assemble_newton_matrix's entries and Jacobian
// semantics), one warp per row: the lanes clear the row, lane 0 writes the
// identity and the entries; mdiag[i] = the FP64 diagonal before the cast.
template <typename LT>
__device__ void task_assemble(const WideWs<LT> &W, const Net &m, const double *x, double h,
                              double *mdiag) {
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kWarps + (threadIdx.x >> 5), nw = gridDim.x * kWarps;
    const int N = W.N, ld = W.ld;
    for (int i = gw; i < N; i += nw) {
        LT *Ar = W.A + (int64_t)i * ld;
        for (int c = lane; c < ld; c += 32) Ar[c] = LT(0);
        __syncwarp();
        if (lane == 0) {
            Ar[i] = LT(1);
            double di = 1.0;
            const int e0 = m.sptr[i], e1 = m.sptr[i + 1];
            for (int e = e0; e < e1; e++) {
                const int y = ent_index(m.sent[e]);
                for (int q = m.rptr[y]; q < m.rptr[y + 1]; q++) {
                    const int g = ent_index(m.rent[q]);
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
                        for (int q2 = b2; q2 < en2; q2++)
                            if (ent_index(m.rent[q2]) == g) { a = ent_coef(m.rent[q2]); break; }
                        if (a < 1) continue;
                        double temp = 0.0;
                        if (a == 1) temp = temp + (double)s2 * m.kk[y2];
                        else temp = temp + (double)s2 * m.kk[y2] * (double)a * mypow(x[g], a - 1);
                        for (int q2 = b2; q2 < en2; q2++) {
                            const int o = ent_index(m.rent[q2]);
                            if (o != g) temp = temp * x[o];
                        }
                        J = J + temp;
                    }
                    const double v = ((i == g) ? 1.0 : 0.0) - h * J;
                    Ar[g] = (LT)v;
                    if (g == i) di = v;
                }
            }
            mdiag[i] = di;
        }
    }
}

// Leader: SNAP = M[P_J, C] for the columns C of the super-panel's tile, the
// panel's pivot rows before the panel's update (the update's CTAs form
// PR = D^-1 * SNAP from it; the CTAs that own pivot rows overwrite them).
template <typename LT>
__device__ void leader_snapshot(const WideWs<LT> &W, int j0, int pb, int s0) {
    const int ld = W.ld;
    for (int q = threadIdx.x; q < kWPB * kWSP; q += kThreads) {
        const int k = q / kWSP, c = s0 + (q - k * kWSP);
        W.SNAP[q] = (k < pb && c < ld) ? W.A[(int64_t)W.piv[j0 + k] * ld + c] : LT(0);
    }
    __syncthreads();
}

// Before the first panel of super-panel S updates a row tile, the tile's
// CTA keeps AJS = M[rows, S] (the super-panel's rank-kWSP update needs the
// columns of S as they were before S).
template <typename LT>
__device__ void snapshot_ajs(const WideWs<LT> &W, int r0, int s0, int rows = kWT) {
    const int N = W.N, ld = W.ld, sw = min(kWSP, N - s0);
    for (int q = threadIdx.x; q < rows * (kWSP / 4); q += kThreads) {
        const int r = q / (kWSP / 4), k4 = (q - r * (kWSP / 4)) * 4;
        if (r0 + r >= N) continue;
        const LT *src = W.A + (int64_t)(r0 + r) * ld + s0 + k4;
        LT v[4];
        if (k4 + 4 <= sw) {
            load4(src, v);
        } else {
#pragma unroll
            for (int b = 0; b < 4; b++) v[b] = (k4 + b < sw) ? src[b] : LT(0);
        }
        store4(W.AJS + (int64_t)(r0 + r) * kWSP + k4, v);
    }
}

// The panel's rank-kWPB update of the super-panel's column tile in tiles of
// kNarrowRows rows, on the FP32 (or FP64) pipes: the strip is N x 128, so
// 128-row tiles would keep only N / 128 CTAs busy.  Thread (ty, tx) owns
// rows 2*ty, 2*ty+1 and columns tx*4.. of a tile.  Columns in J start from 0
// and use D^-1 in place of PR; the panel's pivot rows take their new values
// (PR, D^-1) directly.
constexpr int kNarrowRows = 32;
template <typename LT>
__device__ void task_update_narrow(const WideWs<LT> &W, int j0, int pb, LT *smem, int s0) {
    static_assert(kNarrowRows == 2 * kWarps && kWT == 4 * 32, "2 rows x 4 columns a thread");
    LT *sAJ = smem;                       // [kWPB][kNarrowRows]: panel columns, K-major
    LT *sB = smem + kWPB * kNarrowRows;   // [kWPB][kWT]: [PR | D^-1] over the tile's columns
    LT *sD = sB + kWPB * kWT;             // [kWPB][kWPB]: D^-1
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int N = W.N, ld = W.ld;
    const int nrt = (N + kNarrowRows - 1) / kNarrowRows;
    if ((int)blockIdx.x < nrt) {
        // B = [PR | D^-1] with PR = D^-1 * SNAP, formed by every CTA with
        // tiles (the same products in the same order in each)
        for (int q = tid; q < kWPB * kWPB; q += kThreads) sD[q] = W.Dinv[q];
        __syncthreads();
        for (int q = tid; q < (kWPB / 4) * kWT; q += kThreads) {
            const int g = q / kWT, cc = q - g * kWT, c = s0 + cc;
            const bool inJ = c >= j0 && c < j0 + kWPB;
            LT a[kWPB];
#pragma unroll
            for (int k = 0; k < kWPB; k++) a[k] = W.SNAP[k * kWSP + cc];
#pragma unroll
            for (int rr = 0; rr < 4; rr++) {
                const int r = g * 4 + rr;
                LT v = LT(0);
                if (r < pb && c < ld) {
                    if (inJ) {
                        v = (c - j0 < pb) ? sD[r * kWPB + (c - j0)] : LT(0);
                    } else {
#pragma unroll
                        for (int k = 0; k < kWPB; k++) v = lt_fma(sD[r * kWPB + k], a[k], v);
                    }
                }
                sB[r * kWT + cc] = v;
            }
        }
    }
    for (int t = blockIdx.x; t < nrt; t += gridDim.x) {
        const int r0 = t * kNarrowRows, c0 = s0;
        __syncthreads();
        if (j0 == s0) snapshot_ajs<LT>(W, r0, s0, kNarrowRows);
        // the panel columns of this tile's rows (only this CTA writes them)
        for (int q = tid; q < kNarrowRows * kWPB; q += kThreads) {
            const int r = q / kWPB, k = q - r * kWPB;
            sAJ[k * kNarrowRows + r] =
                (r0 + r < N && k < pb) ? W.A[(int64_t)(r0 + r) * ld + j0 + k] : LT(0);
        }
        __syncthreads();
        const int col = c0 + tx * 4;
        if (col >= ld) continue;
        const bool inJ = col >= j0 && col < j0 + kWPB;
        const int rl0 = ty * 2;
        LT acc[2][4];
#pragma unroll
        for (int a = 0; a < 2; a++) {
            const int row = r0 + rl0 + a;
            if (row < N && !inJ) {
                load4(W.A + (int64_t)row * ld + col, acc[a]);
            } else {
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = LT(0);
            }
        }
#pragma unroll 8
        for (int k = 0; k < kWPB; k++) {
            LT bv[4];
            load4(sB + k * kWT + tx * 4, bv);
            const LT a0 = sAJ[k * kNarrowRows + rl0], a1 = sAJ[k * kNarrowRows + rl0 + 1];
#pragma unroll
            for (int b = 0; b < 4; b++) {
                acc[0][b] = lt_fma(-a0, bv[b], acc[0][b]);
                acc[1][b] = lt_fma(-a1, bv[b], acc[1][b]);
            }
        }
#pragma unroll
        for (int a = 0; a < 2; a++) {
            const int row = r0 + rl0 + a;
            if (row >= N) break;
            const int pr = W.pos[row];
            if (pr >= 0) load4(sB + pr * kWT + tx * 4, acc[a]);
            store4(W.A + (int64_t)row * ld + col, acc[a]);
        }
    }
}

// ---------------------------------------------------------------- super-panel
//
// After the panels of super-panel S (columns s0 .. s0+sw-1, pivot rows P_S)
// have been eliminated within S's column tile, the columns of S hold the
// in-place inverse of its block, X[P_S[r]][s0 + k] = DS^-1[r][k] with
// DS[k][r] = M[P_S[k]][s0 + r] before S; every other column C then takes
//     PRS = DS^-1 * M[P_S, C],   M[i, C] -= AJS[i, :] * PRS   (i not in P_S),
//     M[P_S, C] = PRS,
// the same matrix the panels' rank-kWPB updates would give, in one pass.

// PRS over the columns outside S's tile (rows >= sw zero): DS^-1 and P_S
// staged in shared memory, by (group of 8 rows, column) over the grid.
template <typename LT>
__device__ void task_panel_s(const WideWs<LT> &W, int s0, int sw, LT *smem) {
    constexpr int RG = 8, KC = 16;
    LT *sDS = smem;                                               // [kWSP][kWSP]
    int *spiv = reinterpret_cast<int *>(sDS + kWSP * kWSP);       // [kWSP]
    const int tid = threadIdx.x, N = W.N, ld = W.ld;
    (void)N;
    for (int q = tid; q < kWSP; q += kThreads) spiv[q] = q < sw ? W.piv[s0 + q] : 0;
    __syncthreads();
    for (int q = tid; q < kWSP * kWSP; q += kThreads) {
        const int r = q / kWSP, k = q - r * kWSP;
        sDS[q] = (r < sw && k < sw) ? W.A[(int64_t)spiv[r] * ld + s0 + k] : LT(0);
    }
    __syncthreads();
    const int tw = min(s0 + kWSP, ld) - s0, cw = ld - tw;  // columns outside the tile
    const int gt = blockIdx.x * kThreads + tid, nt = gridDim.x * kThreads;
    for (int q = gt; q < (kWSP / RG) * cw; q += nt) {
        const int g = q / cw, cc = q - g * cw;
        const int c = cc < s0 ? cc : cc + tw;
        LT acc[RG];
#pragma unroll
        for (int r = 0; r < RG; r++) acc[r] = LT(0);
        if (g * RG < sw) {
            for (int k0 = 0; k0 < sw; k0 += KC) {
                LT b[KC];
#pragma unroll
                for (int k = 0; k < KC; k++)
                    b[k] = (k0 + k < sw) ? W.A[(int64_t)spiv[k0 + k] * ld + c] : LT(0);
#pragma unroll
                for (int r = 0; r < RG; r++)
#pragma unroll
                    for (int k = 0; k < KC; k++)
                        acc[r] = lt_fma(sDS[(g * RG + r) * kWSP + k0 + k], b[k], acc[r]);
            }
        }
#pragma unroll
        for (int r = 0; r < RG; r++) W.PRS[(int64_t)(g * RG + r) * ld + c] = acc[r];
    }
}

// The rank-kWSP update of every column tile but S's, on the FP32 (or FP64)
// pipes: 128 x 128 tiles, thread (ty, tx) owning rows ty*8.. and columns
// tx*4.., K in chunks of kWPB staged in shared memory.
template <typename LT>
__device__ void task_update_s(const WideWs<LT> &W, int s0, int sw, LT *smem) {
    constexpr int AS = kWT + 4;
    LT *sAJ = smem;                       // [kWPB][AS]
    LT *sB = smem + kWPB * AS;            // [kWPB][kWT]
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int N = W.N, ld = W.ld;
    const int nrt = (N + kWT - 1) / kWT, nct = (ld + kWT - 1) / kWT, st = s0 / kWT;
    if (nct < 2) return;
    for (int t = blockIdx.x; t < nrt * (nct - 1); t += gridDim.x) {
        const int ct = t % (nct - 1);
        const int r0 = (t / (nct - 1)) * kWT, c0 = (ct < st ? ct : ct + 1) * kWT;
        const int col = c0 + tx * 4, rl0 = ty * 8;
        const bool live = col < ld;
        LT acc[8][4];
#pragma unroll
        for (int a = 0; a < 8; a++) {
            const int row = r0 + rl0 + a;
            if (live && row < N && W.pos[row] < 0) {
                load4(W.A + (int64_t)row * ld + col, acc[a]);
            } else {
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = LT(0);
            }
        }
        for (int k0 = 0; k0 < sw; k0 += kWPB) {
            __syncthreads();
            for (int q = tid; q < kWT * kWPB; q += kThreads) {
                const int r = q / kWPB, k = q - r * kWPB;
                sAJ[k * AS + r] = (r0 + r < N) ? W.AJS[(int64_t)(r0 + r) * kWSP + k0 + k] : LT(0);
            }
            for (int q = tid; q < kWPB * kWT; q += kThreads) {
                const int k = q / kWT, cc = q - k * kWT;
                const int c = c0 + cc;
                sB[q] = (c < ld) ? W.PRS[(int64_t)(k0 + k) * ld + c] : LT(0);
            }
            __syncthreads();
#pragma unroll 4
            for (int k = 0; k < kWPB; k++) {
                LT av[8], bv[4];
                load8(sAJ + k * AS + rl0, av);
                load4(sB + k * kWT + tx * 4, bv);
#pragma unroll
                for (int a = 0; a < 8; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) acc[a][b] = lt_fma(-av[a], bv[b], acc[a][b]);
            }
        }
        if (!live) continue;
#pragma unroll
        for (int a = 0; a < 8; a++) {
            const int row = r0 + rl0 + a;
            if (row >= N) break;
            const int pr = W.pos[row];
            if (pr >= 0) load4(W.PRS + (int64_t)pr * ld + col, acc[a]);
            store4(W.A + (int64_t)row * ld + col, acc[a]);
        }
    }
}

// task_update_s on the tensor cores: per 128 x 128 tile, K chunks of kTcK
// with A = AJS rows and B = PRS columns split into TF32 high and low parts
// (W.tc_on == 2: rounded to BF16) in the canonical K-major layout,
// accumulated in tensor memory, read back once; each thread finishes 32
// entries of its row (pivot rows of S take PRS, the rest subtract).  False
// if a tensor-core wait ran out (the control block's abort flag is then
// set).
__device__ bool task_update_s_tc(const WideWs<float> &W, int s0, int sw, float *smem) {
    // two operand buffers: chunk k+1 is staged while the MMAs of chunk k run
    constexpr int kSet = 2 * kTcM * kTcK + 2 * kTcN * kTcK;  // floats of one split set
    const bool bf16 = W.tc_on == 2;
    const int tid = threadIdx.x;
    const int N = W.N, ld = W.ld;
    const int nrt = (N + kTcM - 1) / kTcM, nct = (ld + kTcN - 1) / kTcN, st = s0 / kTcN;
    uint32_t phase = *W.tc_phase;
    bool ok = true;
    for (int t = blockIdx.x; nct > 1 && t < nrt * (nct - 1) && ok; t += gridDim.x) {
        const int ct = t % (nct - 1);
        const int r0 = (t / (nct - 1)) * kTcM, c0 = (ct < st ? ct : ct + 1) * kTcN;
        // chunk k0 of A = AJS rows and B = PRS columns into buffer set `b`
        auto stage = [&](int k0, int b) {
            float *base = smem + b * kSet;
            if (bf16) {
                uint16_t *sA16 = reinterpret_cast<uint16_t *>(base), *sB16 = sA16 + kTcM * kTcK;
                for (int q = tid; q < kTcM * (kTcK / 4); q += kThreads) {
                    const int r = q >> 3, k4 = (q & 7) * 4;
                    float v[4] = {0.f, 0.f, 0.f, 0.f};
                    if (r0 + r < N) load4(W.AJS + (int64_t)(r0 + r) * kWSP + k0 + k4, v);
                    uint2 pk;
                    pk.x = (uint32_t)bf16_bits(v[0]) | ((uint32_t)bf16_bits(v[1]) << 16);
                    pk.y = (uint32_t)bf16_bits(v[2]) | ((uint32_t)bf16_bits(v[3]) << 16);
                    *reinterpret_cast<uint2 *>(sA16 + tc_off16(r, k4) / 2) = pk;
                }
                for (int q = tid; q < kTcN * (kTcK / 4); q += kThreads) {
                    const int n = q & (kTcN - 1), k4 = (q / kTcN) * 4;
                    const int c = c0 + n;
                    uint16_t h[4];
#pragma unroll
                    for (int e = 0; e < 4; e++)
                        h[e] = bf16_bits(c < ld ? W.PRS[(int64_t)(k0 + k4 + e) * ld + c] : 0.f);
                    uint2 pk;
                    pk.x = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
                    pk.y = (uint32_t)h[2] | ((uint32_t)h[3] << 16);
                    *reinterpret_cast<uint2 *>(sB16 + tc_off16(n, k4) / 2) = pk;
                }
            } else {
                float *sAh = base, *sAl = sAh + kTcM * kTcK, *sBh = sAl + kTcM * kTcK,
                      *sBl = sBh + kTcN * kTcK;
                for (int q = tid; q < kTcM * (kTcK / 4); q += kThreads) {
                    const int r = q >> 3, k4 = (q & 7) * 4;
                    float v[4] = {0.f, 0.f, 0.f, 0.f};
                    if (r0 + r < N) load4(W.AJS + (int64_t)(r0 + r) * kWSP + k0 + k4, v);
                    float h[4], l[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        h[e] = tf32_hi(v[e]);
                        l[e] = v[e] - h[e];
                    }
                    const int o = tc_off(r, k4) / 4;
                    store4(sAh + o, h);
                    store4(sAl + o, l);
                }
                for (int q = tid; q < kTcN * (kTcK / 4); q += kThreads) {
                    const int n = q & (kTcN - 1), k4 = (q / kTcN) * 4;
                    const int c = c0 + n;
                    float h[4], l[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const float x = c < ld ? W.PRS[(int64_t)(k0 + k4 + e) * ld + c] : 0.f;
                        h[e] = tf32_hi(x);
                        l[e] = x - h[e];
                    }
                    const int o = tc_off(n, k4) / 4;
                    store4(sBh + o, h);
                    store4(sBl + o, l);
                }
            }
            tc_proxy_fence();
            __syncthreads();
        };
        auto issue = [&](int b, bool acc) {
            float *base = smem + b * kSet;
            if (bf16) {
                const uint16_t *sA16 = reinterpret_cast<const uint16_t *>(base);
                tc_chunk_issue_bf16(sA16, sA16 + kTcM * kTcK, W.tc_bar, W.tc_tmem, acc);
            } else {
                tc_chunk_issue(base, base + kTcM * kTcK, base + 2 * kTcM * kTcK,
                               base + 2 * kTcM * kTcK + kTcN * kTcK, W.tc_bar, W.tc_tmem, acc);
            }
        };
        stage(0, 0);
        issue(0, false);
        int kc = 1;
        for (int k0 = kTcK; k0 < sw && ok; k0 += kTcK, kc++) {
            stage(k0, kc & 1);                     // while chunk kc-1 multiplies
            ok = tc_chunk_wait(W.tc_bar, phase);  // chunk kc-1 done: its buffer is free
            if (ok) issue(kc & 1, true);
        }
        if (ok) ok = tc_chunk_wait(W.tc_bar, phase);
        if (!ok) break;
        float out[32];
        tc_tile_read(W.tc_tmem, out);
        const int w = tid >> 5;
        const int row = r0 + (w & 3) * 32 + (tid & 31), cb = c0 + (w >> 2) * 32;
        if (row < N && cb < ld) {
            const int pr = W.pos[row];
            float *dst = W.A + (int64_t)row * ld;
#pragma unroll
            for (int g = 0; g < 8; g++) {
                const int c = cb + 4 * g;
                if (c >= ld) break;
                float v[4];
                if (pr >= 0) {
                    load4(W.PRS + (int64_t)pr * ld + c, v);
                } else {
                    load4(dst + c, v);
#pragma unroll
                    for (int b = 0; b < 4; b++) v[b] -= out[4 * g + b];
                }
                store4(dst + c, v);
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        *W.tc_phase = phase;
        if (!ok) atomicExch(&W.ctl->abort, 1);
    }
    __syncthreads();
    return ok;
}

// vout = A * vin, one warp per row, vin staged in shared memory.
template <typename LT>
__device__ void task_matvec(const WideWs<LT> &W, LT *svin) {
    const int tid = threadIdx.x, lane = tid & 31;
    const int N = W.N, ld = W.ld;
    for (int c = tid; c < ld; c += kThreads) svin[c] = (c < N) ? W.vin[c] : LT(0);
    __syncthreads();
    const int gw = blockIdx.x * kWarps + (tid >> 5), nw = gridDim.x * kWarps;
    for (int i = gw; i < N; i += nw) {
        const LT *Ar = W.A + (int64_t)i * ld;
        LT acc = LT(0);
        for (int c = lane * 4; c < ld; c += 128) {
            LT a[4];
            load4(Ar + c, a);
#pragma unroll
            for (int b = 0; b < 4; b++) acc = lt_fma(a[b], svin[c + b], acc);
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) W.vout[i] = acc;
    }
}

// RKF45 tasks: the stages of an attempt with every species and reaction
// spread over the whole grid (rkf_stage, rkf_final: the batched engine's
// arithmetic).
__device__ void task_rates(const Net &m, const double *x, double *pw, double *rate) {
    const int gt = blockIdx.x * kThreads + threadIdx.x, nt = gridDim.x * kThreads;
    for (int y = gt; y < m.r; y += nt) {
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

__device__ void task_rkf(const Net &m, const Vecs &V, int stg, double dt, const double *pw,
                         const double *rate) {
    const int gt = blockIdx.x * kThreads + threadIdx.x, nt = gridDim.x * kThreads;
    for (int s = gt; s < m.n; s += nt) rkf_stage(stg, V, s, rhs_species_r(m, s, pw, rate), dt);
}

// Last stage; this CTA's accept flag and min delta (bit pattern, NaN as +inf)
// go to part[blockIdx.x] and part[kWideMaxGrid + blockIdx.x].  Returns
// whether species 0's delta is NaN (meaningful in the CTA that owns it).
__device__ bool task_rkf_final(long long *part, const Net &m, const Vecs &V, double dt,
                               bool root_sqrt, const double *pw, const double *rate,
                               double *red) {
    const int gt = blockIdx.x * kThreads + threadIdx.x, nt = gridDim.x * kThreads;
    bool ok = true, d0nan = false;
    double dloc = INFINITY;
    for (int s = gt; s < m.n; s += nt)
        rkf_final(V, s, rhs_species_r(m, s, pw, rate), dt, root_sqrt, ok, dloc, d0nan);
    const int all = __syncthreads_and(ok);
    const int dn = __syncthreads_or(d0nan);
    const double dmin = block_min_nonnan(dloc, red);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = all;
        part[kWideMaxGrid + blockIdx.x] = __double_as_longlong(dmin);
    }
    return dn != 0;
}

// Refinement tasks (mixed form; the Newton vectors are the leader's aliases:
// res = k6, dx = k4, xr = k3, xf = k5, mdiag = k1).
// Solve: vout = X * (res[piv] * sc), the scaled residual staged per CTA.
template <typename LT>
__device__ void task_solve(const WideWs<LT> &W, const double *res, double sc, LT *svin) {
    const int tid = threadIdx.x, lane = tid & 31;
    const int N = W.N, ld = W.ld;
    for (int c = tid; c < ld; c += kThreads) svin[c] = (c < N) ? (LT)(res[W.piv[c]] * sc) : LT(0);
    __syncthreads();
    const int gw = blockIdx.x * kWarps + (tid >> 5), nw = gridDim.x * kWarps;
    for (int i = gw; i < N; i += nw) {
        const LT *Ar = W.A + (int64_t)i * ld;
        LT acc = LT(0);
        for (int c = lane * 4; c < ld; c += 128) {
            LT a[4];
            load4(Ar + c, a);
#pragma unroll
            for (int b = 0; b < 4; b++) acc = lt_fma(a[b], svin[c + b], acc);
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) W.vout[i] = acc;
    }
}

// Update: dx += x * isc (x[s] = vout[piv[s]]) plus the FP64 diagonal part of
// residuals below the FP32 range; this CTA's max |correction| and max |dx|
// (bit patterns, NaN ignored) go to part[g] and part[kWideMaxGrid + g].
template <typename LT>
__device__ void task_solve_update(const WideWs<LT> &W, const Vecs &V, double sc, double isc,
                                  long long lost, double *red) {
    const int gt = blockIdx.x * kThreads + threadIdx.x, nt = gridDim.x * kThreads;
    const double *res = V.k6, *mdiag = V.k1;
    double *dx = V.k4;
    long long cmb = 0, xmb = 0;
    for (int s = gt; s < W.N; s += nt) {
        double c = (double)W.vout[W.piv[s]] * isc;
        if ((__double_as_longlong(res[s]) & 0x7fffffffffffffffLL) < lost) {
            const double rs = res[s] * sc;
            if (fabs(mdiag[s]) >= 0.5) c += (rs - (double)(float)rs) * isc / mdiag[s];
        }
        const double nx = dx[s] + c;
        dx[s] = nx;
        cmb = max(cmb, absbits_nonan(c));
        xmb = max(xmb, absbits_nonan(nx));
    }
    double cm = __longlong_as_double(cmb), xm = __longlong_as_double(xmb);
    block_max2(cm, xm, red);
    if (threadIdx.x == 0) {
        W.part[blockIdx.x] = __double_as_longlong(cm);
        W.part[kWideMaxGrid + blockIdx.x] = __double_as_longlong(xm);
    }
}

// Newton residual of the backward-Euler step (kernels.cuh:289-300):
// xr = -(yv - y1 - dt * f(yv)), and xf = yv at the first iteration
// (yv = k2, xr = k3, xf = k5); the rates of yv are in pw/rate.
__device__ void task_newton_rhs(const Net &m, const Vecs &V, double dt, bool first,
                                const double *pw, const double *rate) {
    const int gt = blockIdx.x * kThreads + threadIdx.x, nt = gridDim.x * kThreads;
    for (int s = gt; s < m.n; s += nt) {
        const double f = rhs_species_r(m, s, pw, rate);
        V.k3[s] = -(V.k2[s] - V.y1[s] - dt * f);
        if (first) V.k5[s] = V.k2[s];
    }
}

__device__ void task_jv(const Net &m, const double *x, const double *v, double *qr) {
    const int gt = blockIdx.x * kThreads + threadIdx.x, nt = gridDim.x * kThreads;
    for (int y = gt; y < m.r; y += nt) qr[y] = jv_reaction(m, x, v, y);
}

// res = xr - (dx - dt * J v); this CTA's max |res| (NaN ignored) to part[g].
__device__ void task_residual(long long *part, const Net &m, const Vecs &V, double dt,
                              const double *qr, double *red) {
    const int gt = blockIdx.x * kThreads + threadIdx.x, nt = gridDim.x * kThreads;
    const double *xr = V.k3, *dx = V.k4;
    double *res = V.k6;
    long long rlb = 0;
    for (int s = gt; s < m.n; s += nt) {
        const double jv = jv_species(m, s, qr);
        const double r = xr[s] - (dx[s] - dt * jv);
        res[s] = r;
        rlb = max(rlb, absbits_nonan(r));
    }
    const double rm = block_max(__longlong_as_double(rlb), red);
    if (threadIdx.x == 0) part[blockIdx.x] = __double_as_longlong(rm);
}

// ---------------------------------------------------------------- pivot search
//
// Partial pivoting chooses each panel column's pivot among all rows not yet
// used, which makes a leader-only pass over the whole panel per column.
// With more candidates than one CTA holds in shared memory (tour_max), the
// search is a tournament: every CTA runs partial pivoting on groups of
// kTourGroup candidates and keeps each group's chosen rows, until the
// survivors fit the leader, which runs partial pivoting on their panel rows.
// The chosen rows of a group span the group's panel rows, so the survivors
// keep the panel's rank; with at most tour_max candidates the choice is
// plain partial pivoting.

// Ordered compaction by the whole CTA: writes the kept entries of 0..n-1 to
// out in order -- with in == nullptr row i where used[i] == 0, otherwise
// in[i] where in[i] >= 0 -- and returns their count (uniform).
__device__ int cta_compact(const int *in, const int *used, int n, int *out) {
    __shared__ int sscan[kWarps];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int chunk = (n + kThreads - 1) / kThreads;
    const int b = min(n, tid * chunk), e = min(n, b + chunk);
    auto keep = [&](int i) { return in ? in[i] >= 0 : used[i] == 0; };
    int cnt = 0;
    for (int i = b; i < e; i++) cnt += keep(i) ? 1 : 0;
    int x = cnt;  // inclusive scan over the warp
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sscan[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < kWarps ? sscan[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kWarps) sscan[lane] = w;
    }
    __syncthreads();
    int off = x - cnt + (warp > 0 ? sscan[warp - 1] : 0);
    for (int i = b; i < e; i++)
        if (keep(i)) out[off++] = in ? in[i] : i;
    const int total = sscan[kWarps - 1];
    __syncthreads();
    return total;
}

// Partial pivoting restricted to the C candidate rows rows[0..C)
// (C <= tour_max): their values in the panel columns j0 .. j0+pb-1 are
// staged in shared memory; per column the candidate not chosen yet with the
// largest |value| (ties to the earlier candidate, NaN never wins) becomes
// the next pivot and the column is eliminated from the others.  sel[k]
// (shared) = the k-th chosen row; returns how many were chosen (uniform),
// fewer than pb only when a column has no nonzero candidate left.
template <typename LT>
__device__ int cta_select(const WideWs<LT> &W, const int *rows, int C, int j0, int pb,
                          unsigned char *smem, int *sel) {
    static_assert(kWPB == 32 && kThreads * 2 >= 1024, "one panel row per 32 lanes, 2 rows a thread");
    constexpr int SP = kWPB + 1;  // row stride: lanes on consecutive rows hit distinct banks
    constexpr int RPT = 2;        // candidates per thread
    const int tmax = tour_max((int)sizeof(LT));
    LT *sp = reinterpret_cast<LT *>(smem);
    int *srow = reinterpret_cast<int *>(sp + (int64_t)tmax * SP);
    LT *sv = reinterpret_cast<LT *>(srow + tmax);
    int *si = reinterpret_cast<int *>(sv + 2 * kWarps);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ld = W.ld;
    for (int q = tid; q < C * kWPB; q += kThreads) {
        const int r = q >> 5, c = q & 31;
        const int row = rows[r];
        if (c == 0) srow[r] = row;
        sp[r * SP + c] = c < pb ? W.A[(int64_t)row * ld + j0 + c] : LT(0);
    }
    __syncthreads();
    bool alive[RPT];
#pragma unroll
    for (int i = 0; i < RPT; i++) alive[i] = tid + i * kThreads < C;
    int n = 0;
    for (int k = 0; k < pb; k++) {
        PivT<LT> best{LT(-1), 1 << 30};
#pragma unroll
        for (int i = 0; i < RPT; i++) {
            const int r = tid + i * kThreads;
            if (!alive[i]) continue;
            const LT v = fabs(sp[r * SP + k]);
            if (!isnan(v)) best = piv_better(best, PivT<LT>{v, r});
        }
        for (int o = 16; o > 0; o >>= 1) {
            PivT<LT> other{__shfl_xor_sync(0xffffffffu, best.v, o),
                           __shfl_xor_sync(0xffffffffu, best.i, o)};
            best = piv_better(best, other);
        }
        // per-warp results in alternating slots: one barrier per column
        const int b = (k & 1) * kWarps;
        if (lane == 0) {
            sv[b + warp] = best.v;
            si[b + warp] = best.i;
        }
        __syncthreads();
        PivT<LT> all{LT(-1), 1 << 30};
        if (lane < kWarps) all = PivT<LT>{sv[b + lane], si[b + lane]};
        for (int o = kWarps / 2; o > 0; o >>= 1) {
            PivT<LT> other{__shfl_xor_sync(0xffffffffu, all.v, o),
                           __shfl_xor_sync(0xffffffffu, all.i, o)};
            all = piv_better(all, other);
        }
        const int p = __shfl_sync(0xffffffffu, all.i, 0);
        const LT pv = __shfl_sync(0xffffffffu, all.v, 0);
        if (p >= C || !(pv > LT(0))) break;  // uniform
        if (tid == 0) sel[k] = srow[p];
        n = k + 1;
        // the pivot row was last written before this column's barrier
        const LT rd = LT(1) / sp[p * SP + k];
#pragma unroll
        for (int i = 0; i < RPT; i++) {
            const int r = tid + i * kThreads;
            if (!alive[i]) continue;
            if (r == p) {
                alive[i] = false;
                continue;
            }
            const LT l = sp[r * SP + k] * rd;
            for (int c = k + 1; c < pb; c++)
                sp[r * SP + c] = lt_fma(-l, sp[p * SP + c], sp[r * SP + c]);
        }
    }
    __syncthreads();
    return n;
}

// One tournament level: the C candidates of list `src` in groups of
// kTourGroup, each group's chosen rows (kWPB slots, -1 for none) into the
// other list at 32 * group.
template <typename LT>
__device__ void task_pivot_level(const WideWs<LT> &W, int j0, int pb, int C, int src,
                                 unsigned char *smem) {
    __shared__ int sel[kWPB];
    const int *in = W.cand + (int64_t)src * W.N;
    int *out = W.cand + (int64_t)(src ^ 1) * W.N;
    const int ng = (C + kTourGroup - 1) / kTourGroup;
    for (int g = blockIdx.x; g < ng; g += gridDim.x) {
        const int c = min(kTourGroup, C - g * kTourGroup);
        const int n = cta_select<LT>(W, in + (int64_t)g * kTourGroup, c, j0, pb, smem, sel);
        if (threadIdx.x < kWPB) out[g * kWPB + threadIdx.x] = (int)threadIdx.x < n ? sel[threadIdx.x] : -1;
        __syncthreads();
    }
}

// Worker CTA: serve tasks until the leader sends kTaskExit (or a wait runs
// out of time).
template <typename LT>
__device__ void wide_worker(const WideWs<LT> &W, const Net &m, double *mdiag, unsigned char *smem,
                            uint64_t limit) {
    __shared__ int s_task, s_j0, s_pb, s_ok;
    __shared__ double s_h;
    __shared__ const double *s_x;
    LT *sm = reinterpret_cast<LT *>(smem);
    unsigned gen = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            s_ok = wide_wait(&W.ctl->gen, gen + 1, W.ctl, limit);
            if (s_ok) {
                s_task = W.ctl->task;
                s_j0 = W.ctl->j0;
                s_pb = W.ctl->pb;
                s_h = W.ctl->h;
                s_x = W.ctl->x;
            }
        }
        __syncthreads();
        if (!s_ok || s_task == kTaskExit) return;
        gen++;
        switch (s_task) {
        case kTaskAssemble: task_assemble<LT>(W, m, s_x, s_h, mdiag); break;
        case kTaskUpdate: task_update_narrow<LT>(W, s_j0, s_pb, sm, W.ctl->pad0); break;
        case kTaskPanelS: task_panel_s<LT>(W, s_j0, s_pb, sm); break;
        case kTaskUpdateS:
            if constexpr (std::is_same<LT, float>::value) {
                if (W.tc_on) {
                    task_update_s_tc(W, s_j0, s_pb, sm);
                    break;
                }
            }
            task_update_s<LT>(W, s_j0, s_pb, sm);
            break;
        case kTaskMatvec: task_matvec<LT>(W, sm); break;
        case kTaskPivotLevel:
            task_pivot_level<LT>(W, s_j0, s_pb, W.ctl->pad0, W.ctl->pad1, smem);
            break;
        case kTaskRates: task_rates(m, s_x, W.pw, W.qr); break;
        case kTaskSolve: {
            const Vecs v = W.ctl->vecs;
            task_solve<LT>(W, v.k6, W.ctl->sc, sm);
            break;
        }
        case kTaskSolveUpdate: {
            const Vecs v = W.ctl->vecs;
            task_solve_update<LT>(W, v, W.ctl->sc, W.ctl->isc, W.ctl->lost,
                                  reinterpret_cast<double *>(sm));
            break;
        }
        case kTaskJv: {
            const Vecs v = W.ctl->vecs;
            task_jv(m, v.k5, v.k4, W.qr);
            break;
        }
        case kTaskResidual: {
            const Vecs v = W.ctl->vecs;
            task_residual(W.part, m, v, s_h, W.qr, reinterpret_cast<double *>(sm));
            break;
        }
        case kTaskNewtonRhs: {
            const Vecs v = W.ctl->vecs;
            task_newton_rhs(m, v, s_h, s_j0 != 0, W.pw, W.qr);
            break;
        }
        case kTaskRkf: {
            const Vecs v = W.ctl->vecs;
            task_rkf(m, v, s_j0, s_h, W.pw, W.qr);
            break;
        }
        case kTaskRkfFinal: {
            const Vecs v = W.ctl->vecs;
            task_rkf_final(W.part, m, v, s_h, W.ctl->root_sqrt != 0, W.pw, W.qr,
                           reinterpret_cast<double *>(sm));
            break;
        }
        default: break;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            red_release_add1(&W.ctl->done);
        }
    }
}

// Leader: publish a task (the leader then does its own share).
template <typename LT>
__device__ void wide_fork(const WideWs<LT> &W, int task, int j0, int pb, double h,
                          const double *x) {
    __syncthreads();
    if (threadIdx.x == 0) {
        WideCtl *c = W.ctl;
        c->task = task;
        c->j0 = j0;
        c->pb = pb;
        c->h = h;
        c->x = x;
        c->done = 0;
        red_release_add1(&c->gen);
    }
}

// Leader: wait for the other CTAs; false if a wait ran out of time.
template <typename LT>
__device__ bool wide_join(const WideWs<LT> &W, uint64_t limit, int *sflag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        *sflag = wide_wait(&W.ctl->done, gridDim.x - 1, W.ctl, limit) ? 1 : 0;
    }
    __syncthreads();
    return *sflag != 0;
}

// Leader: inverse of the pivot block D = A[piv[j0+r]][j0+k] into W.Dinv by
// the whole leader CTA (cta_block_inverse; scratch: 32 * 32 + 194 LT); false
// if a pivot is zero or the inverse is not finite.
template <typename LT>
__device__ bool wide_pivot_block(const WideWs<LT> &W, int j0, int pb, LT *scratch) {
    for (int q = threadIdx.x; q < kWPB * kWPB; q += kThreads) {
        const int r = q / kWPB, c = q - r * kWPB;
        scratch[q] = (r < pb && c < pb) ? W.A[(int64_t)W.piv[j0 + r] * W.ld + j0 + c] : LT(0);
    }
    __syncthreads();
    return cta_block_inverse<LT>(scratch, kWPB, pb, W.Dinv, scratch + kWPB * kWPB);
}

// Leader: the panel's pivot rows among the rows not used yet (the
// tournament above when they outnumber tour_max), into piv[j0..] with
// used[] set.  0: done; 1: a column has no nonzero candidate (singular);
// 2: a wait ran out of time.
template <typename LT>
__device__ int wide_select_pivots(const WideWs<LT> &W, int j0, int pb, unsigned char *smem,
                                  uint64_t limit, int *sflag) {
    __shared__ int sel[kWPB];
    const int N = W.N;
    int C = cta_compact(nullptr, W.used, N, W.cand);
    int src = 0;
    while (C > tour_max((int)sizeof(LT))) {
        if (threadIdx.x == 0) {
            W.ctl->pad0 = C;
            W.ctl->pad1 = src;
        }
        wide_fork<LT>(W, kTaskPivotLevel, j0, pb, 0.0, nullptr);
        task_pivot_level<LT>(W, j0, pb, C, src, smem);
        if (!wide_join<LT>(W, limit, sflag)) return 2;
        const int ng = (C + kTourGroup - 1) / kTourGroup;
        C = cta_compact(W.cand + (int64_t)(src ^ 1) * N, nullptr, ng * kWPB,
                        W.cand + (int64_t)src * N);
    }
    const int n = cta_select<LT>(W, W.cand + (int64_t)src * N, C, j0, pb, smem, sel);
    if (n < pb) return 1;
    if (threadIdx.x < pb) {
        W.piv[j0 + threadIdx.x] = sel[threadIdx.x];
        W.used[sel[threadIdx.x]] = 1;
    }
    __syncthreads();
    return 0;
}

// Leader: assemble M = I - h*J(x) on all CTAs and invert it in place.
// Returns 0 (fresh pivots), 3 (the last fresh factorisation's pivot order,
// when `fresh` is false and it still gives invertible pivot blocks),
// 1 (a zero pivot column: singular), 2 (a wait ran out).
// cyc (thread 0): [0] += leader-only work (pivot searches, pivot-block
// inverses), [1] += panel-product tasks, [2] += assembly and rank-update tasks
// (each from fork to join).
template <typename LT>
__device__ int wide_factor(const WideWs<LT> &W, const Net &m, const double *x, double h,
                           bool fresh, double *mdiag, unsigned char *smem, double *red,
                           int *ired, uint64_t limit, int *sflag, long long *cyc) {
    const int tid = threadIdx.x, N = W.N;
    LT *sm = reinterpret_cast<LT *>(smem);
    bool use_old = !fresh && ld_acquire_i(W.flags) != 0;
    long long c0 = clock64(), c1;
    auto tick = [&](int slot) {
        c1 = clock64();
        if (tid == 0) cyc[slot] += c1 - c0;
        c0 = c1;
    };
    for (int attempt = 0; attempt < 2; attempt++) {
        wide_fork<LT>(W, kTaskAssemble, 0, 0, h, x);
        task_assemble<LT>(W, m, x, h, mdiag);
        if (!wide_join<LT>(W, limit, sflag)) return 2;
        tick(2);
        for (int i = tid; i < N; i += kThreads) {
            W.pos[i] = -1;
            if (!use_old) W.used[i] = 0;
        }
        __syncthreads();
        bool ok = true;
        for (int s0 = 0; s0 < N && ok; s0 += kWSP) {
            const int sw = min(kWSP, N - s0);
            // the panels of super-panel S, each updating S's column tile only
            for (int j0 = s0; j0 < s0 + sw; j0 += kWPB) {
                const int pb = min(kWPB, N - j0);
                if (!use_old) {
                    const int rc = wide_select_pivots<LT>(W, j0, pb, smem, limit, sflag);
                    if (rc == 2) return 2;
                    if (rc == 1) {
                        if (tid == 0) W.flags[0] = 0;
                        __syncthreads();
                        return 1;
                    }
                }
                __syncthreads();
                tick(0);
                if (j0 > s0 && tid < kWPB) W.pos[W.piv[j0 - kWPB + tid]] = -1;
                __syncthreads();
                if (tid < pb) W.pos[W.piv[j0 + tid]] = tid;
                if (!wide_pivot_block<LT>(W, j0, pb, sm)) {
                    ok = false;
                    break;
                }
                leader_snapshot<LT>(W, j0, pb, s0);
                tick(0);
                if (tid == 0) W.ctl->pad0 = s0;
                wide_fork<LT>(W, kTaskUpdate, j0, pb, h, x);
                task_update_narrow<LT>(W, j0, pb, sm, s0);
                if (!wide_join<LT>(W, limit, sflag)) return 2;
                tick(2);
            }
            if (!ok) break;
            // the last panel's pivots leave pos, S's pivots enter it
            const int jl = s0 + ((sw - 1) / kWPB) * kWPB;
            if (tid < s0 + sw - jl) W.pos[W.piv[jl + tid]] = -1;
            __syncthreads();
            if (sw < N) {
                // one rank-sw update of every other column tile
                if (tid < sw) W.pos[W.piv[s0 + tid]] = tid;
                wide_fork<LT>(W, kTaskPanelS, s0, sw, h, x);
                task_panel_s<LT>(W, s0, sw, sm);
                if (!wide_join<LT>(W, limit, sflag)) return 2;
                tick(1);
                wide_fork<LT>(W, kTaskUpdateS, s0, sw, h, x);
                bool tc_done = false;
                if constexpr (std::is_same<LT, float>::value) {
                    if (W.tc_on) {
                        task_update_s_tc(W, s0, sw, sm);
                        tc_done = true;
                    }
                }
                if (!tc_done) task_update_s<LT>(W, s0, sw, sm);
                if (!wide_join<LT>(W, limit, sflag)) return 2;
                tick(2);
                if (tid < sw) W.pos[W.piv[s0 + tid]] = -1;
                __syncthreads();
            }
        }
        if (ok) {
            if (tid == 0) W.flags[0] = 1;
            __syncthreads();
            return use_old ? 3 : 0;
        }
        if (!use_old) {
            if (tid == 0) W.flags[0] = 0;
            __syncthreads();
            return 1;
        }
        use_old = false;  // the old pivot order failed here: search afresh
    }
    return 1;
}

// Leader: W.vin holds r gathered by the pivot rows (vin[j] = r[piv[j]]);
// replaces it by the solution x[j] = (X * vin)[piv[j]].  False if a wait ran
// out of time.
template <typename LT>
__device__ bool wide_apply(const WideWs<LT> &W, unsigned char *smem, uint64_t limit,
                           int *sflag) {
    wide_fork<LT>(W, kTaskMatvec, 0, 0, 0.0, nullptr);
    task_matvec<LT>(W, reinterpret_cast<LT *>(smem));
    if (!wide_join<LT>(W, limit, sflag)) return false;
    for (int j = threadIdx.x; j < W.N; j += kThreads) W.vin[j] = W.vout[W.piv[j]];
    __syncthreads();
    return true;
}

// Leader: one RKF45 attempt over the grid.  Sets ok (all species accepted),
// dloc (min delta over the non-NaN deltas, +inf if none) and d0nan; sets
// abort if a wait ran out.
template <typename LT>
__device__ void wide_rkf_attempt(const WideWs<LT> &W, const Net &m, const Vecs &V, double dt,
                                 bool root_sqrt, double *pw, double *rate, uint64_t limit,
                                 int *sflag, bool &ok, double &dloc, bool &d0nan, bool &abort) {
    if (threadIdx.x == 0) {
        W.ctl->vecs = V;
        W.ctl->root_sqrt = root_sqrt ? 1 : 0;
    }
    for (int stg = 0; stg < 5; stg++) {
        const double *x = stg == 0 ? V.y1 : V.u;
        wide_fork<LT>(W, kTaskRates, 0, 0, dt, x);
        task_rates(m, x, pw, rate);
        if (!wide_join<LT>(W, limit, sflag)) { abort = true; return; }
        wide_fork<LT>(W, kTaskRkf, stg, 0, dt, x);
        task_rkf(m, V, stg, dt, pw, rate);
        if (!wide_join<LT>(W, limit, sflag)) { abort = true; return; }
    }
    wide_fork<LT>(W, kTaskRates, 0, 0, dt, V.u);
    task_rates(m, V.u, pw, rate);
    if (!wide_join<LT>(W, limit, sflag)) { abort = true; return; }
    wide_fork<LT>(W, kTaskRkfFinal, 0, 0, dt, V.u);
    // species 0 belongs to the leader (global thread 0)
    __shared__ double red2[2 * kWarps + 1];
    d0nan = task_rkf_final(W.part, m, V, dt, root_sqrt, pw, rate, red2);
    if (!wide_join<LT>(W, limit, sflag)) { abort = true; return; }
    long long mn = 0x7ff0000000000000LL;
    int all = 1;
    for (int g = 0; g < (int)gridDim.x; g++) {
        all &= (int)W.part[g];
        const long long b = W.part[kWideMaxGrid + g];
        mn = b < mn ? b : mn;
    }
    ok = all != 0;
    dloc = __longlong_as_double(mn);
}

// Leader: one refinement sweep's solve and update over the grid; cmax, xmax
// as the batched engine's (uniform).  False if a wait ran out.
template <typename LT>
__device__ bool wide_solve_update(const WideWs<LT> &W, const Vecs &V, double sc, double isc,
                                  long long lost, LT *sm, uint64_t limit, int *sflag,
                                  double &cmax, double &xmax) {
    __shared__ double red3[2 * kWarps + 1];
    if (threadIdx.x == 0) {
        W.ctl->vecs = V;
        W.ctl->sc = sc;
        W.ctl->isc = isc;
        W.ctl->lost = lost;
    }
    wide_fork<LT>(W, kTaskSolve, 0, 0, 0.0, nullptr);
    task_solve<LT>(W, V.k6, sc, sm);
    if (!wide_join<LT>(W, limit, sflag)) return false;
    wide_fork<LT>(W, kTaskSolveUpdate, 0, 0, 0.0, nullptr);
    task_solve_update<LT>(W, V, sc, isc, lost, red3);
    if (!wide_join<LT>(W, limit, sflag)) return false;
    long long cm = 0, xm = 0;
    for (int g = 0; g < (int)gridDim.x; g++) {
        cm = max(cm, W.part[g]);
        xm = max(xm, W.part[kWideMaxGrid + g]);
    }
    cmax = __longlong_as_double(cm);
    xmax = __longlong_as_double(xm);
    return true;
}

// Leader: res = xr - (dx - dt * J(xf) dx) over the grid and its max (rmax).
template <typename LT>
__device__ bool wide_residual(const WideWs<LT> &W, const Net &m, const Vecs &V, double dt,
                              uint64_t limit, int *sflag, double &rmax) {
    __shared__ double red4[2 * kWarps + 1];
    if (threadIdx.x == 0) W.ctl->vecs = V;
    wide_fork<LT>(W, kTaskJv, 0, 0, dt, nullptr);
    task_jv(m, V.k5, V.k4, W.qr);
    if (!wide_join<LT>(W, limit, sflag)) return false;
    wide_fork<LT>(W, kTaskResidual, 0, 0, dt, nullptr);
    task_residual(W.part, m, V, dt, W.qr, red4);
    if (!wide_join<LT>(W, limit, sflag)) return false;
    long long rm = 0;
    for (int g = 0; g < (int)gridDim.x; g++) rm = max(rm, W.part[g]);
    rmax = __longlong_as_double(rm);
    return true;
}

// Leader: the Newton residual over the grid (task_newton_rhs).
template <typename LT>
__device__ bool wide_newton_rhs(const WideWs<LT> &W, const Net &m, const Vecs &V, double dt,
                                bool first, uint64_t limit, int *sflag) {
    if (threadIdx.x == 0) W.ctl->vecs = V;
    wide_fork<LT>(W, kTaskRates, 0, 0, dt, V.k2);
    task_rates(m, V.k2, W.pw, W.qr);
    if (!wide_join<LT>(W, limit, sflag)) return false;
    wide_fork<LT>(W, kTaskNewtonRhs, first ? 1 : 0, 0, dt, nullptr);
    task_newton_rhs(m, V, dt, first, W.pw, W.qr);
    return wide_join<LT>(W, limit, sflag);
}

// Leader: release the workers.
template <typename LT>
__device__ void wide_exit(const WideWs<LT> &W) {
    wide_fork<LT>(W, kTaskExit, 0, 0, 0.0, nullptr);
}
