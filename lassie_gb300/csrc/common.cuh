// Shared device/host definitions of the LASSIE GB300 engine.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "lassie_gb300.h"

namespace lassie {

// One CTA integrates one instance at a time; 512 threads = 16 warps.
constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
// Largest network of the wide engine (one instance over the whole GPU).
constexpr int kWideMaxSpecies = 16384;

// Packed sparse entries: value = index * 256 + (int8 coefficient).
__host__ __device__ __forceinline__ int ent_index(int e) { return e >> 8; }
__host__ __device__ __forceinline__ int ent_coef(int e) {
    return (int)(int8_t)(uint8_t)(e & 255);
}
__host__ __device__ __forceinline__ int make_ent(int index, int coef) {
    return index * 256 + (coef & 255);
}

// Per-instance descriptor: offsets into the int / double / output arenas.
struct InstDesc {
    int32_t n, r, nt, ncs;
    int32_t nnz_a, nnz_h, flags, pad;
    int64_t rxn_ptr, rxn_ent, sp_ptr, sp_ent;  // int arena
    int64_t hr_ptr, hr_ent, as_ptr, as_ent;    // int arena (adjoint structure)
    int64_t cs;                                // int arena, -1 = all species
    int64_t k, x0, feed, atol, t;              // double arena, feed/atol -1 = none
    int64_t out;                               // output arena
    double rkf_step, be_step, newton_tol, stiffness_tol;
    int64_t newton_iter, max_steps;
};

// Per-instance result; layout identical to lassie_stats.
struct InstResult {
    int64_t outer_iters, rkf_accepts, rkf_retries, be_steps, newton_iters,
        lu_factorisations, lu_failures, nan_reverts, refine_sweeps;
    int64_t cycles_rkf, cycles_matrix, cycles_lu, cycles_solve;
    int64_t cycles_lu_panel, cycles_lu_rows, cycles_lu_trailing, cycles_solve_tri;
    double t_final, dt_be_final;
    int32_t status, pad;
    int64_t jac_evals, rhs_evals;  // BDF controller
    int32_t order_final, pad2;
    int64_t cycles_total;  // the instance's whole integration
};
static_assert(sizeof(InstResult) == sizeof(lassie_stats), "stats layout");

// Per-instance record of the forward step sequence (adjoint).  Step kinds:
// 0 accepted RKF45 step, 1 backward-Euler step, 2 backward-Euler step that
// left the state unchanged (LU failure), 3 backward-Euler step with reverted
// species.  The output state of every backward-Euler step is stored; accepted
// RKF45 steps store their output every `ckpt_every` steps (the others are
// recomputed in the backward pass).  Slot 0 holds the initial state.
struct AdjDesc {
    int64_t rec;       // offset into rec_kind / rec_dt / rec_slot
    int64_t states;    // offset into the state store (doubles)
    int64_t samp;      // offset into samp_step (one per sample)
    int64_t grad;      // offset into grad: d loss / d log k [R], then d loss / d x0 [N]
    int32_t cap_steps, cap_states;
};

struct AdjArrays {
    const AdjDesc *desc;
    int32_t *rec_kind;
    double *rec_dt;
    int32_t *rec_slot;
    double *states;
    int32_t *nsteps;     // per instance
    int32_t *samp_step;
    const double *target;  // same layout as the outputs
    double *grad;
    double *scratch;       // per CTA: (ckpt_every + 1) states for recomputation
    int64_t scratch_stride;
    int32_t ckpt_every;
};

struct LaunchParams {
    const InstDesc *inst;
    int32_t n_inst;
    const int32_t *order;  // processing order (largest first)
    int32_t *queue;        // work-queue counter, zeroed before launch
    const int32_t *iarena;
    const double *darena;
    double *out;
    InstResult *res;
    unsigned char *workspace;  // per-CTA Newton matrix
    int64_t ws_stride;         // bytes per CTA
    int32_t nmax, rmax, amax, hmax;  // largest N, R, nnz_A, nnz_H in the batch
    int32_t precision, refine_max, lu_reuse, tensor_cores;
    uint64_t deadline_ns;      // per-launch wall-clock limit (ns), 0 = none
    AdjArrays adj;             // adj.desc == nullptr: no recording
    // controller: 0 LASSIE's loop (integrate), 1 BDF with rtol/atol (bdf_integrate)
    int32_t controller, max_order;
    double rtol, atol, first_step, max_step;
};

// Dynamic shared-memory layout of the integrator (bytes), identical on host
// and device.  Vectors are nvec FP64 N-vectors (10 for LASSIE's loop, more
// for the BDF controller's differences); the sparse structure of the
// network is staged here too; lt holds the factor panel column-major
// (PB x (round_up32(N) + 4), plus slack for the 8-row tile reads past its end),
// utile one PB x 128 tile of U12, rowbuf the pivot and swap rows.
struct SmemLayout {
    int64_t vec, kk, pw, qr, rptr, sptr, sent, rent, perm, slot, bvec, lt, utile, rowbuf, dblk, total;
    __host__ __device__ static int64_t align(int64_t v) { return (v + 15) & ~int64_t(15); }
    __host__ __device__ SmemLayout(int nmax, int rmax, int amax, int hmax, int lt_bytes, int pb,
                                   int tn, int nvec = 10) {
        int64_t o = 0;
        vec = o;    o = align(o + int64_t(nvec) * nmax * 8);
        kk = o;     o = align(o + int64_t(rmax) * 8);
        pw = o;     o = align(o + int64_t(amax > 0 ? amax : 1) * 8);
        qr = o;     o = align(o + int64_t(rmax) * 8);
        rptr = o;   o = align(o + int64_t(rmax + 1) * 4);
        sptr = o;   o = align(o + int64_t(nmax + 1) * 4);
        sent = o;   o = align(o + int64_t(hmax > 0 ? hmax : 1) * 4);
        rent = o;   o = align(o + int64_t(amax > 0 ? amax : 1) * 4);
        perm = o;   o = align(o + int64_t(nmax) * 4);
        slot = o;   o = align(o + int64_t(nmax) * 4);
        bvec = o;   o = align(o + int64_t(nmax) * lt_bytes);
        // 160 elements of slack (1280 bytes whatever the element type, so that
        // an FP64 panel of half the width also fits)
        lt = o;     o = align(o + int64_t(pb) * (((nmax + 31) & ~31) + 4) * lt_bytes + 160 * 8);
        utile = o;  o = align(o + int64_t(pb) * tn * lt_bytes);
        rowbuf = o; o = align(o + int64_t(2 * pb) * lt_bytes);
        dblk = o;   o = align(o + int64_t(pb) * pb * lt_bytes);
        total = o;
    }
};

// Panel width and trailing tile width of the per-CTA LU, per element type.
template <typename LT> struct LuShape;
template <> struct LuShape<float> { static constexpr int PB = 32, TN = 128; };
template <> struct LuShape<double> { static constexpr int PB = 16, TN = 128; };

__host__ __device__ __forceinline__ int round_up4(int n) { return (n + 3) & ~3; }

}  // namespace lassie
