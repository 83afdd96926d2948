// C ABI of the LASSIE GB300 engine: model compiler, batch packing, device
// memory, launches.  Host code only; the kernels are in compat_engine.cu.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <numeric>
#include <tuple>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"
#include "lassie_gb300.h"

namespace lassie {
int64_t compat_smem_bytes(int nmax, int rmax, int amax, int hmax, int precision,
                          int controller);
cudaError_t compat_configure(int precision, int64_t smem);
cudaError_t compat_launch(const LaunchParams &P, int grid, int64_t smem, cudaStream_t stream);
int64_t wide_workspace_bytes(int N, int R, int nnz_a, int precision);
int64_t wide_flags_offset(int N, int R, int nnz_a, int precision);
int64_t wide_dynamic_smem(int N, int precision);
int wide_configure(int precision, int64_t smem, int sm_count);
cudaError_t wide_launch(const LaunchParams &P, int grid, int64_t smem, cudaStream_t stream);
cudaError_t rhs_batch_launch(int n_inst, int N, int R, int nnz_a, int nnz_h, const int *rptr,
                             const int *rent, const int *sptr, const int *sent, const int *order,
                             const double *k, const double *x, double *dx, int sm_count,
                             cudaStream_t stream);
cudaError_t newton_matrix_launch(int N, int R, int nnz_a, const int *rptr, const int *rent,
                                 const int *sptr, const int *sent, const double *k,
                                 const double *x, double h, double *M, cudaStream_t stream);
cudaError_t newton_batch_launch(int n_inst, int N, int R, const int *rptr, const int *rent,
                                const int *jac, int64_t nnz, const double *k, const double *x,
                                double h, void *M, bool fp32, int sm_count, cudaStream_t stream);
cudaError_t lu_solve_launch(int N, void *A, int ld, const double *b, double *x, int *info,
                            int precision, cudaStream_t stream);
int64_t lu_solve_smem(int N, int precision);
int64_t adjoint_smem_bytes(int nmax, int rmax, int amax, int hmax);
cudaError_t adjoint_launch(const LaunchParams &P, int grid, int64_t smem, cudaStream_t stream);
int64_t tune_factor_smem(int N, int precision);
int64_t float_smem_bytes(int nmax, int rmax, int amax, int hmax);
cudaError_t float_configure(int64_t smem);
cudaError_t float_launch(const LaunchParams &P, int grid, int64_t smem, cudaStream_t stream);
cudaError_t tune_factor_launch(int precision, int N, int rm, int reps, void *ws,
                               int64_t ws_stride, int grid, int *fails, cudaStream_t stream);
}  // namespace lassie

using namespace lassie;

// ----------------------------------------------------------- error state

static thread_local std::string g_last_error;

static int set_error(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}

#define CU(call)                                                                     \
    do {                                                                             \
        cudaError_t _e = (call);                                                     \
        if (_e != cudaSuccess)                                                       \
            return set_error(LASSIE_ERR_CUDA, std::string(#call) + ": " +           \
                                                  cudaGetErrorString(_e));           \
    } while (0)

// ----------------------------------------------------------------- model

struct lassie_model {
    int32_t N = 0, R = 0;
    std::vector<int32_t> rxn_ptr, rxn_ent, sp_ptr, sp_ent;
    // for vector-Jacobian products (adjoint): net stoichiometry by reaction
    // (species * 256 + coefficient), and the reactant entries of each species
    // (indices into rxn_ent)
    std::vector<int32_t> hr_ptr, hr_ent, as_ptr, as_ent;
    std::mutex mu;
    int dev = -1;
    int32_t *d_struct = nullptr;  // [rxn_ptr | rxn_ent | sp_ptr | sp_ent]
    // structural nonzeros of J and their terms (model_jac_device), built on
    // the first batched Newton-matrix call
    int32_t *d_jac = nullptr;
    int64_t jac_nnz = 0;
    // reactions, then species, in descending order of their loop trip counts
    // in the batched RHS (model_order_device)
    int32_t *d_order = nullptr;

    int64_t off_rent() const { return R + 1; }
    int64_t off_sptr() const { return off_rent() + (int64_t)rxn_ent.size(); }
    int64_t off_sent() const { return off_sptr() + N + 1; }
    int64_t off_hrptr() const { return off_sent() + (int64_t)sp_ent.size(); }
    int64_t off_hrent() const { return off_hrptr() + R + 1; }
    int64_t off_asptr() const { return off_hrent() + (int64_t)hr_ent.size(); }
    int64_t off_asent() const { return off_asptr() + N + 1; }
    int64_t struct_len() const { return off_asent() + (int64_t)as_ent.size(); }
    void pack(std::vector<int32_t> &out) const {
        out.insert(out.end(), rxn_ptr.begin(), rxn_ptr.end());
        out.insert(out.end(), rxn_ent.begin(), rxn_ent.end());
        out.insert(out.end(), sp_ptr.begin(), sp_ptr.end());
        out.insert(out.end(), sp_ent.begin(), sp_ent.end());
        out.insert(out.end(), hr_ptr.begin(), hr_ptr.end());
        out.insert(out.end(), hr_ent.begin(), hr_ent.end());
        out.insert(out.end(), as_ptr.begin(), as_ptr.end());
        out.insert(out.end(), as_ent.begin(), as_ent.end());
    }
};

static const int kMaxIndex = (1 << 23) - 1;

// Simulation.cuh:397-418, 1061-1130: reactants by reaction (species
// ascending), net stoichiometry H = (B-A)^T by species (reactions ascending).
static int build_model(int32_t N, int32_t R, const std::vector<std::vector<std::pair<int, int>>> &A,
                       const std::vector<std::vector<std::pair<int, int>>> &H, lassie_model **out) {
    lassie_model *m = new (std::nothrow) lassie_model;
    if (!m) return set_error(LASSIE_ERR_ALLOC, "model allocation");
    m->N = N;
    m->R = R;
    m->rxn_ptr.resize(R + 1);
    for (int j = 0; j < R; j++) {
        m->rxn_ptr[j] = (int32_t)m->rxn_ent.size();
        for (auto &e : A[j]) {
            if (e.second < -128 || e.second > 127) {
                delete m;
                return set_error(LASSIE_ERR_TOO_LARGE, "stoichiometry outside [-128,127]");
            }
            m->rxn_ent.push_back(make_ent(e.first, e.second));
        }
    }
    m->rxn_ptr[R] = (int32_t)m->rxn_ent.size();
    std::vector<std::vector<std::pair<int, int>>> bys(N);
    for (int j = 0; j < R; j++)
        for (auto &e : H[j]) bys[e.first].push_back({j, e.second});
    m->sp_ptr.resize(N + 1);
    for (int s = 0; s < N; s++) {
        m->sp_ptr[s] = (int32_t)m->sp_ent.size();
        for (auto &e : bys[s]) {
            if (e.second < -128 || e.second > 127) {
                delete m;
                return set_error(LASSIE_ERR_TOO_LARGE, "net stoichiometry outside [-128,127]");
            }
            m->sp_ent.push_back(make_ent(e.first, e.second));
        }
    }
    m->sp_ptr[N] = (int32_t)m->sp_ent.size();
    m->hr_ptr.resize(R + 1);
    for (int j = 0; j < R; j++) {
        m->hr_ptr[j] = (int32_t)m->hr_ent.size();
        for (auto &e : H[j]) m->hr_ent.push_back(make_ent(e.first, e.second));
    }
    m->hr_ptr[R] = (int32_t)m->hr_ent.size();
    std::vector<std::vector<int>> as(N);
    for (int j = 0; j < R; j++)
        for (int q = m->rxn_ptr[j]; q < m->rxn_ptr[j + 1]; q++) as[ent_index(m->rxn_ent[q])].push_back(q);
    m->as_ptr.resize(N + 1);
    for (int sp = 0; sp < N; sp++) {
        m->as_ptr[sp] = (int32_t)m->as_ent.size();
        for (int q : as[sp]) m->as_ent.push_back(q);
    }
    m->as_ptr[N] = (int32_t)m->as_ent.size();
    *out = m;
    return LASSIE_OK;
}

extern "C" int lassie_model_create_dense(int32_t N, int32_t R, const int32_t *left,
                                         const int32_t *right, lassie_model **out) {
    if (!out || !left || !right || N <= 0 || R <= 0 || N > kMaxIndex || R > kMaxIndex)
        return set_error(LASSIE_ERR_ARGS, "model_create_dense: bad arguments");
    std::vector<std::vector<std::pair<int, int>>> A(R), H(R);
    for (int j = 0; j < R; j++) {
        const int32_t *l = left + (int64_t)j * N, *r = right + (int64_t)j * N;
        for (int s = 0; s < N; s++) {
            if (l[s] != 0) A[j].push_back({s, l[s]});
            const int h = r[s] - l[s];
            if (h != 0) H[j].push_back({s, h});
        }
    }
    return build_model(N, R, A, H, out);
}

extern "C" int lassie_model_create_csr(int32_t N, int32_t R, const int32_t *rp,
                                       const int32_t *rs, const int32_t *rc, const int32_t *pp,
                                       const int32_t *ps, const int32_t *pc, lassie_model **out) {
    if (!out || !rp || !pp || N <= 0 || R <= 0 || N > kMaxIndex || R > kMaxIndex)
        return set_error(LASSIE_ERR_ARGS, "model_create_csr: bad arguments");
    std::vector<std::vector<std::pair<int, int>>> A(R), H(R);
    for (int j = 0; j < R; j++) {
        std::map<int, int> a, b;
        for (int q = rp[j]; q < rp[j + 1]; q++) {
            if (rs[q] < 0 || rs[q] >= N) return set_error(LASSIE_ERR_ARGS, "species index");
            a[rs[q]] += rc[q];
        }
        for (int q = pp[j]; q < pp[j + 1]; q++) {
            if (ps[q] < 0 || ps[q] >= N) return set_error(LASSIE_ERR_ARGS, "species index");
            b[ps[q]] += pc[q];
        }
        std::map<int, int> h;
        for (auto &e : a)
            if (e.second != 0) A[j].push_back(e);
        for (auto &e : a) h[e.first] -= e.second;
        for (auto &e : b) h[e.first] += e.second;
        for (auto &e : h)
            if (e.second != 0) H[j].push_back(e);
    }
    return build_model(N, R, A, H, out);
}

extern "C" void lassie_model_destroy(lassie_model *m) {
    if (!m) return;
    if (m->d_struct) {
        int cur = 0;
        cudaGetDevice(&cur);
        cudaSetDevice(m->dev);
        cudaFree(m->d_struct);
        if (m->d_jac) cudaFree(m->d_jac);
        if (m->d_order) cudaFree(m->d_order);
        cudaSetDevice(cur);
    }
    delete m;
}

extern "C" int lassie_model_info(const lassie_model *m, int32_t *n, int32_t *r, int32_t *na,
                                 int32_t *nh) {
    if (!m) return set_error(LASSIE_ERR_ARGS, "null model");
    if (n) *n = m->N;
    if (r) *r = m->R;
    if (na) *na = (int32_t)m->rxn_ent.size();
    if (nh) *nh = (int32_t)m->sp_ent.size();
    return LASSIE_OK;
}

// Device copy of a model's structure (for the single-evaluation entry points).
static int model_device(lassie_model *m, const int32_t **d) {
    std::lock_guard<std::mutex> g(m->mu);
    int dev = 0;
    CU(cudaGetDevice(&dev));
    if (m->d_struct && m->dev == dev) {
        *d = m->d_struct;
        return LASSIE_OK;
    }
    if (m->d_struct) {
        return set_error(LASSIE_ERR_ARGS, "model already bound to another device");
    }
    std::vector<int32_t> h;
    m->pack(h);
    CU(cudaMalloc(&m->d_struct, h.size() * sizeof(int32_t)));
    CU(cudaMemcpy(m->d_struct, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    m->dev = dev;
    *d = m->d_struct;
    return LASSIE_OK;
}

namespace lassie {
// Host-side packing of a model for lassie_solve_noalloc (no device memory).
int model_pack_for_noalloc(const lassie_model *m, std::vector<int32_t> &out, int32_t *n,
                           int32_t *r, int32_t *nnz_a, int32_t *nnz_h, int64_t offs[8]) {
    if (!m) return set_error(LASSIE_ERR_ARGS, "null model");
    out.clear();
    m->pack(out);
    *n = m->N;
    *r = m->R;
    *nnz_a = (int32_t)m->rxn_ent.size();
    *nnz_h = (int32_t)m->sp_ent.size();
    offs[0] = 0;
    offs[1] = m->off_rent();
    offs[2] = m->off_sptr();
    offs[3] = m->off_sent();
    offs[4] = m->off_hrptr();
    offs[5] = m->off_hrent();
    offs[6] = m->off_asptr();
    offs[7] = m->off_asent();
    return LASSIE_OK;
}
int set_error_noalloc(int status, const char *msg) { return set_error(status, msg); }
}  // namespace lassie

// ------------------------------------------------------------- utilities

extern "C" void lassie_opts_default(lassie_opts *o) {
    if (!o) return;
    o->rkf_step = 1e-3;
    o->be_step = 0.01;
    o->newton_tol = 1e-6;
    o->stiffness_tol = 1e-6;
    o->newton_iter = 10000;
    o->max_steps = 0;
    o->deadline_s = 0.0;
    o->precision = LASSIE_PREC_MIXED;
    o->refine_max = 0;
    o->quarter_root = LASSIE_ROOT_POW;
    o->lu_reuse = 1;
    o->tensor_cores = LASSIE_TC_TF32;
    o->controller = LASSIE_CTRL_COMPAT;
    o->rtol = 1e-6;
    o->atol = 1e-9;
    o->first_step = 0.0;
    o->max_step = 0.0;
    o->max_order = 5;
    o->tile_rows = 0;
}

extern "C" const char *lassie_status_string(int s) {
    switch (s) {
    case LASSIE_OK: return "ok";
    case LASSIE_ERR_INPUT_FOLDER: return "the input folder does not exist";
    case LASSIE_ERR_MANDATORY: return "a mandatory input file is missing or inconsistent";
    case LASSIE_ERR_MODELKIND: return "modelkind must be deterministic/concentration or stochastic/number";
    case LASSIE_ERR_VOLUME: return "stochastic model without a volume";
    case LASSIE_ERR_ORDER: return "a reaction has order higher than two";
    case LASSIE_ERR_CUDA: return "CUDA error";
    case LASSIE_ERR_ARGS: return "invalid argument";
    case LASSIE_ERR_MAX_STEPS: return "maximum number of steps reached";
    case LASSIE_ERR_ALLOC: return "allocation failed";
    case LASSIE_ERR_TOO_LARGE: return "network too large for the engine";
    case LASSIE_ERR_DEADLINE: return "device deadline elapsed";
    case LASSIE_ERR_NO_DEVICE: return "no sm_103 CUDA device";
    case LASSIE_ERR_RECORD_FULL: return "adjoint step record is full";
    case LASSIE_ERR_STEP_TOO_SMALL: return "BDF step size below 10 ulp of t";
    default: return "unknown status";
    }
}

extern "C" const char *lassie_last_error(void) { return g_last_error.c_str(); }

extern "C" int lassie_device_ok(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return 0;
    }
    int dev = 0;
    cudaDeviceProp p;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess)
        return 0;
    return (p.major == 10 && p.minor == 3) ? 1 : 0;
}

// Grow-only device buffer.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    int grow(size_t n) {
        if (n <= cap) return LASSIE_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(n, 256);
        if (cudaMalloc(&p, want) != cudaSuccess) {
            cudaGetLastError();
            return set_error(LASSIE_ERR_ALLOC, "cudaMalloc of " + std::to_string(want) + " bytes");
        }
        cap = want;
        return LASSIE_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// ----------------------------------------------------------------- batch

struct lassie_batch {
    int dev = 0;
    int n = 0;
    int sm_count = 0;
    lassie_opts opts{};
    std::vector<InstDesc> desc;
    std::vector<int32_t> order;
    int64_t n_int = 0, n_dbl = 0, n_out = 0;
    int32_t nmax = 0, rmax = 0, amax = 0, hmax = 0;
    int64_t smem = 0;
    int grid = 0;
    bool wide = false;       // one instance above kThreads species: the wide engine
    int64_t wide_flags = 0;  // offset of the wide engine's pivot-order flag
    DevBuf d_int, d_dbl, d_out, d_desc, d_order, d_res, d_queue, d_ws;
    cudaStream_t stream = nullptr;
    LaunchParams P{};
    ~lassie_batch() {
        d_int.release();
        d_dbl.release();
        d_out.release();
        d_desc.release();
        d_order.release();
        d_res.release();
        d_queue.release();
        d_ws.release();
    }
};

static int validate_instance(const lassie_instance &q) {
    if (!q.model || !q.k || !q.x0 || (q.nt > 0 && (!q.t || !q.out)) || q.nt < 0)
        return set_error(LASSIE_ERR_ARGS, "instance: missing buffer");
    const int N = q.model->N;
    if (q.cs) {
        if (q.ncs < 0) return set_error(LASSIE_ERR_ARGS, "instance: ncs");
        for (int j = 0; j < q.ncs; j++)
            if (q.cs[j] < 0 || q.cs[j] >= N)
                return set_error(LASSIE_ERR_ARGS, "instance: cs out of range");
    }
    return LASSIE_OK;
}

// ------------------------------------------------------------ autotuner
// The per-CTA factorisation's trailing update runs in 128 x 16*rows tiles;
// rows = 8 suits large networks (register blocking), 4 or 2 keep more of the
// CTA busy on small ones.  Per network-size band the candidates are timed on
// the device -- every CTA of the batch's grid factoring a test matrix of the
// band's size, three times, after a warm-up -- and the fastest is kept
// unless the default (8) is within 5 %.  Choices are cached per device,
// precision, size and grid, so a process decides once and later batches
// repeat the decision.  Results do not depend on the choice.
static const int kTuneBandEdge[] = {32, 64, 128, 256, 512};
static const int kTuneBandSize[] = {24, 48, 96, 192, 384};  // size timed per band

static int tune_band(int n) {
    int b = 0;
    while (b < 4 && n > kTuneBandEdge[b]) b++;
    return b;
}

static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int>, int> g_tune_cache;

static int tuned_tile_rows(lassie_batch *b, int precision, int N) {
    const auto key = std::make_tuple(b->dev, precision, N, b->grid);
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) return it->second;
    const int64_t smem = tune_factor_smem(N, precision);
    int max_optin = 0;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->dev);
    int choice = 8;
    if (smem <= max_optin - 1024) {
        cudaEvent_t e0, e1;
        if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
            const int rows[3] = {8, 4, 2};
            float ms[3] = {0.f, 0.f, 0.f};
            bool ok = true;
            int *fails = reinterpret_cast<int *>(b->d_queue.p);
            for (int c = 0; c < 3 && ok; c++) {
                ok = tune_factor_launch(precision, N, rows[c], 1, b->d_ws.p, b->P.ws_stride,
                                        b->grid, fails, nullptr) == cudaSuccess &&
                     cudaEventRecord(e0, nullptr) == cudaSuccess &&
                     tune_factor_launch(precision, N, rows[c], 3, b->d_ws.p, b->P.ws_stride,
                                        b->grid, fails, nullptr) == cudaSuccess &&
                     cudaEventRecord(e1, nullptr) == cudaSuccess &&
                     cudaEventSynchronize(e1) == cudaSuccess &&
                     cudaEventElapsedTime(&ms[c], e0, e1) == cudaSuccess;
            }
            if (ok) {
                int best = 0;
                for (int c = 1; c < 3; c++)
                    if (ms[c] < ms[best]) best = c;
                if (ms[best] < 0.95f * ms[0]) choice = rows[best];
            }
            cudaGetLastError();
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    g_tune_cache[key] = choice;
    return choice;
}

static int tile_code(int rows) { return rows == 4 ? 1 : (rows == 2 ? 2 : 0); }

extern "C" int lassie_batch_tile_rows(const lassie_batch *b, int32_t *rows) {
    if (!b || (b->n > 0 && !rows)) return set_error(LASSIE_ERR_ARGS, "batch_tile_rows");
    for (int q = 0; q < b->n; q++) {
        const int c = (b->desc[q].flags >> 4) & 3;
        rows[q] = c == 1 ? 4 : (c == 2 ? 2 : 8);
    }
    return LASSIE_OK;
}

extern "C" int lassie_batch_create(const lassie_instance *inst, int32_t n, const lassie_opts *opts,
                                   lassie_batch **out) {
    if (!out || (n > 0 && !inst) || n < 0) return set_error(LASSIE_ERR_ARGS, "batch_create");
    lassie_opts o;
    if (opts) o = *opts;
    else lassie_opts_default(&o);
    if (o.precision != LASSIE_PREC_FP64 && o.precision != LASSIE_PREC_MIXED &&
        o.precision != LASSIE_PREC_FLOAT)
        return set_error(LASSIE_ERR_ARGS, "precision");
    if (o.controller != LASSIE_CTRL_COMPAT && o.controller != LASSIE_CTRL_BDF)
        return set_error(LASSIE_ERR_ARGS, "controller");
    const bool fmode = o.precision == LASSIE_PREC_FLOAT;
    if (fmode && o.controller != LASSIE_CTRL_COMPAT)
        return set_error(LASSIE_ERR_ARGS, "the float mode runs LASSIE's controller only");
    if (o.tile_rows != 0 && o.tile_rows != 8 && o.tile_rows != 4 && o.tile_rows != 2)
        return set_error(LASSIE_ERR_ARGS, "tile_rows must be 0 (autotuned), 8, 4 or 2");
    const bool bdf = o.controller == LASSIE_CTRL_BDF;
    if (bdf) {
        if (!(o.rtol > 0.0) || !(o.atol >= 0.0) || o.max_order < 1 || o.max_order > 5 ||
            o.first_step < 0.0 || o.max_step < 0.0)
            return set_error(LASSIE_ERR_ARGS, "BDF controller options");
    }
    for (int q = 0; q < n; q++) {
        int rc = validate_instance(inst[q]);
        if (rc) return rc;
        if (bdf && inst[q].model->N > kThreads)
            return set_error(LASSIE_ERR_TOO_LARGE, "the BDF controller runs networks of at most " +
                                                       std::to_string(kThreads) + " species");
        if (bdf)  // the BDF loop advances to t[nt-1] through finite, ordered samples
            for (int i = 0; i < inst[q].nt; i++)
                if (!std::isfinite(inst[q].t[i]) || (i > 0 && !(inst[q].t[i] >= inst[q].t[i - 1])))
                    return set_error(LASSIE_ERR_ARGS,
                                     "BDF controller: sample times must be finite and ascending");
    }
    lassie_batch *b = new (std::nothrow) lassie_batch;
    if (!b) return set_error(LASSIE_ERR_ALLOC, "batch allocation");
    b->n = n;
    b->opts = o;
    int rc;
    if (cudaGetDevice(&b->dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->dev) !=
            cudaSuccess) {
        delete b;
        cudaGetLastError();
        return set_error(LASSIE_ERR_NO_DEVICE, "no CUDA device");
    }
    // pack arenas: one copy of each distinct network
    std::map<const lassie_model *, int64_t> model_off;
    std::vector<int32_t> hint;
    std::vector<double> hdbl;
    b->desc.resize(n);
    int64_t outpos = 0;
    for (int q = 0; q < n; q++) {
        const lassie_instance &I = inst[q];
        const lassie_model *m = I.model;
        auto it = model_off.find(m);
        int64_t base;
        if (it == model_off.end()) {
            base = (int64_t)hint.size();
            model_off[m] = base;
            m->pack(hint);
        } else {
            base = it->second;
        }
        InstDesc &D = b->desc[q];
        D.n = m->N;
        D.r = m->R;
        D.nt = I.nt;
        D.ncs = I.cs ? I.ncs : m->N;
        D.nnz_a = (int32_t)m->rxn_ent.size();
        D.nnz_h = (int32_t)m->sp_ent.size();
        D.rxn_ptr = base;
        D.rxn_ent = base + m->off_rent();
        D.sp_ptr = base + m->off_sptr();
        D.sp_ent = base + m->off_sent();
        D.hr_ptr = base + m->off_hrptr();
        D.hr_ent = base + m->off_hrent();
        D.as_ptr = base + m->off_asptr();
        D.as_ent = base + m->off_asent();
        if (I.cs) {
            D.cs = (int64_t)hint.size();
            hint.insert(hint.end(), I.cs, I.cs + I.ncs);
        } else {
            D.cs = -1;
        }
        auto put = [&](const double *src, int64_t len) -> int64_t {
            if (!src) return -1;
            int64_t o = (int64_t)hdbl.size();
            hdbl.insert(hdbl.end(), src, src + len);
            return o;
        };
        D.k = put(I.k, m->R);
        D.x0 = put(I.x0, m->N);
        D.feed = put(I.feed, m->N);
        D.atol = put(I.atol, m->N);
        D.t = I.nt > 0 ? put(I.t, I.nt) : 0;
        D.out = outpos;
        outpos += (int64_t)I.nt * D.ncs;
        D.rkf_step = o.rkf_step;
        D.be_step = o.be_step;
        D.newton_tol = o.newton_tol;
        D.stiffness_tol = o.stiffness_tol;
        D.newton_iter = o.newton_iter;
        D.max_steps = o.max_steps;
        D.flags = o.quarter_root == LASSIE_ROOT_SQRT ? 1 : 0;
        b->nmax = std::max(b->nmax, m->N);
        b->rmax = std::max(b->rmax, m->R);
        b->amax = std::max(b->amax, (int32_t)m->rxn_ent.size());
        b->hmax = std::max(b->hmax, (int32_t)m->sp_ent.size());
    }
    if (hdbl.empty()) hdbl.push_back(0.0);
    if (hint.empty()) hint.push_back(0);
    b->n_int = (int64_t)hint.size();
    b->n_dbl = (int64_t)hdbl.size();
    b->n_out = std::max<int64_t>(outpos, 1);
    // largest networks first: the dense LU cost grows as N^3
    b->order.resize(n);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(),
                     [&](int a, int c) { return b->desc[a].n > b->desc[c].n; });
    int max_optin = 0;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->dev);
    int64_t ws_stride = 0, ws_total = 0;
    if (fmode && b->nmax > kThreads) {
        delete b;
        return set_error(LASSIE_ERR_TOO_LARGE, "the float mode runs networks of at most " +
                                                   std::to_string(kThreads) + " species");
    }
    if (fmode) {
        b->smem = float_smem_bytes(b->nmax, b->rmax, b->amax, b->hmax);
        if (n > 0 && b->smem > max_optin - 1024) {
            delete b;
            return set_error(LASSIE_ERR_TOO_LARGE, "float mode: shared memory");
        }
        b->grid = std::max(1, std::min(n, b->sm_count));
        ws_stride = ((int64_t)b->nmax * round_up4(b->nmax) * 4 + 255) / 256 * 256;
        ws_total = ws_stride * b->grid;
    } else if (b->nmax > kThreads) {
        // one network above kThreads species: the whole GPU integrates it
        if (n != 1) {
            delete b;
            return set_error(LASSIE_ERR_TOO_LARGE,
                             "networks above " + std::to_string(kThreads) +
                                 " species run one per launch (lassie_solve), not in a batch");
        }
        if (b->nmax > kWideMaxSpecies) {
            delete b;
            return set_error(LASSIE_ERR_TOO_LARGE, "networks of at most " +
                                                       std::to_string(kWideMaxSpecies) +
                                                       " species are supported");
        }
        b->wide = true;
        b->smem = wide_dynamic_smem(b->nmax, o.precision);
        if (b->smem > max_optin - 1024) {
            delete b;
            return set_error(LASSIE_ERR_TOO_LARGE, "wide engine: shared memory");
        }
        b->grid = wide_configure(o.precision, b->smem, b->sm_count);
        if (b->grid < 1) {
            delete b;
            return set_error(LASSIE_ERR_CUDA, std::string("wide engine configure: ") +
                                                  cudaGetErrorString(cudaGetLastError()));
        }
        ws_total = wide_workspace_bytes(b->nmax, b->rmax, b->amax, o.precision);
        ws_stride = ws_total;
        b->wide_flags = wide_flags_offset(b->nmax, b->rmax, b->amax, o.precision);
    } else {
        b->smem = compat_smem_bytes(b->nmax, b->rmax, b->amax, b->hmax, o.precision,
                                    o.controller);
        if (n > 0 && b->smem > max_optin - 1024) {
            delete b;
            return set_error(LASSIE_ERR_TOO_LARGE, "network needs " + std::to_string(b->smem) +
                                                       " bytes of shared memory per CTA");
        }
        b->grid = std::max(1, std::min(n, b->sm_count));
        // the mixed BDF form may fall back to an FP64 factorisation: FP64 room
        const int lt = (o.precision == LASSIE_PREC_FP64 || bdf) ? 8 : 4;
        // FP32 inverses of the 32x32 diagonal blocks after the matrix: the mixed
        // forward's solves and the adjoint's transposed solves (either form) use them
        const int64_t dinv_bytes = (int64_t)((b->nmax + 31) / 32) * 2048 * 4;
        ws_stride = ((int64_t)b->nmax * round_up4(b->nmax) * lt + dinv_bytes + 255) / 256 * 256;
        ws_total = ws_stride * b->grid;
    }
    if ((rc = b->d_int.grow(b->n_int * 4)) || (rc = b->d_dbl.grow(b->n_dbl * 8)) ||
        (rc = b->d_out.grow(b->n_out * 8)) ||
        (rc = b->d_desc.grow(std::max<size_t>(1, b->desc.size()) * sizeof(InstDesc))) ||
        (rc = b->d_order.grow(std::max<size_t>(1, b->order.size()) * 4)) ||
        (rc = b->d_res.grow(std::max<size_t>(1, b->desc.size()) * sizeof(InstResult))) ||
        (rc = b->d_queue.grow(16)) || (rc = b->d_ws.grow((size_t)ws_total))) {
        delete b;
        return rc;
    }
    b->P.ws_stride = ws_stride;
    if (!b->wide && !bdf && !fmode && n > 0) {
        // trailing-update tiles per instance: fixed by the caller or autotuned
        // per size band (LASSIE's loop; the BDF controller keeps the default)
        int band_rows[5] = {0, 0, 0, 0, 0};
        for (int q = 0; q < n; q++) {
            int rows = o.tile_rows;
            if (rows == 0) {
                const int band = tune_band(b->desc[q].n);
                if (!band_rows[band])
                    band_rows[band] =
                        tuned_tile_rows(b, o.precision, std::min(kTuneBandSize[band], b->nmax));
                rows = band_rows[band];
            }
            b->desc[q].flags |= tile_code(rows) << 4;
        }
    }
    auto cpy = [&](DevBuf &d, const void *h, size_t bytes) {
        return cudaMemcpy(d.p, h, bytes, cudaMemcpyHostToDevice);
    };
    if (cpy(b->d_int, hint.data(), hint.size() * 4) != cudaSuccess ||
        cpy(b->d_dbl, hdbl.data(), hdbl.size() * 8) != cudaSuccess ||
        (n > 0 && cpy(b->d_desc, b->desc.data(), b->desc.size() * sizeof(InstDesc)) != cudaSuccess) ||
        (n > 0 && cpy(b->d_order, b->order.data(), b->order.size() * 4) != cudaSuccess) ||
        cudaMemset(b->d_out.p, 0, b->n_out * 8) != cudaSuccess) {
        delete b;
        return set_error(LASSIE_ERR_CUDA, std::string("batch upload: ") +
                                              cudaGetErrorString(cudaGetLastError()));
    }
    if (!b->wide && (fmode ? float_configure(b->smem) : compat_configure(o.precision, b->smem)) !=
                        cudaSuccess) {
        delete b;
        return set_error(LASSIE_ERR_CUDA, std::string("kernel configure: ") +
                                              cudaGetErrorString(cudaGetLastError()));
    }
    LaunchParams &P = b->P;
    P.inst = (const InstDesc *)b->d_desc.p;
    P.n_inst = n;
    P.order = (const int32_t *)b->d_order.p;
    P.queue = (int32_t *)b->d_queue.p;
    P.iarena = (const int32_t *)b->d_int.p;
    P.darena = (const double *)b->d_dbl.p;
    P.out = (double *)b->d_out.p;
    P.res = (InstResult *)b->d_res.p;
    P.workspace = (unsigned char *)b->d_ws.p;
    P.ws_stride = ws_stride;
    P.nmax = b->nmax;
    P.rmax = b->rmax;
    P.amax = b->amax;
    P.hmax = b->hmax;
    P.precision = o.precision;
    P.refine_max = o.refine_max;
    P.lu_reuse = o.lu_reuse;
    P.tensor_cores = o.tensor_cores;
    P.deadline_ns = o.deadline_s > 0 ? (uint64_t)(o.deadline_s * 1e9) : 0;
    P.controller = o.controller;
    P.max_order = o.max_order;
    P.rtol = o.rtol;
    P.atol = o.atol;
    P.first_step = o.first_step;
    P.max_step = o.max_step;
    *out = b;
    return LASSIE_OK;
}

extern "C" int lassie_batch_run(lassie_batch *b, void *stream) {
    if (!b) return set_error(LASSIE_ERR_ARGS, "null batch");
    if (b->n == 0) return LASSIE_OK;
    b->stream = (cudaStream_t)stream;
    CU(cudaMemsetAsync(b->d_queue.p, 0, 16, b->stream));
    if (b->wide) {
        // control block and pivot-order flag start at zero
        CU(cudaMemsetAsync(b->d_ws.p, 0, 256, b->stream));
        CU(cudaMemsetAsync((unsigned char *)b->d_ws.p + b->wide_flags, 0, 16, b->stream));
        CU(wide_launch(b->P, b->grid, b->smem, b->stream));
    } else if (b->opts.precision == LASSIE_PREC_FLOAT) {
        CU(float_launch(b->P, b->grid, b->smem, b->stream));
    } else {
        CU(compat_launch(b->P, b->grid, b->smem, b->stream));
    }
    return LASSIE_OK;
}

extern "C" int lassie_batch_launches(const lassie_batch *b) { return (b && b->n > 0) ? 1 : 0; }

// Longest-processing-time order for the persistent work queue: the last
// run's whole-integration cycles per instance, longest first (ties keep the
// current order, largest network first at creation).  Each CTA integrates
// its instance alone, so the order changes no result.
extern "C" int lassie_batch_order_by_cost(lassie_batch *b) {
    if (!b) return set_error(LASSIE_ERR_ARGS, "null batch");
    if (b->n <= 1 || b->wide) return LASSIE_OK;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CU(cudaStreamIsCapturing(b->stream, &cap));
    if (cap != cudaStreamCaptureStatusNone)
        return set_error(LASSIE_ERR_ARGS, "lassie_batch_order_by_cost: stream is being captured");
    std::vector<InstResult> hres(b->n);
    CU(cudaMemcpyAsync(hres.data(), b->d_res.p, hres.size() * sizeof(InstResult),
                       cudaMemcpyDeviceToHost, b->stream));
    CU(cudaStreamSynchronize(b->stream));
    bool measured = false;
    for (const InstResult &r : hres) measured = measured || r.cycles_total > 0;
    if (!measured) return LASSIE_OK;  // no run yet
    std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int c) {
        return hres[a].cycles_total > hres[c].cycles_total;
    });
    CU(cudaMemcpyAsync(b->d_order.p, b->order.data(), b->order.size() * 4, cudaMemcpyHostToDevice,
                       b->stream));
    CU(cudaStreamSynchronize(b->stream));
    return LASSIE_OK;
}

extern "C" int lassie_batch_bytes(const lassie_batch *b, int64_t *h2d, int64_t *d2h) {
    if (!b) return set_error(LASSIE_ERR_ARGS, "null batch");
    if (h2d)
        *h2d = b->n_int * 4 + b->n_dbl * 8 + (int64_t)b->desc.size() * sizeof(InstDesc) +
               (int64_t)b->order.size() * 4;
    if (d2h) *d2h = b->n_out * 8 + (int64_t)b->n * sizeof(InstResult);
    return LASSIE_OK;
}

extern "C" int lassie_batch_sync(lassie_batch *b) {
    if (!b) return set_error(LASSIE_ERR_ARGS, "null batch");
    CU(cudaStreamSynchronize(b->stream));
    return LASSIE_OK;
}

extern "C" int lassie_batch_read(lassie_batch *b, const lassie_instance *inst,
                                 lassie_stats *stats) {
    if (!b) return set_error(LASSIE_ERR_ARGS, "null batch");
    if (b->n == 0) return LASSIE_OK;
    std::vector<double> hout((size_t)b->n_out);
    std::vector<InstResult> hres(b->n);
    CU(cudaMemcpyAsync(hout.data(), b->d_out.p, hout.size() * 8, cudaMemcpyDeviceToHost,
                       b->stream));
    CU(cudaMemcpyAsync(hres.data(), b->d_res.p, hres.size() * sizeof(InstResult),
                       cudaMemcpyDeviceToHost, b->stream));
    CU(cudaStreamSynchronize(b->stream));
    int first_bad = LASSIE_OK;
    for (int q = 0; q < b->n; q++) {
        const InstDesc &D = b->desc[q];
        if (inst && inst[q].out)
            std::memcpy(inst[q].out, hout.data() + D.out, sizeof(double) * (size_t)D.nt * D.ncs);
        if (stats) std::memcpy(&stats[q], &hres[q], sizeof(lassie_stats));
        if (hres[q].status != LASSIE_OK && first_bad == LASSIE_OK) first_bad = hres[q].status;
    }
    return first_bad;
}

extern "C" void lassie_batch_destroy(lassie_batch *b) { delete b; }

extern "C" int lassie_solve_batch(const lassie_instance *inst, int32_t n, const lassie_opts *opts,
                                  lassie_stats *stats) {
    lassie_batch *b = nullptr;
    int rc = lassie_batch_create(inst, n, opts, &b);
    if (rc) return rc;
    rc = lassie_batch_run(b, nullptr);
    if (!rc) rc = lassie_batch_sync(b);
    if (!rc) rc = lassie_batch_read(b, inst, stats);
    lassie_batch_destroy(b);
    return rc;
}

extern "C" int lassie_solve(const lassie_model *model, const double *k, const double *x0,
                            const double *feed, const double *atol, const double *t, int32_t nt,
                            const int32_t *cs, int32_t ncs, const lassie_opts *opts, double *out,
                            lassie_stats *stats) {
    lassie_instance I;
    I.model = model;
    I.k = k;
    I.x0 = x0;
    I.feed = feed;
    I.atol = atol;
    I.t = t;
    I.nt = nt;
    I.ncs = ncs;
    I.cs = cs;
    I.out = out;
    return lassie_solve_batch(&I, 1, opts, stats);
}

// --------------------------------------------------------------- adjoint

extern "C" int lassie_adjoint_batch(const lassie_instance *inst, int32_t n,
                                    const double *const *targets, const lassie_opts *opts,
                                    int32_t ckpt_every, int32_t max_record, double *loss,
                                    double *const *grad_logk, double *const *grad_x0,
                                    lassie_stats *stats) {
    if (n < 0 || (n > 0 && (!inst || !targets || !grad_logk)))
        return set_error(LASSIE_ERR_ARGS, "adjoint_batch");
    if (n == 0) return LASSIE_OK;
    lassie_opts o;
    if (opts) o = *opts;
    else lassie_opts_default(&o);
    // the recorded forward and its reverse are LASSIE's loop
    if (o.controller != LASSIE_CTRL_COMPAT)
        return set_error(LASSIE_ERR_ARGS, "adjoint_batch: LASSIE's controller only");
    if (o.precision == LASSIE_PREC_FLOAT)
        return set_error(LASSIE_ERR_ARGS, "adjoint_batch: the float mode has no adjoint");
    const int K = ckpt_every > 0 ? ckpt_every : 8;
    const int cap = max_record > 0 ? max_record : 100000;
    lassie_batch *b = nullptr;
    int rc = lassie_batch_create(inst, n, &o, &b);
    if (rc) return rc;
    // per-instance record layout
    std::vector<AdjDesc> ad(n);
    int64_t rec = 0, st = 0, samp = 0, grad = 0;
    for (int q = 0; q < n; q++) {
        const InstDesc &D = b->desc[q];
        ad[q].rec = rec;
        ad[q].states = st;
        ad[q].samp = samp;
        ad[q].grad = grad;
        ad[q].cap_steps = cap;
        ad[q].cap_states = cap + 1;
        rec += cap;
        st += (int64_t)(cap + 1) * D.n;
        samp += D.nt;
        grad += D.r + D.n;
    }
    if (st * 8 > (int64_t)64 << 30) {
        lassie_batch_destroy(b);
        return set_error(LASSIE_ERR_TOO_LARGE, "adjoint record needs more than 64 GiB");
    }
    std::vector<double> htarget((size_t)b->n_out, 0.0);
    for (int q = 0; q < n; q++) {
        const InstDesc &D = b->desc[q];
        if (!targets[q]) {
            lassie_batch_destroy(b);
            return set_error(LASSIE_ERR_ARGS, "adjoint_batch: missing target");
        }
        std::memcpy(htarget.data() + D.out, targets[q], sizeof(double) * (size_t)D.nt * D.ncs);
    }
    DevBuf d_ad, d_kind, d_dt, d_slot, d_states, d_nsteps, d_samp, d_target, d_grad, d_scratch;
    const int64_t scratch_stride = (int64_t)(K + 1) * b->nmax;
    auto cleanup = [&]() {
        d_ad.release(); d_kind.release(); d_dt.release(); d_slot.release(); d_states.release();
        d_nsteps.release(); d_samp.release(); d_target.release(); d_grad.release();
        d_scratch.release();
        lassie_batch_destroy(b);
    };
    if ((rc = d_ad.grow(sizeof(AdjDesc) * n)) || (rc = d_kind.grow(rec * 4)) ||
        (rc = d_dt.grow(rec * 8)) || (rc = d_slot.grow(rec * 4)) || (rc = d_states.grow(st * 8)) ||
        (rc = d_nsteps.grow(4 * n)) || (rc = d_samp.grow(std::max<int64_t>(samp, 1) * 4)) ||
        (rc = d_target.grow(htarget.size() * 8)) || (rc = d_grad.grow(grad * 8)) ||
        (rc = d_scratch.grow((size_t)scratch_stride * 8 * b->grid))) {
        cleanup();
        return rc;
    }
    if (cudaMemcpy(d_ad.p, ad.data(), sizeof(AdjDesc) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d_target.p, htarget.data(), htarget.size() * 8, cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemset(d_nsteps.p, 0, 4 * n) != cudaSuccess ||
        cudaMemset(d_samp.p, 0, std::max<int64_t>(samp, 1) * 4) != cudaSuccess) {
        cleanup();
        return set_error(LASSIE_ERR_CUDA, "adjoint upload");
    }
    AdjArrays &A = b->P.adj;
    A.desc = (const AdjDesc *)d_ad.p;
    A.rec_kind = (int32_t *)d_kind.p;
    A.rec_dt = (double *)d_dt.p;
    A.rec_slot = (int32_t *)d_slot.p;
    A.states = (double *)d_states.p;
    A.nsteps = (int32_t *)d_nsteps.p;
    A.samp_step = (int32_t *)d_samp.p;
    A.target = (const double *)d_target.p;
    A.grad = (double *)d_grad.p;
    A.scratch = (double *)d_scratch.p;
    A.scratch_stride = scratch_stride;
    A.ckpt_every = K;
    // forward with recording
    rc = lassie_batch_run(b, nullptr);
    if (!rc) rc = lassie_batch_sync(b);
    std::vector<lassie_stats> hst(n);
    if (!rc) rc = lassie_batch_read(b, inst, hst.data());
    if (stats) std::memcpy(stats, hst.data(), sizeof(lassie_stats) * n);
    if (rc) {
        cleanup();
        return rc;
    }
    for (int q = 0; q < n; q++) {
        const InstDesc &D = b->desc[q];
        double L = 0.0;
        for (int64_t i = 0; i < (int64_t)D.nt * D.ncs; i++) {
            const double d = inst[q].out[i] - targets[q][i];
            L += d * d;
        }
        if (loss) loss[q] = L;
    }
    // backward
    const int64_t smem = adjoint_smem_bytes(b->nmax, b->rmax, b->amax, b->hmax);
    int max_optin = 0;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->dev);
    if (smem > max_optin - 1024) {
        cleanup();
        return set_error(LASSIE_ERR_TOO_LARGE, "adjoint shared memory");
    }
    if (cudaMemset(b->d_queue.p, 0, 16) != cudaSuccess ||
        adjoint_launch(b->P, b->grid, smem, nullptr) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess) {
        std::string msg = cudaGetErrorString(cudaGetLastError());
        cleanup();
        return set_error(LASSIE_ERR_CUDA, "adjoint kernel: " + msg);
    }
    std::vector<double> hgrad(grad);
    if (cudaMemcpy(hgrad.data(), d_grad.p, grad * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cleanup();
        return set_error(LASSIE_ERR_CUDA, "adjoint download");
    }
    for (int q = 0; q < n; q++) {
        const InstDesc &D = b->desc[q];
        std::memcpy(grad_logk[q], hgrad.data() + ad[q].grad, sizeof(double) * D.r);
        if (grad_x0 && grad_x0[q])
            std::memcpy(grad_x0[q], hgrad.data() + ad[q].grad + D.r, sizeof(double) * D.n);
    }
    cleanup();
    return LASSIE_OK;
}

// ---------------------------------------------------- single evaluations

// Work order of the batched RHS: reactions by their number of reactants,
// species by the work of their sums (an entry of coefficient +-1 is one
// addition, any other a product over the reaction's reactants), both
// descending and stable, so that the lanes of a warp run loops of equal
// length.  [reactions R | species N], uploaded once per model.
static int model_order_device(lassie_model *m, const int32_t **d) {
    std::lock_guard<std::mutex> g(m->mu);
    if (m->d_order) {
        *d = m->d_order;
        return LASSIE_OK;
    }
    std::vector<int32_t> rord(m->R), sord(m->N);
    std::vector<int64_t> rw(m->R), sw(m->N, 0);
    for (int y = 0; y < m->R; y++) rw[y] = m->rxn_ptr[y + 1] - m->rxn_ptr[y];
    for (int s = 0; s < m->N; s++)
        for (int e = m->sp_ptr[s]; e < m->sp_ptr[s + 1]; e++) {
            const int c = ent_coef(m->sp_ent[e]);
            sw[s] += (c == 1 || c == -1) ? 1 : 2 + rw[ent_index(m->sp_ent[e])];
        }
    std::iota(rord.begin(), rord.end(), 0);
    std::iota(sord.begin(), sord.end(), 0);
    std::stable_sort(rord.begin(), rord.end(), [&](int a, int b) { return rw[a] > rw[b]; });
    std::stable_sort(sord.begin(), sord.end(), [&](int a, int b) { return sw[a] > sw[b]; });
    rord.insert(rord.end(), sord.begin(), sord.end());
    int dev = 0;
    CU(cudaGetDevice(&dev));
    if (m->d_struct && m->dev != dev)
        return set_error(LASSIE_ERR_ARGS, "model already bound to another device");
    CU(cudaMalloc(&m->d_order, rord.size() * sizeof(int32_t)));
    CU(cudaMemcpy(m->d_order, rord.data(), rord.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    *d = m->d_order;
    return LASSIE_OK;
}

extern "C" int lassie_rhs_device(const lassie_model *cm, int32_t n_inst, const double *k,
                                 const double *x, double *dx, void *stream) {
    lassie_model *m = const_cast<lassie_model *>(cm);
    if (!m || n_inst < 0 || (n_inst > 0 && (!k || !x || !dx)))
        return set_error(LASSIE_ERR_ARGS, "rhs_device");
    if (n_inst == 0) return LASSIE_OK;
    const int32_t *d = nullptr, *dord = nullptr;
    int rc = model_device(m, &d);
    if (!rc) rc = model_order_device(m, &dord);
    if (rc) return rc;
    int dev = 0, sms = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CU(rhs_batch_launch(n_inst, m->N, m->R, (int)m->rxn_ent.size(), (int)m->sp_ent.size(), d,
                        d + m->off_rent(), d + m->off_sptr(), d + m->off_sent(), dord, k, x, dx,
                        sms, (cudaStream_t)stream));
    return LASSIE_OK;
}

extern "C" int lassie_rhs(const lassie_model *m, const double *k, const double *x, double *dx) {
    if (!m || !k || !x || !dx) return set_error(LASSIE_ERR_ARGS, "rhs");
    double *dk = nullptr, *dxv = nullptr, *ddx = nullptr;
    CU(cudaMalloc(&dk, sizeof(double) * m->R));
    CU(cudaMalloc(&dxv, sizeof(double) * m->N));
    CU(cudaMalloc(&ddx, sizeof(double) * m->N));
    int rc = LASSIE_OK;
    if (cudaMemcpy(dk, k, sizeof(double) * m->R, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dxv, x, sizeof(double) * m->N, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = set_error(LASSIE_ERR_CUDA, "rhs upload");
    if (!rc) rc = lassie_rhs_device(m, 1, dk, dxv, ddx, nullptr);
    if (!rc && cudaMemcpy(dx, ddx, sizeof(double) * m->N, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = set_error(LASSIE_ERR_CUDA, "rhs download");
    cudaFree(dk);
    cudaFree(dxv);
    cudaFree(ddx);
    return rc;
}

extern "C" int lassie_newton_matrix(const lassie_model *cm, const double *k, const double *x,
                                    double h, double *M) {
    lassie_model *m = const_cast<lassie_model *>(cm);
    if (!m || !k || !x || !M) return set_error(LASSIE_ERR_ARGS, "newton_matrix");
    const int32_t *d = nullptr;
    int rc = model_device(m, &d);
    if (rc) return rc;
    const size_t nn = (size_t)m->N * m->N;
    double *dk = nullptr, *dxv = nullptr, *dM = nullptr;
    CU(cudaMalloc(&dk, sizeof(double) * m->R));
    CU(cudaMalloc(&dxv, sizeof(double) * m->N));
    CU(cudaMalloc(&dM, sizeof(double) * nn));
    if (cudaMemcpy(dk, k, sizeof(double) * m->R, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dxv, x, sizeof(double) * m->N, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = set_error(LASSIE_ERR_CUDA, "newton_matrix upload");
    cudaError_t e = cudaSuccess;
    if (!rc)
        e = newton_matrix_launch(m->N, m->R, (int)m->rxn_ent.size(), d, d + m->off_rent(),
                                 d + m->off_sptr(), d + m->off_sent(), dk, dxv, h, dM, nullptr);
    if (!rc && e != cudaSuccess) rc = set_error(LASSIE_ERR_CUDA, cudaGetErrorString(e));
    if (!rc && cudaMemcpy(M, dM, sizeof(double) * nn, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = set_error(LASSIE_ERR_CUDA, "newton_matrix download");
    cudaFree(dk);
    cudaFree(dxv);
    cudaFree(dM);
    return rc;
}

// Structural nonzeros of J: column g is in row i when some reaction with net
// stoichiometry in species i has g among its reactants (the entries
// createJac fills, kernels.cuh:219-271).  Per row the columns ascend; per
// nonzero (i,g) the terms are the reactions of row i, in ascending order,
// that have g among their reactants: (make_ent(reaction, net coefficient),
// coefficient of g).  Layout [jptr N+1 | jcol | jrow | tptr nnz+1 | pad to
// 8 bytes | terms as int pairs], uploaded once per model.
static int model_jac_device(lassie_model *m, const int32_t **d) {
    std::lock_guard<std::mutex> g(m->mu);
    if (m->d_jac) {
        *d = m->d_jac;
        return LASSIE_OK;
    }
    const int N = m->N;
    std::vector<int32_t> ptr(N + 1), col, row, tptr, tent;
    std::vector<int32_t> mark(N, -1);
    for (int i = 0; i < N; i++) {
        ptr[i] = (int32_t)col.size();
        const size_t first = col.size();
        for (int e = m->sp_ptr[i]; e < m->sp_ptr[i + 1]; e++) {
            const int y = ent_index(m->sp_ent[e]);
            for (int q = m->rxn_ptr[y]; q < m->rxn_ptr[y + 1]; q++) {
                const int gcol = ent_index(m->rxn_ent[q]);
                if (mark[gcol] != i) {
                    mark[gcol] = i;
                    col.push_back(gcol);
                }
            }
        }
        std::sort(col.begin() + first, col.end());
        for (size_t p = first; p < col.size(); p++) {
            row.push_back(i);
            tptr.push_back((int32_t)(tent.size() / 2));
            for (int e = m->sp_ptr[i]; e < m->sp_ptr[i + 1]; e++) {
                const int y = ent_index(m->sp_ent[e]);
                for (int q = m->rxn_ptr[y]; q < m->rxn_ptr[y + 1]; q++) {
                    if (ent_index(m->rxn_ent[q]) != col[p]) continue;
                    const int a = ent_coef(m->rxn_ent[q]);
                    if (a > 0) {
                        tent.push_back(m->sp_ent[e]);
                        tent.push_back(a);
                    }
                    break;
                }
            }
        }
    }
    ptr[N] = (int32_t)col.size();
    tptr.push_back((int32_t)(tent.size() / 2));
    std::vector<int32_t> h(ptr);
    h.insert(h.end(), col.begin(), col.end());
    h.insert(h.end(), row.begin(), row.end());
    h.insert(h.end(), tptr.begin(), tptr.end());
    if (h.size() & 1) h.push_back(0);
    h.insert(h.end(), tent.begin(), tent.end());
    int dev = 0;
    CU(cudaGetDevice(&dev));
    if (m->d_struct && m->dev != dev)
        return set_error(LASSIE_ERR_ARGS, "model already bound to another device");
    CU(cudaMalloc(&m->d_jac, h.size() * sizeof(int32_t)));
    CU(cudaMemcpy(m->d_jac, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    m->jac_nnz = (int64_t)col.size();
    *d = m->d_jac;
    return LASSIE_OK;
}

extern "C" int lassie_newton_matrix_device(const lassie_model *cm, int32_t n_inst, double h,
                                           const double *k, const double *x, void *M,
                                           int32_t precision, void *stream) {
    lassie_model *m = const_cast<lassie_model *>(cm);
    if (!m || n_inst < 0 || (n_inst > 0 && (!k || !x || !M)) ||
        (precision != LASSIE_PREC_FP64 && precision != LASSIE_PREC_MIXED))
        return set_error(LASSIE_ERR_ARGS, "newton_matrix_device");
    if (int64_t(m->N + m->R) * 8 > 160 * 1024)
        return set_error(LASSIE_ERR_TOO_LARGE, "newton_matrix_device: N + R above 20480");
    if (n_inst == 0) return LASSIE_OK;
    const int32_t *d = nullptr, *dj = nullptr;
    int rc = model_device(m, &d);
    if (!rc) rc = model_jac_device(m, &dj);
    if (rc) return rc;
    int dev = 0, sms = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CU(newton_batch_launch(n_inst, m->N, m->R, d, d + m->off_rent(), dj, m->jac_nnz, k, x, h, M,
                           precision == LASSIE_PREC_MIXED, sms, (cudaStream_t)stream));
    return LASSIE_OK;
}

// Host-only: column g is in row i when a reaction with net stoichiometry in
// species i has g among its reactants; columns ascending per row.
static void jac_pattern_host(const lassie_model *m, std::vector<int32_t> &ptr,
                             std::vector<int32_t> &col) {
    ptr.assign(m->N + 1, 0);
    col.clear();
    std::vector<int32_t> mark(m->N, -1);
    for (int i = 0; i < m->N; i++) {
        ptr[i] = (int32_t)col.size();
        const size_t first = col.size();
        for (int e = m->sp_ptr[i]; e < m->sp_ptr[i + 1]; e++) {
            const int y = ent_index(m->sp_ent[e]);
            for (int q = m->rxn_ptr[y]; q < m->rxn_ptr[y + 1]; q++) {
                const int g = ent_index(m->rxn_ent[q]);
                if (mark[g] != i) {
                    mark[g] = i;
                    col.push_back(g);
                }
            }
        }
        std::sort(col.begin() + first, col.end());
    }
    ptr[m->N] = (int32_t)col.size();
}

extern "C" int lassie_jacobian_nnz(const lassie_model *m, int64_t *nnz) {
    if (!m || !nnz) return set_error(LASSIE_ERR_ARGS, "jacobian_nnz");
    std::vector<int32_t> ptr, col;
    jac_pattern_host(m, ptr, col);
    *nnz = (int64_t)col.size();
    return LASSIE_OK;
}

extern "C" int lassie_jacobian_pattern(const lassie_model *m, int32_t *row_ptr, int32_t *cols) {
    if (!m || !row_ptr || !cols) return set_error(LASSIE_ERR_ARGS, "jacobian_pattern");
    std::vector<int32_t> ptr, col;
    jac_pattern_host(m, ptr, col);
    std::memcpy(row_ptr, ptr.data(), ptr.size() * sizeof(int32_t));
    if (!col.empty()) std::memcpy(cols, col.data(), col.size() * sizeof(int32_t));
    return LASSIE_OK;
}

extern "C" int lassie_lu_solve(int32_t n, const double *a, const double *b, double *x,
                               int32_t precision) {
    if (n <= 0 || !a || !b || !x ||
        (precision != LASSIE_PREC_FP64 && precision != LASSIE_PREC_MIXED))
        return set_error(LASSIE_ERR_ARGS, "lu_solve");
    int dev = 0, max_optin = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (n > kThreads || lu_solve_smem(n, precision) > max_optin - 1024)
        return set_error(LASSIE_ERR_TOO_LARGE, "lu_solve: n too large for one CTA");
    const int ld = round_up4(n);
    const int lt = precision == LASSIE_PREC_FP64 ? 8 : 4;
    const size_t dinv_bytes = lt == 4 ? (size_t)((n + 31) / 32) * 2048 * 4 : 0;
    std::vector<unsigned char> h((size_t)n * ld * lt + dinv_bytes, 0);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const double v = a[(size_t)i * n + j];
            if (lt == 8) ((double *)h.data())[(size_t)i * ld + j] = v;
            else ((float *)h.data())[(size_t)i * ld + j] = (float)v;
        }
    void *dA = nullptr;
    double *db = nullptr, *dx = nullptr;
    int *dinfo = nullptr;
    CU(cudaMalloc(&dA, h.size()));
    CU(cudaMalloc(&db, sizeof(double) * n));
    CU(cudaMalloc(&dx, sizeof(double) * n));
    CU(cudaMalloc(&dinfo, sizeof(int)));
    int rc = LASSIE_OK, info = 0;
    if (cudaMemcpy(dA, h.data(), h.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(db, b, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = set_error(LASSIE_ERR_CUDA, "lu_solve upload");
    cudaError_t e = cudaSuccess;
    if (!rc) e = lu_solve_launch(n, dA, ld, db, dx, dinfo, precision, nullptr);
    if (!rc && e != cudaSuccess) rc = set_error(LASSIE_ERR_CUDA, cudaGetErrorString(e));
    if (!rc && (cudaMemcpy(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = set_error(LASSIE_ERR_CUDA, "lu_solve download");
    cudaFree(dA);
    cudaFree(db);
    cudaFree(dx);
    cudaFree(dinfo);
    if (!rc && info) return info;
    return rc;
}
