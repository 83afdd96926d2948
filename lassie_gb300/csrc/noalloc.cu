// lassie_solve_noalloc: one integration without any device allocation.
//
// Some callers cannot call cudaMalloc: a host that runs inside another
// framework's memory pool (which owns all device memory and forbids outside
// allocations), a plugin whose process forbids driver allocations after
// start-up, a real-time loop that must not block on the allocator.  This
// entry point gives them the integrator with all of its working memory in
// one fixed arena compiled into the library: a file-scope static __device__
// array of LASSIE_NOALLOC_ARENA_BYTES bytes that every device which loads the
// library holds until the process exits.  The caller passes device buffers
// for the inputs (k, x0, t) and for the trajectory; the network structure,
// the instance descriptor, the Newton matrix, the diagonal-block inverses,
// the work-queue counter and the per-instance result all live in the arena.
//
// Set-up: the first call on a device takes the arena's device address with
// cudaGetSymbolAddress (host code must not use the array's name as an
// address: it is a host-side stand-in) and keeps it for that device; make
// that first call before any stream capture.  The kept address does not
// survive a cudaDeviceReset of that device.  Every call shares the arena,
// which keeps the previous call's contents: the work-queue counter and the
// result are cleared on each call, everything else is overwritten.  Calls
// that overlap on the GPU (two host threads, or two streams) race on the
// arena: serialise them.  A call synchronises its stream before it returns,
// so it refuses (LASSIE_ERR_ARGS) a stream that is being captured.
#include <cstdint>
#include <cstring>
#include <mutex>
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
int model_pack_for_noalloc(const lassie_model *m, std::vector<int32_t> &out, int32_t *n,
                           int32_t *r, int32_t *nnz_a, int32_t *nnz_h, int64_t offs[8]);
int set_error_noalloc(int status, const char *msg);
}  // namespace lassie

using namespace lassie;

static __device__ __align__(256) unsigned char g_noalloc_arena[LASSIE_NOALLOC_ARENA_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_arena_ptr[kMaxDevices] = {};

// Device address of the arena on the current device (set-up on first use).
int arena_address(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return set_error_noalloc(LASSIE_ERR_NO_DEVICE, "noalloc: no current CUDA device");
    }
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_arena_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_arena);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return set_error_noalloc(LASSIE_ERR_CUDA, "noalloc: cudaGetSymbolAddress failed");
        }
        g_arena_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_arena_ptr[dev];
    return LASSIE_OK;
}

int64_t up256(int64_t v) { return (v + 255) & ~int64_t(255); }

}  // namespace

extern "C" int lassie_solve_noalloc(const lassie_model *model, const double *d_k,
                                    const double *d_x0, const double *d_t, int32_t nt,
                                    const lassie_opts *opts, double *d_out, lassie_stats *stats,
                                    void *stream) {
    if (!model || !d_k || !d_x0 || nt < 0 || (nt > 0 && (!d_t || !d_out)))
        return set_error_noalloc(LASSIE_ERR_ARGS, "noalloc: missing buffer");
    lassie_opts o;
    if (opts) o = *opts;
    else lassie_opts_default(&o);
    if (o.precision != LASSIE_PREC_FP64 && o.precision != LASSIE_PREC_MIXED)
        return set_error_noalloc(LASSIE_ERR_ARGS, "noalloc: precision");
    if (o.controller != LASSIE_CTRL_COMPAT)
        return set_error_noalloc(LASSIE_ERR_ARGS, "noalloc: LASSIE's controller only");
    {
        // the call ends with a synchronisation of the stream, which would
        // invalidate a capture in progress
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap) != cudaSuccess) {
            cudaGetLastError();
            return set_error_noalloc(LASSIE_ERR_CUDA, "noalloc: cudaStreamIsCapturing failed");
        }
        if (cap != cudaStreamCaptureStatusNone)
            return set_error_noalloc(LASSIE_ERR_ARGS,
                                     "noalloc: the stream is being captured; this call "
                                     "synchronises its stream and cannot run inside a capture");
    }
    std::vector<int32_t> ints;
    int32_t N = 0, R = 0, na = 0, nh = 0;
    int64_t offs[8];
    int rc = model_pack_for_noalloc(model, ints, &N, &R, &na, &nh, offs);
    if (rc) return rc;
    if (N > LASSIE_NOALLOC_MAX_SPECIES || R > LASSIE_NOALLOC_MAX_REACTIONS ||
        nt > LASSIE_NOALLOC_MAX_SAMPLES)
        return set_error_noalloc(LASSIE_ERR_TOO_LARGE,
                                 "noalloc: the network or the sampling exceeds the arena limits "
                                 "(species <= 128, reactions <= 256, samples <= 4096)");
    // arena layout (bytes): descriptor | result | queue + order | ints |
    // doubles (k, x0, t) | Newton workspace
    const int lt = o.precision == LASSIE_PREC_FP64 ? 8 : 4;
    const int ld = round_up4(N);
    const int64_t ws = up256((int64_t)N * ld * lt +
                             (o.precision == LASSIE_PREC_MIXED ? (int64_t)((N + 31) / 32) * 2048 * 4
                                                               : 0));
    const int64_t off_desc = 0;
    const int64_t off_res = up256(off_desc + (int64_t)sizeof(InstDesc));
    const int64_t off_queue = up256(off_res + (int64_t)sizeof(InstResult));
    const int64_t off_ints = up256(off_queue + 16);
    const int64_t off_dbl = up256(off_ints + (int64_t)ints.size() * 4);
    const int64_t n_dbl = (int64_t)R + N + nt;
    const int64_t off_ws = up256(off_dbl + n_dbl * 8);
    const int64_t total = off_ws + ws;
    if (total > LASSIE_NOALLOC_ARENA_BYTES)
        return set_error_noalloc(LASSIE_ERR_TOO_LARGE, "noalloc: arena too small for this network");
    const int64_t smem = compat_smem_bytes(N, R, na, nh, o.precision, LASSIE_CTRL_COMPAT);
    int dev = 0, max_optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess) {
        cudaGetLastError();
        return set_error_noalloc(LASSIE_ERR_NO_DEVICE, "noalloc: device query failed");
    }
    if (smem > max_optin - 1024) return set_error_noalloc(LASSIE_ERR_TOO_LARGE, "noalloc: smem");

    unsigned char *A = nullptr;
    rc = arena_address(&A);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    InstDesc D{};
    D.n = N;
    D.r = R;
    D.nt = nt;
    D.ncs = N;
    D.nnz_a = na;
    D.nnz_h = nh;
    D.rxn_ptr = offs[0];
    D.rxn_ent = offs[1];
    D.sp_ptr = offs[2];
    D.sp_ent = offs[3];
    D.hr_ptr = offs[4];
    D.hr_ent = offs[5];
    D.as_ptr = offs[6];
    D.as_ent = offs[7];
    D.cs = -1;
    D.k = 0;
    D.x0 = R;
    D.feed = -1;
    D.atol = -1;
    D.t = R + N;
    D.out = 0;
    D.rkf_step = o.rkf_step;
    D.be_step = o.be_step;
    D.newton_tol = o.newton_tol;
    D.stiffness_tol = o.stiffness_tol;
    D.newton_iter = o.newton_iter;
    D.max_steps = o.max_steps;
    D.flags = o.quarter_root == LASSIE_ROOT_SQRT ? 1 : 0;
    double *dbl = reinterpret_cast<double *>(A + off_dbl);
    // inputs into the arena (device-to-device and from the host; no allocation)
    if (cudaMemcpyAsync(A + off_desc, &D, sizeof(D), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(A + off_res, 0, sizeof(InstResult), s) != cudaSuccess ||
        cudaMemsetAsync(A + off_queue, 0, 16, s) != cudaSuccess ||
        cudaMemcpyAsync(A + off_ints, ints.data(), ints.size() * 4, cudaMemcpyHostToDevice, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(dbl, d_k, sizeof(double) * R, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(dbl + R, d_x0, sizeof(double) * N, cudaMemcpyDeviceToDevice, s) !=
            cudaSuccess ||
        (nt > 0 && cudaMemcpyAsync(dbl + R + N, d_t, sizeof(double) * nt,
                                   cudaMemcpyDeviceToDevice, s) != cudaSuccess)) {
        const std::string msg = cudaGetErrorString(cudaGetLastError());
        return set_error_noalloc(LASSIE_ERR_CUDA, ("noalloc: arena upload: " + msg).c_str());
    }
    LaunchParams P{};
    P.inst = reinterpret_cast<const InstDesc *>(A + off_desc);
    P.n_inst = 1;
    // order[0] = 0: the second int of the queue block
    P.queue = reinterpret_cast<int32_t *>(A + off_queue);
    P.order = reinterpret_cast<const int32_t *>(A + off_queue) + 1;
    P.iarena = reinterpret_cast<const int32_t *>(A + off_ints);
    P.darena = dbl;
    P.out = d_out;
    P.res = reinterpret_cast<InstResult *>(A + off_res);
    P.workspace = A + off_ws;
    P.ws_stride = ws;
    P.nmax = N;
    P.rmax = R;
    P.amax = na;
    P.hmax = nh;
    P.precision = o.precision;
    P.refine_max = o.refine_max;
    P.lu_reuse = o.lu_reuse;
    P.deadline_ns = o.deadline_s > 0 ? (uint64_t)(o.deadline_s * 1e9) : 0;
    if (compat_configure(o.precision, smem) != cudaSuccess ||
        compat_launch(P, 1, smem, s) != cudaSuccess) {
        const std::string msg = cudaGetErrorString(cudaGetLastError());
        return set_error_noalloc(LASSIE_ERR_CUDA, ("noalloc: launch: " + msg).c_str());
    }
    InstResult res{};
    if (cudaMemcpyAsync(&res, P.res, sizeof(res), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        const std::string msg = cudaGetErrorString(cudaGetLastError());
        return set_error_noalloc(LASSIE_ERR_CUDA, ("noalloc: " + msg).c_str());
    }
    if (stats) std::memcpy(stats, &res, sizeof(res));
    return res.status;
}
