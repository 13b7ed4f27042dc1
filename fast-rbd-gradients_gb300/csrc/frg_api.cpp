// C ABI of the engine (include/frg.h): contexts, the plain / host / batched
// calls, plans, and the launch-shape autotuner.
#include "frg.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "frg_internal.h"
#include "frg_kernels.cuh"
#include "frg_model_select.h"

using frg::LaunchShape;
using frg::Segment;

namespace {

thread_local std::string g_orphan_error;  // errors of calls without a context

bool check(frg_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    frg_set_error(ctx, std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

bool valid_traj(const frg_traj &t) {
    if (t.n_knots < 0) return false;
    if (t.n_knots == 0) return true;
    return t.q && t.qd && t.u && t.dqdd && t.qdd && t.minv;
}

}  // namespace

void frg_set_error(frg_ctx *ctx, const std::string &msg) {
    if (ctx) ctx->err = msg;
    else g_orphan_error = msg;
}

// ----------------------------------------------------------- batch lists ---

bool frg_build_batch(int n_traj, const frg_traj *trajs, HostBatch &hb, std::string &err) {
    hb.segs.clear();
    hb.tile_seg.clear();
    hb.segs.reserve(static_cast<size_t>(n_traj) + 1);
    long long begin = 0;
    for (int t = 0; t < n_traj; t++) {
        const frg_traj &tr = trajs[t];
        if (!valid_traj(tr)) {
            err = "trajectory " + std::to_string(t) + ": negative length or null pointer";
            return false;
        }
        hb.segs.push_back(Segment{tr.q, tr.qd, tr.u, tr.dqdd, tr.qdd, tr.minv, begin});
        begin += tr.n_knots;
    }
    hb.segs.push_back(Segment{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, begin});
    hb.nknots = begin;
    // contiguous: each non-empty trajectory starts where the previous one ended
    hb.contiguous = begin > 0 && begin <= INT_MAX;
    const frg_traj *prev = nullptr;
    for (int t = 0; t < n_traj && hb.contiguous; t++) {
        const frg_traj &tr = trajs[t];
        if (tr.n_knots == 0) continue;
        if (prev) {
            const int64_t m = prev->n_knots;
            using frg::kN;
            hb.contiguous = tr.q == prev->q + kN * m && tr.qd == prev->qd + kN * m && tr.u == prev->u + kN * m &&
                            tr.dqdd == prev->dqdd + frg::kDqddN * m && tr.qdd == prev->qdd + kN * m &&
                            tr.minv == prev->minv + frg::kMinvN * m;
        } else {
            hb.whole = tr;
        }
        prev = &tr;
    }
    if (hb.contiguous) hb.whole.n_knots = begin;
    const long long ntiles = (begin + 31) / 32;
    if (ntiles > INT_MAX / 2) {
        err = "batch too large: " + std::to_string(begin) + " knots";
        return false;
    }
    hb.tile_seg.resize(static_cast<size_t>(ntiles));
    int s = 0;
    for (long long tile = 0; tile < ntiles; tile++) {
        const long long g = tile * 32;
        while (s + 1 < n_traj && hb.segs[s + 1].knot_begin <= g) s++;
        hb.tile_seg[static_cast<size_t>(tile)] = s;
    }
    return true;
}

bool DeviceBatch::reserve(int nseg_total, int ntiles_cap, std::string &err) {
    if (nseg_total > seg_cap) {
        cudaFree(segs);
        segs = nullptr;
        seg_cap = 0;
        if (cudaMalloc(&segs, sizeof(Segment) * static_cast<size_t>(nseg_total)) != cudaSuccess) {
            err = "cudaMalloc of the segment list failed";
            return false;
        }
        seg_cap = nseg_total;
    }
    if (ntiles_cap > tile_cap) {
        cudaFree(tile_seg);
        tile_seg = nullptr;
        tile_cap = 0;
        if (cudaMalloc(&tile_seg, sizeof(int) * static_cast<size_t>(std::max(ntiles_cap, 1))) != cudaSuccess) {
            err = "cudaMalloc of the tile list failed";
            return false;
        }
        tile_cap = ntiles_cap;
    }
    if (!counter) {
        if (cudaMalloc(&counter, sizeof(unsigned int)) != cudaSuccess || cudaMemset(counter, 0, sizeof(unsigned int)) != cudaSuccess) {
            err = "cudaMalloc of the work counter failed";
            return false;
        }
    }
    return true;
}

void DeviceBatch::release() {
    cudaFree(segs);
    cudaFree(tile_seg);
    cudaFree(counter);
    segs = nullptr;
    tile_seg = nullptr;
    counter = nullptr;
    seg_cap = tile_cap = 0;
}

cudaError_t frg_launch_batch(frg_ctx *ctx, const DeviceBatch &db, int nseg, int ntiles, cudaStream_t stream) {
    return frg::launch_ragged(ctx->damping, ctx->mpc, ctx->ragged_shape, ctx->num_sms, db.segs, nseg, db.tile_seg,
                              ntiles, db.counter, stream);
}

cudaError_t frg_launch_whole(frg_ctx *ctx, const frg_traj &w, cudaStream_t stream) {
    return frg::launch_plain(ctx->damping, ctx->mpc, ctx->shape, static_cast<int>(w.n_knots), w.q, w.qd, w.u, w.dqdd,
                             w.qdd, w.minv, stream);
}

// ------------------------------------------------------------------ C ABI ---

extern "C" {

void frg_options_default(frg_options *opt) {
    if (!opt) return;
    opt->device = 0;
    opt->vel_damping = 0;
    opt->mpc_mode = 0;
    opt->warps_per_cta = 0;
    opt->ctas_per_sm = 0;
    opt->lanes_per_knot = 0;
}

const char *frg_model_name(void) { return FRG_MODEL_NAME; }

int frg_model_dofs(void) { return frg::kN; }

const char *frg_status_string(frg_status s) {
    switch (s) {
        case FRG_OK: return "ok";
        case FRG_ERR_INVALID_ARGUMENT: return "invalid argument";
        case FRG_ERR_CUDA: return "CUDA error";
        case FRG_ERR_OUT_OF_MEMORY: return "out of memory";
        case FRG_ERR_NOT_READY: return "not ready";
        case FRG_ERR_ADMISSION: return "request can never be admitted";
        case FRG_ERR_TIMEOUT: return "timeout";
        case FRG_ERR_SHUTDOWN: return "shut down";
        case FRG_ERR_NOT_FOUND: return "not found";
        case FRG_ERR_INTERNAL: return "internal error";
        case FRG_ERR_CANCELLED: return "cancelled";
    }
    return "unknown status";
}

frg_status frg_create(frg_ctx **out, const frg_options *opt_in) {
    if (!out) {
        frg_set_error(nullptr, "frg_create: out is NULL");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    frg_options opt;
    frg_options_default(&opt);
    if (opt_in) opt = *opt_in;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        frg_set_error(nullptr, std::string("frg_create: no CUDA device: ") + cudaGetErrorString(e));
        return FRG_ERR_CUDA;
    }
    if (opt.device < 0 || opt.device >= ndev) {
        frg_set_error(nullptr, "frg_create: device ordinal out of range");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (opt.warps_per_cta < 0 || opt.warps_per_cta > frg::max_warps_per_cta() || opt.ctas_per_sm < 0 ||
        (opt.lanes_per_knot != 0 && opt.lanes_per_knot != 1 && opt.lanes_per_knot != 8)) {
        frg_set_error(nullptr, "frg_create: invalid launch shape");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    frg_ctx *ctx = new (std::nothrow) frg_ctx();
    if (!ctx) return FRG_ERR_OUT_OF_MEMORY;
    ctx->device = opt.device;
    ctx->damping = opt.vel_damping != 0;
    ctx->mpc = opt.mpc_mode != 0;
    DeviceGuard g(ctx->device);
    cudaDeviceProp prop;
    if (!check(ctx, cudaGetDeviceProperties(&prop, ctx->device), "cudaGetDeviceProperties") ||
        !check(ctx, frg::init_kernels(), "kernel set-up") ||
        !check(ctx, frg::init_group_kernels(), "latency kernel set-up") ||
        !check(ctx, frg::init_ext_kernels(), "fext / forward-dynamics kernel set-up") ||
        !check(ctx, frg::init_f64_kernels(), "FP64 kernel set-up") ||
        !check(ctx, cudaStreamCreateWithFlags(&ctx->io_stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !check(ctx, cudaStreamCreateWithFlags(&ctx->io_stream2, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !check(ctx, cudaStreamCreateWithFlags(&ctx->flight[0], cudaStreamNonBlocking), "cudaStreamCreate") ||
        !check(ctx, cudaStreamCreateWithFlags(&ctx->flight[1], cudaStreamNonBlocking), "cudaStreamCreate") ||
        !check(ctx, cudaStreamCreateWithFlags(&ctx->flight[2], cudaStreamNonBlocking), "cudaStreamCreate") ||
        !check(ctx, cudaEventCreateWithFlags(&ctx->flight_fork, cudaEventDisableTiming), "cudaEventCreate") ||
        !check(ctx, cudaEventCreateWithFlags(&ctx->flight_join, cudaEventDisableTiming), "cudaEventCreate") ||
        !check(ctx, cudaEventCreateWithFlags(&ctx->scratch_done, cudaEventDisableTiming), "cudaEventCreate") ||
        !check(ctx, cudaEventCreateWithFlags(&ctx->batch_done[0], cudaEventDisableTiming), "cudaEventCreate") ||
        !check(ctx, cudaEventCreateWithFlags(&ctx->batch_done[1], cudaEventDisableTiming), "cudaEventCreate") ||
        !check(ctx, cudaEventCreateWithFlags(&ctx->batch_done[2], cudaEventDisableTiming), "cudaEventCreate")) {
        g_orphan_error = ctx->err;
        frg_destroy(ctx);
        return FRG_ERR_CUDA;
    }
    ctx->num_sms = prop.multiProcessorCount;
    ctx->shape = frg::default_shape();
    if (opt.warps_per_cta) ctx->shape.warps_per_cta = opt.warps_per_cta;
    if (opt.ctas_per_sm) ctx->shape.ctas_per_sm = opt.ctas_per_sm;
    if (opt.lanes_per_knot) ctx->shape.lanes_per_knot = opt.lanes_per_knot;
    ctx->ragged_shape = ctx->shape;
    *out = ctx;
    return FRG_OK;
}

void frg_destroy(frg_ctx *ctx) {
    if (!ctx) return;
    {
        DeviceGuard g(ctx->device);
        if (ctx->io_stream) cudaStreamSynchronize(ctx->io_stream);
        if (ctx->io_stream2) cudaStreamSynchronize(ctx->io_stream2);
        for (cudaStream_t f : ctx->flight)
            if (f) cudaStreamSynchronize(f);
        if (ctx->scratch_done) cudaEventSynchronize(ctx->scratch_done);
        ctx->scratch.release();
        cudaFree(ctx->host_buf);
        cudaFree(ctx->host_buf2);
        cudaFree(ctx->f64_buf);
        if (ctx->io_stream) cudaStreamDestroy(ctx->io_stream);
        if (ctx->io_stream2) cudaStreamDestroy(ctx->io_stream2);
        for (cudaStream_t f : ctx->flight)
            if (f) cudaStreamDestroy(f);
        if (ctx->flight_fork) cudaEventDestroy(ctx->flight_fork);
        if (ctx->flight_join) cudaEventDestroy(ctx->flight_join);
        if (ctx->scratch_done) cudaEventDestroy(ctx->scratch_done);
        for (cudaEvent_t e : ctx->batch_done)
            if (e) cudaEventDestroy(e);
        delete ctx->expander;  // joins its threads (no job is in flight between calls)
        for (float *p : ctx->minv_stage) cudaFreeHost(p);
    }
    delete ctx;
}

const char *frg_last_error(const frg_ctx *ctx) { return ctx ? ctx->err.c_str() : g_orphan_error.c_str(); }

frg_status frg_set_launch_shape(frg_ctx *ctx, int warps_per_cta, int ctas_per_sm) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (warps_per_cta < 1 || warps_per_cta > frg::max_warps_per_cta() || ctas_per_sm < 1) {
        frg_set_error(ctx, "frg_set_launch_shape: warps_per_cta must be in [1, 8], ctas_per_sm >= 1");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    ctx->shape.warps_per_cta = ctx->ragged_shape.warps_per_cta = warps_per_cta;
    ctx->shape.ctas_per_sm = ctx->ragged_shape.ctas_per_sm = ctas_per_sm;
    return FRG_OK;
}

frg_status frg_set_lanes_per_knot(frg_ctx *ctx, int lanes_per_knot) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (lanes_per_knot != 1 && lanes_per_knot != 8) {
        frg_set_error(ctx, "frg_set_lanes_per_knot: 1 (throughput mapping) or 8 (latency mapping)");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    ctx->shape.lanes_per_knot = ctx->ragged_shape.lanes_per_knot = lanes_per_knot;
    return FRG_OK;
}

int frg_get_lanes_per_knot(const frg_ctx *ctx) { return ctx ? ctx->shape.lanes_per_knot : 0; }

frg_status frg_get_launch_shape(const frg_ctx *ctx, int *warps_per_cta, int *ctas_per_sm) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (warps_per_cta) *warps_per_cta = ctx->shape.warps_per_cta;
    if (ctas_per_sm) *ctas_per_sm = ctx->shape.ctas_per_sm;
    return FRG_OK;
}

frg_status frg_gradient(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u, float *dqdd,
                        float *qdd, float *minv, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 0 || (n_knots > 0 && !(q && qd && u && dqdd && qdd && minv))) {
        frg_set_error(ctx, "frg_gradient: negative n_knots or null pointer");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_knots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    if (!check(ctx, frg::launch_plain(ctx->damping, ctx->mpc, ctx->shape, n_knots, q, qd, u, dqdd, qdd, minv, stream),
               "frg_gradient launch"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_single_knot_latency(frg_ctx *ctx, int lanes_per_knot, int iters, const float *q, const float *qd,
                                   const float *u, float *dqdd, float *qdd, float *minv, frg_stream stream,
                                   double *us_per_knot) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if ((lanes_per_knot != 1 && lanes_per_knot != 8) || iters < 1 || !(q && qd && u && dqdd && qdd && minv)) {
        frg_set_error(ctx, "frg_single_knot_latency: lanes_per_knot must be 1 or 8, iters >= 1, arrays non-null");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    DeviceGuard g(ctx->device);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (us_per_knot) {
        if (!check(ctx, cudaEventCreate(&e0), "cudaEventCreate") || !check(ctx, cudaEventCreate(&e1), "cudaEventCreate") ||
            !check(ctx, cudaEventRecord(e0, stream), "cudaEventRecord")) {
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            return FRG_ERR_CUDA;
        }
    }
    bool ok = check(ctx, frg::launch_single_knot(ctx->damping, ctx->mpc, lanes_per_knot, iters, q, qd, u, dqdd, qdd,
                                                 minv, stream),
                    "frg_single_knot_latency launch");
    if (us_per_knot) {
        float ms = 0.0f;
        ok = ok && check(ctx, cudaEventRecord(e1, stream), "cudaEventRecord") &&
             check(ctx, cudaEventSynchronize(e1), "cudaEventSynchronize") &&
             check(ctx, cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        if (ok) *us_per_knot = 1e3 * static_cast<double>(ms) / iters;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    return ok ? FRG_OK : FRG_ERR_CUDA;
}

frg_status frg_gradient_fext(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                             const float *fext, float *dqdd, float *qdd, float *minv, frg_stream stream) {
    if (!fext) return frg_gradient(ctx, n_knots, q, qd, u, dqdd, qdd, minv, stream);
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 0 || (n_knots > 0 && !(q && qd && u && dqdd && qdd && minv))) {
        frg_set_error(ctx, "frg_gradient_fext: negative n_knots or null pointer");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_knots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    if (!check(ctx, frg::launch_ext(ctx->damping, ctx->mpc, ctx->shape, n_knots, q, qd, u, fext, dqdd, qdd, minv, false,
                                    stream),
               "frg_gradient_fext launch"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_forward_dynamics(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                                const float *fext, float *qdd, float *minv, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 0 || (n_knots > 0 && !(q && qd && u && qdd))) {
        frg_set_error(ctx, "frg_forward_dynamics: negative n_knots or null pointer");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_knots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    if (!check(ctx, frg::launch_ext(ctx->damping, ctx->mpc, ctx->shape, n_knots, q, qd, u, fext, nullptr, qdd, minv, true,
                                    stream),
               "frg_forward_dynamics launch"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_discrete_jacobians(frg_ctx *ctx, int n_knots, const float *dqdd, const float *minv, float dt, float *A,
                                  float *B, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 0 || (n_knots > 0 && !(dqdd && minv && A && B)) || !(dt == dt)) {
        frg_set_error(ctx, "frg_discrete_jacobians: negative n_knots, null pointer or NaN dt");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_knots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    if (!check(ctx, frg::launch_discretize(n_knots, dqdd, minv, dt, A, B, stream), "frg_discrete_jacobians launch"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_gradient_knots(frg_ctx *ctx, int n_knots, float *knots, float *dqdd, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 0 || (n_knots > 0 && !(knots && dqdd))) {
        frg_set_error(ctx, "frg_gradient_knots: negative n_knots or null pointer");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_knots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    if (!check(ctx, frg::launch_knots(ctx->damping, ctx->mpc, ctx->shape, n_knots, knots, dqdd, stream),
               "frg_gradient_knots launch"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_knot_status(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                           const float *dqdd, const float *qdd, const float *minv, uint32_t *status,
                           frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 0 || (n_knots > 0 && !(q && qd && u && status))) {
        frg_set_error(ctx, "frg_knot_status: negative n_knots or null input / status pointer");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_knots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    if (!check(ctx, frg::launch_knot_status(ctx->num_sms, n_knots, q, qd, u, dqdd, qdd, minv, status, stream),
               "frg_knot_status launch"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_gradient_f64(frg_ctx *ctx, int n_knots, const double *q, const double *qd, const double *u,
                            double *dqdd, double *qdd, double *minv, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 0 || (n_knots > 0 && !(q && qd && u && dqdd && qdd && minv))) {
        frg_set_error(ctx, "frg_gradient_f64: negative n_knots or null pointer");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_knots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    if (!check(ctx, frg::launch_plain_f64(ctx->damping, ctx->mpc, ctx->num_sms, n_knots, q, qd, u, dqdd, qdd, minv,
                                          stream),
               "frg_gradient_f64 launch"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_verify_f64(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                          const float *dqdd, const float *qdd, const float *minv, double *err, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 0 || (n_knots > 0 && !(q && qd && u && dqdd && qdd && minv && err))) {
        frg_set_error(ctx, "frg_verify_f64: negative n_knots or null pointer");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_knots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    const size_t n = static_cast<size_t>(n_knots), need = frg::kSlotN * n;
    if (ctx->f64_buf_doubles < need) {
        cudaFree(ctx->f64_buf);  // waits for earlier work that may still read it
        ctx->f64_buf = nullptr;
        ctx->f64_buf_doubles = 0;
        if (cudaMalloc(&ctx->f64_buf, sizeof(double) * need) != cudaSuccess) {
            cudaGetLastError();
            ctx->f64_buf = nullptr;
            frg_set_error(ctx, "frg_verify_f64: out of device memory for the FP64 scratch");
            return FRG_ERR_OUT_OF_MEMORY;
        }
        ctx->f64_buf_doubles = need;
    }
    double *b = ctx->f64_buf;
    double *q64 = b, *qd64 = b + frg::kSlotQd * n, *u64 = b + frg::kSlotU * n;
    double *dqdd64 = b + frg::kSlotDqdd * n, *qdd64 = b + frg::kSlotQdd * n, *minv64 = b + frg::kSlotMinv * n;
    if (!check(ctx, frg::launch_widen_inputs(ctx->num_sms, n_knots, q, qd, u, b, stream), "frg_verify_f64 widen") ||
        !check(ctx, frg::launch_plain_f64(ctx->damping, ctx->mpc, ctx->num_sms, n_knots, q64, qd64, u64, dqdd64,
                                          qdd64, minv64, stream),
               "frg_verify_f64 launch") ||
        !check(ctx, frg::launch_compare_f64(ctx->num_sms, n_knots, dqdd, qdd, minv, dqdd64, qdd64, minv64, err, stream),
               "frg_verify_f64 compare"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

namespace {

// Grows a ctx-owned device buffer to `need` floats (cudaFree waits for earlier
// work that may still use it).
bool ensure_floats(frg_ctx *ctx, float **buf, size_t *cap, size_t need, const char *who) {
    if (need <= *cap) return true;
    cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    if (cudaMalloc(buf, need * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        *buf = nullptr;
        frg_set_error(ctx, std::string(who) + ": cudaMalloc of " + std::to_string(need * 4) + " bytes failed");
        return false;
    }
    *cap = need;
    return true;
}

// True if the GPU of ctx can load/store `p` directly: pinned (page-locked,
// mapped) host memory, or device memory.
bool device_accessible(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer == p) || a.type == cudaMemoryTypeDevice ||
           a.type == cudaMemoryTypeManaged;
}

// Results a host call returns: dqdd always; q̈ and Minv unless their host
// array is NULL.  The kernel still writes a result that is not asked for --
// into the tail of the ctx-owned relay buffer, [dqdd | q̈ | Minv], so in device
// memory -- and no byte of it crosses the host link.
struct HostOuts {
    float *dqdd, *qdd, *minv;
};

size_t relay_floats(size_t n, const float *qdd, const float *minv) {
    if (!minv) return (frg::kDqddN + frg::kN + frg::kMinvN) * n;
    if (!qdd) return (frg::kDqddN + frg::kN) * n;
    return frg::kDqddN * n;
}

HostOuts host_outs(float *relay, size_t n, float *qdd, float *minv) {
    return HostOuts{relay, qdd ? qdd : relay + frg::kDqddN * n, minv ? minv : relay + (frg::kDqddN + frg::kN) * n};
}

bool host_or_null_accessible(const void *p) { return !p || device_accessible(p); }

}  // namespace

frg_status frg_gradient_host(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                             float *dqdd, float *qdd, float *minv) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 0 || (n_knots > 0 && !(q && qd && u && dqdd))) {
        frg_set_error(ctx, "frg_gradient_host: negative n_knots or null pointer");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_knots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    cudaStream_t s = ctx->io_stream;
    const size_t n = static_cast<size_t>(n_knots);
    // Pinned host arrays: one launch and no copies.  The kernel reads q, qd,
    // u across the host link and writes qdd and Minv in place as whole
    // 16-byte-aligned tiles; dqdd goes through a device buffer (L2-resident
    // while its tile finishes) and leaves as whole lines (launch_host_out).
    // The results stream out while later tiles compute, so the host link's
    // device-to-host rate (about 190 GB/s here) bounds the call.
    if (device_accessible(q) && device_accessible(qd) && device_accessible(u) && device_accessible(dqdd) &&
        host_or_null_accessible(qdd) && host_or_null_accessible(minv)) {
        if (!ensure_floats(ctx, &ctx->host_buf, &ctx->host_buf_floats, relay_floats(n, qdd, minv),
                           "frg_gradient_host"))
            return FRG_ERR_OUT_OF_MEMORY;
        const HostOuts o = host_outs(ctx->host_buf, n, qdd, minv);
        if (!check(ctx,
                   frg::launch_host_out(ctx->damping, ctx->mpc, ctx->shape, n_knots, q, qd, u, o.dqdd, dqdd, o.qdd,
                                        o.minv, s),
                   "frg_gradient_host launch") ||
            !check(ctx, cudaStreamSynchronize(s), "frg_gradient_host sync"))
            return FRG_ERR_CUDA;
        return FRG_OK;
    }
    // Pageable host arrays: stage through device buffers owned by ctx.
    if (!ensure_floats(ctx, &ctx->host_buf, &ctx->host_buf_floats, n * frg::kSlotN, "frg_gradient_host"))
        return FRG_ERR_OUT_OF_MEMORY;
    float *b = ctx->host_buf;
    float *dq = b, *dqd = b + frg::kSlotQd * n, *du = b + frg::kSlotU * n, *ddqdd = b + frg::kSlotDqdd * n,
          *dqdd_ = b + frg::kSlotQdd * n, *dminv = b + frg::kSlotMinv * n;
    const size_t b7 = frg::kN * n * sizeof(float);
    if (!check(ctx, cudaMemcpyAsync(dq, q, b7, cudaMemcpyHostToDevice, s), "H2D q") ||
        !check(ctx, cudaMemcpyAsync(dqd, qd, b7, cudaMemcpyHostToDevice, s), "H2D qd") ||
        !check(ctx, cudaMemcpyAsync(du, u, b7, cudaMemcpyHostToDevice, s), "H2D u") ||
        !check(ctx, frg::launch_plain(ctx->damping, ctx->mpc, ctx->shape, n_knots, dq, dqd, du, ddqdd, dqdd_, dminv, s),
               "frg_gradient_host launch") ||
        !check(ctx, cudaMemcpyAsync(dqdd, ddqdd, frg::kDqddN * n * sizeof(float), cudaMemcpyDeviceToHost, s), "D2H dqdd") ||
        (qdd && !check(ctx, cudaMemcpyAsync(qdd, dqdd_, b7, cudaMemcpyDeviceToHost, s), "D2H qdd")) ||
        (minv &&
         !check(ctx, cudaMemcpyAsync(minv, dminv, frg::kMinvN * n * sizeof(float), cudaMemcpyDeviceToHost, s),
                "D2H minv")) ||
        !check(ctx, cudaStreamSynchronize(s), "frg_gradient_host sync"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

namespace {

// frg_gradient_host_batches when every batch returns Minv: Minv crosses the
// host link as its packed upper triangle (kMinvPackedN instead of kMinvN
// floats per knot: 532 instead of 616 result bytes per knot at 7 joints, and
// the link bounds the call), into one of three pinned staging buffers; host
// threads expand each batch to the caller's dense array while the next
// batches compute and stream.  Expansions run one at a time, in batch order:
// batch j - 1's starts when its launch has ended and batch j - 2's expansion
// is done, right after batch j is launched; so batch j can reuse the staging
// buffer of batch j - 3 without waiting, and two launches stay in flight.
// Bits are those of the dense path (the expansion only copies).
frg_status host_batches_packed(frg_ctx *ctx, int n_batches, const frg_host_batch *batches, size_t max_n) {
    const size_t stage = static_cast<size_t>(frg::kMinvPackedN) * max_n;
    if (ctx->minv_stage_floats < stage) {
        for (float *&p : ctx->minv_stage) {
            cudaFreeHost(p);  // waits for earlier work that may still write it
            p = nullptr;
        }
        ctx->minv_stage_floats = 0;
        for (float *&p : ctx->minv_stage)
            if (cudaHostAlloc(reinterpret_cast<void **>(&p), stage * sizeof(float), cudaHostAllocPortable) !=
                cudaSuccess) {
                cudaGetLastError();
                p = nullptr;
                frg_set_error(ctx, "frg_gradient_host_batches: cudaHostAlloc of the Minv staging failed");
                return FRG_ERR_OUT_OF_MEMORY;
            }
        ctx->minv_stage_floats = stage;
    }
    if (!ctx->expander) {
        const unsigned hw = std::thread::hardware_concurrency();
        // leave two cores to the calling thread and the CUDA driver
        ctx->expander = new (std::nothrow) MinvExpander(static_cast<int>(std::min(14u, std::max(1u, hw > 2 ? hw - 2 : 1u))));
        if (!ctx->expander) return FRG_ERR_OUT_OF_MEMORY;
    }
    MinvExpander &ex = *ctx->expander;
    bool ok = true;
    int j = 0, prev = -1;  // j: nonempty batches launched; prev: the last one
    for (int i = 0; ok && i < n_batches; i++) {
        const frg_host_batch &b = batches[i];
        if (b.n_knots == 0) continue;
        const int k = j % 3, odd = j & 1;
        cudaStream_t st = odd ? ctx->io_stream2 : ctx->io_stream;
        // dqdd relay per stream, and q̈ in the relay's tail when the caller does not want it
        const HostOuts o = host_outs(odd ? ctx->host_buf2 : ctx->host_buf, static_cast<size_t>(b.n_knots), b.qdd,
                                     b.minv);
        ok = check(ctx,
                   frg::launch_host_out(ctx->damping, ctx->mpc, ctx->shape, b.n_knots, b.q, b.qd, b.u, o.dqdd, b.dqdd,
                                        o.qdd, ctx->minv_stage[k], st, true),
                   "frg_gradient_host_batches launch") &&
             check(ctx, cudaEventRecord(ctx->batch_done[k], st), "frg_gradient_host_batches");
        if (ok && prev >= 0) {  // batch j - 1's launch has ended: expand it while batch j runs
            const int kp = (j + 2) % 3;
            ex.wait();  // batch j - 2's expansion
            ok = check(ctx, cudaEventSynchronize(ctx->batch_done[kp]), "frg_gradient_host_batches sync");
            if (ok) ex.start(ctx->minv_stage[kp], batches[prev].minv, static_cast<size_t>(batches[prev].n_knots));
        }
        prev = i;
        j++;
    }
    if (ok && prev >= 0) {
        const int kp = (j + 2) % 3;
        ex.wait();
        ok = check(ctx, cudaEventSynchronize(ctx->batch_done[kp]), "frg_gradient_host_batches sync");
        if (ok) ex.start(ctx->minv_stage[kp], batches[prev].minv, static_cast<size_t>(batches[prev].n_knots));
    }
    ex.wait();
    const cudaError_t e1 = cudaStreamSynchronize(ctx->io_stream), e2 = cudaStreamSynchronize(ctx->io_stream2);
    if (!ok) return FRG_ERR_CUDA;
    if (!check(ctx, e1, "frg_gradient_host_batches sync") || !check(ctx, e2, "frg_gradient_host_batches sync"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

}  // namespace

frg_status frg_gradient_host_batches(frg_ctx *ctx, int n_batches, const frg_host_batch *batches) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_batches < 0 || (n_batches > 0 && !batches)) {
        frg_set_error(ctx, "frg_gradient_host_batches: bad batch list");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    bool pinned = true, all_minv = true;
    size_t need = 0, max_n = 0;
    int nonempty = 0;
    for (int i = 0; i < n_batches; i++) {
        const frg_host_batch &b = batches[i];
        if (b.n_knots < 0 || (b.n_knots > 0 && !(b.q && b.qd && b.u && b.dqdd))) {
            frg_set_error(ctx, "frg_gradient_host_batches: batch " + std::to_string(i) + ": negative size or null pointer");
            return FRG_ERR_INVALID_ARGUMENT;
        }
        if (b.n_knots == 0) continue;
        nonempty++;
        all_minv = all_minv && b.minv;
        max_n = std::max(max_n, static_cast<size_t>(b.n_knots));
        need = std::max(need, relay_floats(static_cast<size_t>(b.n_knots), b.qdd, b.minv));
        pinned = pinned && device_accessible(b.q) && device_accessible(b.qd) && device_accessible(b.u) &&
                 device_accessible(b.dqdd) && host_or_null_accessible(b.qdd) && host_or_null_accessible(b.minv);
    }
    if (!pinned) {  // pageable arrays: one staged call after the other
        for (int i = 0; i < n_batches; i++) {
            const frg_host_batch &b = batches[i];
            const frg_status st = frg_gradient_host(ctx, b.n_knots, b.q, b.qd, b.u, b.dqdd, b.qdd, b.minv);
            if (st != FRG_OK) return st;
        }
        return FRG_OK;
    }
    if (need == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    if (!ensure_floats(ctx, &ctx->host_buf, &ctx->host_buf_floats, need, "frg_gradient_host_batches") ||
        !ensure_floats(ctx, &ctx->host_buf2, &ctx->host_buf2_floats, need, "frg_gradient_host_batches"))
        return FRG_ERR_OUT_OF_MEMORY;
    // Batches alternate between two streams, each with its own dqdd relay
    // buffer, so two launches are in flight at once: one batch's launch and
    // first tiles (before any result exists) overlap the previous batch's
    // results streaming over the host link.  A batch reuses its stream's relay
    // buffer only after the batch two places before it, in stream order.
    if (nonempty >= 2 && all_minv && ctx->shape.lanes_per_knot == 1)
        return host_batches_packed(ctx, n_batches, batches, max_n);
    for (int i = 0; i < n_batches; i++) {
        const frg_host_batch &b = batches[i];
        if (b.n_knots == 0) continue;
        const bool odd = (i & 1) != 0;
        const HostOuts o = host_outs(odd ? ctx->host_buf2 : ctx->host_buf, static_cast<size_t>(b.n_knots), b.qdd,
                                     b.minv);
        if (!check(ctx,
                   frg::launch_host_out(ctx->damping, ctx->mpc, ctx->shape, b.n_knots, b.q, b.qd, b.u, o.dqdd, b.dqdd,
                                        o.qdd, o.minv, odd ? ctx->io_stream2 : ctx->io_stream),
                   "frg_gradient_host_batches launch")) {
            cudaStreamSynchronize(ctx->io_stream);
            cudaStreamSynchronize(ctx->io_stream2);
            return FRG_ERR_CUDA;
        }
    }
    const cudaError_t e1 = cudaStreamSynchronize(ctx->io_stream), e2 = cudaStreamSynchronize(ctx->io_stream2);
    if (!check(ctx, e1, "frg_gradient_host_batches sync") || !check(ctx, e2, "frg_gradient_host_batches sync"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_gradient_per_trajectory(frg_ctx *ctx, int n_traj, const frg_traj *trajs, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_traj < 0 || (n_traj > 0 && !trajs)) {
        frg_set_error(ctx, "frg_gradient_per_trajectory: bad trajectory list");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    for (int t = 0; t < n_traj; t++)
        if (!valid_traj(trajs[t]) || trajs[t].n_knots > INT_MAX) {
            frg_set_error(ctx, "frg_gradient_per_trajectory: trajectory " + std::to_string(t) + " is invalid");
            return FRG_ERR_INVALID_ARGUMENT;
        }
    DeviceGuard g(ctx->device);
    for (int t = 0; t < n_traj; t++) {
        const frg_traj &tr = trajs[t];
        if (tr.n_knots == 0) continue;
        if (!check(ctx,
                   frg::launch_plain(ctx->damping, ctx->mpc, ctx->shape, static_cast<int>(tr.n_knots), tr.q, tr.qd,
                                     tr.u, tr.dqdd, tr.qdd, tr.minv, stream),
                   "per-trajectory launch"))
            return FRG_ERR_CUDA;
    }
    return FRG_OK;
}

frg_status frg_gradient_batched(frg_ctx *ctx, int n_traj, const frg_traj *trajs, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_traj < 0 || (n_traj > 0 && !trajs)) {
        frg_set_error(ctx, "frg_gradient_batched: bad trajectory list");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    HostBatch hb;
    std::string err;
    if (!frg_build_batch(n_traj, trajs, hb, err)) {
        frg_set_error(ctx, "frg_gradient_batched: " + err);
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (hb.nknots == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    if (hb.contiguous) {
        if (!check(ctx, frg_launch_whole(ctx, hb.whole, stream), "batched launch")) return FRG_ERR_CUDA;
        return FRG_OK;
    }
    // the one-shot descriptor buffers are reused: wait for the previous user
    if (!check(ctx, cudaEventSynchronize(ctx->scratch_done), "scratch wait")) return FRG_ERR_CUDA;
    const int nseg = n_traj, ntiles = static_cast<int>(hb.tile_seg.size());
    if (!ctx->scratch.reserve(nseg + 1, ntiles, err)) {
        cudaGetLastError();
        frg_set_error(ctx, "frg_gradient_batched: " + err);
        return FRG_ERR_OUT_OF_MEMORY;
    }
    if (!check(ctx,
               cudaMemcpyAsync(ctx->scratch.segs, hb.segs.data(), sizeof(Segment) * hb.segs.size(),
                               cudaMemcpyHostToDevice, stream),
               "segment list upload") ||
        !check(ctx,
               cudaMemcpyAsync(ctx->scratch.tile_seg, hb.tile_seg.data(), sizeof(int) * hb.tile_seg.size(),
                               cudaMemcpyHostToDevice, stream),
               "tile list upload") ||
        !check(ctx, frg_launch_batch(ctx, ctx->scratch, nseg, ntiles, stream), "batched launch") ||
        !check(ctx, cudaEventRecord(ctx->scratch_done, stream), "cudaEventRecord"))
        return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_gradient_ragged(frg_ctx *ctx, int n_traj, const int64_t *offsets, const float *q, const float *qd,
                               const float *u, float *dqdd, float *qdd, float *minv, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    std::vector<frg_traj> trajs;
    if (!frg_offsets_to_trajs(n_traj, offsets, q, qd, u, dqdd, qdd, minv, trajs)) {
        frg_set_error(ctx, "frg_gradient_ragged: offsets must be n_traj+1 non-decreasing values from 0, arrays non-null");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    return frg_gradient_batched(ctx, n_traj, trajs.data(), stream);
}

void *frg_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void frg_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"

bool frg_offsets_to_trajs(int n_traj, const int64_t *offsets, const float *q, const float *qd, const float *u,
                          float *dqdd, float *qdd, float *minv, std::vector<frg_traj> &out) {
    if (n_traj < 0 || (n_traj > 0 && !offsets)) return false;
    if (n_traj > 0 && offsets[0] != 0) return false;
    for (int t = 0; t < n_traj; t++)
        if (offsets[t + 1] < offsets[t]) return false;
    const int64_t total = n_traj > 0 ? offsets[n_traj] : 0;
    if (total > 0 && !(q && qd && u && dqdd && qdd && minv)) return false;
    out.resize(static_cast<size_t>(n_traj));
    for (int t = 0; t < n_traj; t++) {
        const int64_t o = offsets[t];
        out[t] = frg_traj{offsets[t + 1] - o, q + frg::kN * o, qd + frg::kN * o, u + frg::kN * o,
                          dqdd + frg::kDqddN * o, qdd + frg::kN * o, minv + frg::kMinvN * o};
    }
    return true;
}
