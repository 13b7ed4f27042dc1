// Plans (batched launches prepared once: descriptor lists on the device, launch
// shape fixed) and the launch-shape autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <new>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>

#include "frg.h"
#include "frg_internal.h"
#include "frg_kernels.cuh"

namespace {

bool ok(frg_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    frg_set_error(ctx, std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

// One launch of a plan, with the launch shape the context had when the plan
// was made.  A direct launch rather than a graph replay: launched with
// programmatic stream serialization (frg_launch.cuh), a plan launch that
// follows another on the stream starts while the earlier one's last tiles
// finish, which a graph launch cannot do (6 % of a launch over the 512-mix).
cudaError_t plan_launch(frg_plan *plan, cudaStream_t st) {
    frg_ctx *ctx = plan->ctx;
    if (plan->contiguous)
        return frg::launch_plain(ctx->damping, ctx->mpc, plan->shape, static_cast<int>(plan->whole.n_knots),
                                 plan->whole.q, plan->whole.qd, plan->whole.u, plan->whole.dqdd, plan->whole.qdd,
                                 plan->whole.minv, st);
    return frg::launch_ragged(ctx->damping, ctx->mpc, plan->shape, ctx->num_sms, plan->dev.segs, plan->nseg,
                              plan->dev.tile_seg, plan->ntiles, plan->dev.counter, st);
}

}  // namespace

extern "C" {

frg_status frg_plan_create(frg_ctx *ctx, int n_traj, const frg_traj *trajs, frg_plan **out) {
    if (!ctx || !out) return FRG_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n_traj < 0 || (n_traj > 0 && !trajs)) {
        frg_set_error(ctx, "frg_plan_create: bad trajectory list");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    HostBatch hb;
    std::string err;
    if (!frg_build_batch(n_traj, trajs, hb, err)) {
        frg_set_error(ctx, "frg_plan_create: " + err);
        return FRG_ERR_INVALID_ARGUMENT;
    }
    frg_plan *plan = new (std::nothrow) frg_plan();
    if (!plan) return FRG_ERR_OUT_OF_MEMORY;
    plan->ctx = ctx;
    plan->nseg = n_traj;
    plan->ntiles = static_cast<int>(hb.tile_seg.size());
    plan->nknots = hb.nknots;
    plan->contiguous = hb.contiguous;
    plan->whole = hb.whole;
    if (plan->nknots == 0) {
        *out = plan;
        return FRG_OK;
    }
    DeviceGuard g(ctx->device);
    plan->shape = plan->contiguous ? ctx->shape : ctx->ragged_shape;
    if (plan->contiguous) {  // one plain launch: no descriptor lists on the device
        *out = plan;
        return FRG_OK;
    }
    if (!plan->dev.reserve(plan->nseg + 1, plan->ntiles, err)) {
        cudaGetLastError();
        frg_set_error(ctx, "frg_plan_create: " + err);
        frg_plan_destroy(plan);
        return FRG_ERR_OUT_OF_MEMORY;
    }
    if (!ok(ctx, cudaMemcpy(plan->dev.segs, hb.segs.data(), sizeof(frg::Segment) * hb.segs.size(), cudaMemcpyHostToDevice),
            "plan segment upload") ||
        !ok(ctx, cudaMemcpy(plan->dev.tile_seg, hb.tile_seg.data(), sizeof(int) * hb.tile_seg.size(), cudaMemcpyHostToDevice),
            "plan tile upload")) {
        frg_plan_destroy(plan);
        return FRG_ERR_CUDA;
    }
    *out = plan;
    return FRG_OK;
}

frg_status frg_plan_create_ragged(frg_ctx *ctx, int n_traj, const int64_t *offsets, const float *q, const float *qd,
                                  const float *u, float *dqdd, float *qdd, float *minv, frg_plan **out) {
    if (!ctx || !out) return FRG_ERR_INVALID_ARGUMENT;
    std::vector<frg_traj> trajs;
    if (!frg_offsets_to_trajs(n_traj, offsets, q, qd, u, dqdd, qdd, minv, trajs)) {
        frg_set_error(ctx, "frg_plan_create_ragged: offsets must be n_traj+1 non-decreasing values from 0");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    return frg_plan_create(ctx, n_traj, trajs.data(), out);
}

frg_status frg_plan_launch(frg_plan *plan, frg_stream stream) {
    if (!plan) return FRG_ERR_INVALID_ARGUMENT;
    if (plan->nknots == 0) return FRG_OK;
    DeviceGuard g(plan->ctx->device);
    if (!ok(plan->ctx, plan_launch(plan, reinterpret_cast<cudaStream_t>(stream)), "frg_plan_launch")) return FRG_ERR_CUDA;
    return FRG_OK;
}

frg_status frg_plan_launch_many(frg_ctx *ctx, int n_plans, frg_plan *const *plans, int in_flight,
                                frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_plans < 0 || (n_plans > 0 && !plans) || in_flight < 1 || in_flight > frg_ctx::kMaxInFlight) {
        frg_set_error(ctx, "frg_plan_launch_many: bad plan list or in_flight outside 1.." +
                               std::to_string(frg_ctx::kMaxInFlight));
        return FRG_ERR_INVALID_ARGUMENT;
    }
    std::unordered_map<const frg_plan *, int> residue;  // the stream each plan runs on
    for (int i = 0; i < n_plans; i++) {
        if (!plans[i] || plans[i]->ctx != ctx) {
            frg_set_error(ctx, "frg_plan_launch_many: plan " + std::to_string(i) + " is NULL or of another context");
            return FRG_ERR_INVALID_ARGUMENT;
        }
        const auto it = residue.emplace(plans[i], i % in_flight).first;
        if (it->second != i % in_flight) {
            frg_set_error(ctx, "frg_plan_launch_many: plan " + std::to_string(i) +
                                   " also appears at a position of another residue mod in_flight; those run "
                                   "concurrently");
            return FRG_ERR_INVALID_ARGUMENT;
        }
    }
    if (n_plans == 0) return FRG_OK;
    DeviceGuard g(ctx->device);
    cudaStream_t st[frg_ctx::kMaxInFlight] = {reinterpret_cast<cudaStream_t>(stream)};
    for (int k = 1; k < in_flight; k++) st[k] = ctx->flight[k - 1];
    // the extra streams start after the work queued on `stream` so far
    if (in_flight > 1 && !ok(ctx, cudaEventRecord(ctx->flight_fork, st[0]), "frg_plan_launch_many fork"))
        return FRG_ERR_CUDA;
    for (int k = 1; k < in_flight; k++)
        if (!ok(ctx, cudaStreamWaitEvent(st[k], ctx->flight_fork, 0), "frg_plan_launch_many fork"))
            return FRG_ERR_CUDA;
    bool good = true;
    for (int i = 0; good && i < n_plans; i++)
        good = ok(ctx, plan_launch(plans[i], st[i % in_flight]), "frg_plan_launch_many launch");
    // `stream` continues after every extra stream's launches (joined even after
    // a failed launch, so that no stream is left behind)
    bool joined = true;
    for (int k = 1; k < in_flight; k++)
        joined = ok(ctx, cudaEventRecord(ctx->flight_join, st[k]), "frg_plan_launch_many join") &&
                 ok(ctx, cudaStreamWaitEvent(st[0], ctx->flight_join, 0), "frg_plan_launch_many join") && joined;
    return good && joined ? FRG_OK : FRG_ERR_CUDA;
}

int64_t frg_plan_knots(const frg_plan *plan) { return plan ? plan->nknots : 0; }

void frg_plan_destroy(frg_plan *plan) {
    if (!plan) return;
    {
        DeviceGuard g(plan->ctx->device);
        plan->dev.release();
    }
    delete plan;
}

frg_status frg_autotune(frg_ctx *ctx, int64_t n_knots, double *best_knots_per_s) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_knots < 32 || n_knots > (int64_t(1) << 26)) {
        frg_set_error(ctx, "frg_autotune: n_knots must be in [32, 2^26]");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    DeviceGuard g(ctx->device);
    const size_t n = static_cast<size_t>(n_knots);
    using frg::kN;
    std::vector<float> h(3 * kN * n);
    std::mt19937 rng(12345);
    std::uniform_real_distribution<float> uq(-2.0f, 2.0f), uu(-20.0f, 20.0f);
    for (size_t i = 0; i < 2 * kN * n; i++) h[i] = uq(rng);
    for (size_t i = 2 * kN * n; i < 3 * kN * n; i++) h[i] = uu(rng);
    float *d = nullptr;
    if (cudaMalloc(&d, sizeof(float) * frg::kSlotN * n) != cudaSuccess) {
        cudaGetLastError();
        frg_set_error(ctx, "frg_autotune: out of device memory");
        return FRG_ERR_OUT_OF_MEMORY;
    }
    frg_traj tr{n_knots, d, d + frg::kSlotQd * n, d + frg::kSlotU * n, d + frg::kSlotDqdd * n,
                d + frg::kSlotQdd * n, d + frg::kSlotMinv * n};
    std::string err;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t s = ctx->io_stream;
    bool good = ok(ctx, cudaMemcpy(d, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice), "autotune upload") &&
                ok(ctx, cudaEventCreate(&e0), "cudaEventCreate") && ok(ctx, cudaEventCreate(&e1), "cudaEventCreate");
    const frg::LaunchShape saved = ctx->shape, saved_r = ctx->ragged_shape;
    auto time_ms = [&](auto launch) {
        float ms_min = FLT_MAX;
        for (int rep = 0; rep < 5 && good; rep++) {
            good = ok(ctx, cudaEventRecord(e0, s), "record") && ok(ctx, launch(), "autotune launch") &&
                   ok(ctx, cudaEventRecord(e1, s), "record") && ok(ctx, cudaEventSynchronize(e1), "sync");
            float ms = 0;
            if (good && rep > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) ms_min = std::min(ms_min, ms);
        }
        return ms_min;
    };
    // A candidate replaces the best only when more than 1 % faster: near-ties
    // keep the earlier candidate, and each CTA size is tried at full residency
    // first.  On the tuning batch (whole tiles) shapes with fewer resident warps
    // can tie the full ones, but on batches with split tiles they are slower.
    constexpr float kMargin = 0.99f;
    // 1) contiguous batches: the plain kernel (threads per knot x warps per CTA)
    frg::LaunchShape best = saved;
    float best_ms = FLT_MAX;
    for (int lanes : {1, 8})
        for (int w : {1, 2, 3, 4, 6, 8}) {
            if (!good) break;
            ctx->shape.warps_per_cta = w;
            ctx->shape.lanes_per_knot = lanes;
            const float ms = time_ms([&] { return frg_launch_whole(ctx, tr, s); });
            if (ms < best_ms * kMargin) {
                best_ms = ms;
                best = ctx->shape;
            }
        }
    // 2) scattered trajectories: the persistent kernel (x resident CTAs per SM),
    //    on the same knots cut into trajectories of 8 to 256 knots (seeded),
    //    listed in shuffled order: most tiles then span two trajectories stored
    //    apart, as in a solver's batch.  (Whole-tile trajectories favour shapes
    //    with fewer resident warps that lose on such batches.)
    std::vector<frg_traj> scattered;
    std::uniform_int_distribution<int> uh(8, 256);
    for (size_t k0 = 0; k0 < n;) {
        const size_t m = std::min<size_t>(static_cast<size_t>(uh(rng)), n - k0);
        scattered.push_back(frg_traj{static_cast<int64_t>(m), tr.q + kN * k0, tr.qd + kN * k0, tr.u + kN * k0,
                                     tr.dqdd + frg::kDqddN * k0, tr.qdd + kN * k0, tr.minv + frg::kMinvN * k0});
        k0 += m;
    }
    std::shuffle(scattered.begin(), scattered.end(), rng);
    HostBatch hs;
    DeviceBatch ds;
    good = good && frg_build_batch(static_cast<int>(scattered.size()), scattered.data(), hs, err) &&
           ds.reserve(static_cast<int>(hs.segs.size()), static_cast<int>(hs.tile_seg.size()), err) &&
           ok(ctx, cudaMemcpy(ds.segs, hs.segs.data(), sizeof(frg::Segment) * hs.segs.size(), cudaMemcpyHostToDevice),
              "upload") &&
           ok(ctx, cudaMemcpy(ds.tile_seg, hs.tile_seg.data(), sizeof(int) * hs.tile_seg.size(), cudaMemcpyHostToDevice),
              "upload");
    frg::LaunchShape best_r = saved_r;
    float best_r_ms = FLT_MAX;
    const int nseg = static_cast<int>(scattered.size()), ntiles_s = static_cast<int>(hs.tile_seg.size());
    for (int lanes : {1, 8})
        for (int w : {1, 2, 3, 4, 6, 8}) {
            if (!good) break;
            const int occ = frg::max_ctas_per_sm(w, lanes);
            for (int c = occ; c >= 1; c--) {  // every residency: fewer CTAs can balance the last wave
                ctx->ragged_shape.warps_per_cta = w;
                ctx->ragged_shape.ctas_per_sm = c;
                ctx->ragged_shape.lanes_per_knot = lanes;
                const float ms = time_ms([&] { return frg_launch_batch(ctx, ds, nseg, ntiles_s, s); });
                if (ms < best_r_ms * kMargin) {
                    best_r_ms = ms;
                    best_r = ctx->ragged_shape;
                }
            }
        }
    ds.release();
    if (!good && err.size()) frg_set_error(ctx, "frg_autotune: " + err);
    ctx->shape = good ? best : saved;
    ctx->ragged_shape = good ? best_r : saved_r;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    if (!good) return FRG_ERR_CUDA;
    if (best_knots_per_s) *best_knots_per_s = best_ms < FLT_MAX ? static_cast<double>(n_knots) / (best_ms * 1e-3) : 0.0;
    return FRG_OK;
}

frg_status frg_get_tuning(const frg_ctx *ctx, frg_tuning *out) {
    if (!ctx || !out) return FRG_ERR_INVALID_ARGUMENT;
    out->warps_per_cta = ctx->shape.warps_per_cta;
    out->lanes_per_knot = ctx->shape.lanes_per_knot;
    out->ragged_warps_per_cta = ctx->ragged_shape.warps_per_cta;
    out->ragged_ctas_per_sm = ctx->ragged_shape.ctas_per_sm;
    out->ragged_lanes_per_knot = ctx->ragged_shape.lanes_per_knot;
    return FRG_OK;
}

frg_status frg_set_tuning(frg_ctx *ctx, const frg_tuning *t) {
    if (!ctx || !t) return FRG_ERR_INVALID_ARGUMENT;
    const int wmax = frg::max_warps_per_cta();
    auto lanes_ok = [](int l) { return l == 1 || l == 8; };
    bool good = t->warps_per_cta >= 1 && t->warps_per_cta <= wmax && lanes_ok(t->lanes_per_knot) &&
                t->ragged_warps_per_cta >= 1 && t->ragged_warps_per_cta <= wmax &&
                lanes_ok(t->ragged_lanes_per_knot) && t->ragged_ctas_per_sm >= 1;
    if (good) {
        DeviceGuard g(ctx->device);
        const int occ = frg::max_ctas_per_sm(t->ragged_warps_per_cta, t->ragged_lanes_per_knot);
        good = occ <= 0 || t->ragged_ctas_per_sm <= occ;
    }
    if (!good) {
        frg_set_error(ctx, "frg_set_tuning: warps per CTA in [1, 8], lanes per knot 1 or 8, resident CTAs per SM "
                           "in [1, occupancy]");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    ctx->shape.warps_per_cta = t->warps_per_cta;
    ctx->shape.lanes_per_knot = t->lanes_per_knot;
    ctx->ragged_shape.warps_per_cta = t->ragged_warps_per_cta;
    ctx->ragged_shape.ctas_per_sm = t->ragged_ctas_per_sm;
    ctx->ragged_shape.lanes_per_knot = t->ragged_lanes_per_knot;
    return FRG_OK;
}

}  // extern "C"
