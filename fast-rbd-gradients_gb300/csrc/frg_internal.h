// Host-side internals shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "frg.h"
#include "frg_expand.h"
#include "frg_kernels.cuh"

// Makes `device` current for a scope and restores the caller's device.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != device) cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// Descriptor list of a batched launch, built on the host.  When every
// trajectory's arrays follow the previous one's in memory the batch is one
// contiguous run of knots (`whole`) and runs on the plain kernel, without
// per-tile descriptor lookups.
struct HostBatch {
    std::vector<frg::Segment> segs;  // n_traj + 1 (end sentinel)
    std::vector<int> tile_seg;       // one per 32-knot tile
    long long nknots = 0;
    bool contiguous = false;
    frg_traj whole{};
};

// The same list on the device, plus the persistent kernel's work counter.
struct DeviceBatch {
    frg::Segment *segs = nullptr;
    int *tile_seg = nullptr;
    unsigned int *counter = nullptr;
    int seg_cap = 0, tile_cap = 0;
    bool reserve(int nseg_total, int ntiles_cap, std::string &err);
    void release();
};

struct frg_ctx {
    int device = 0;
    bool damping = false, mpc = false;
    frg::LaunchShape shape;         // plain launches (contiguous knots)
    frg::LaunchShape ragged_shape;  // persistent launches over scattered trajectories
    int num_sms = 0;
    std::string err;
    cudaStream_t io_stream = nullptr;   // frg_gradient_host
    float *host_buf = nullptr;          // device staging for frg_gradient_host (dqdd relay / pageable path)
    size_t host_buf_floats = 0;
    cudaStream_t io_stream2 = nullptr;  // frg_gradient_host_batches: odd batches
    float *host_buf2 = nullptr;         // their dqdd relay
    size_t host_buf2_floats = 0;
    // frg_gradient_host_batches: packed Minv of batches j mod 3 (pinned host
    // memory), the event marking each one's launch complete, and the host
    // threads that expand it to dense
    float *minv_stage[3] = {};
    size_t minv_stage_floats = 0;
    cudaEvent_t batch_done[3] = {};
    MinvExpander *expander = nullptr;
    DeviceBatch scratch;                // frg_gradient_batched descriptors
    double *f64_buf = nullptr;          // frg_verify_f64 scratch (frg::kSlotN doubles per knot)
    size_t f64_buf_doubles = 0;
    cudaEvent_t scratch_done = nullptr;  // last launch that read `scratch`
    // frg_plan_launch_many: the extra launch streams, and the events that fork
    // them from the caller's stream and join them back
    static constexpr int kMaxInFlight = 4;
    cudaStream_t flight[kMaxInFlight - 1] = {};
    cudaEvent_t flight_fork = nullptr, flight_join = nullptr;
};

struct frg_plan {
    frg_ctx *ctx = nullptr;
    DeviceBatch dev;
    int nseg = 0, ntiles = 0;
    long long nknots = 0;
    bool contiguous = false;
    frg_traj whole{};
    frg::LaunchShape shape;  // the context's shape when the plan was made
};

void frg_set_error(frg_ctx *ctx, const std::string &msg);
bool frg_build_batch(int n_traj, const frg_traj *trajs, HostBatch &hb, std::string &err);
cudaError_t frg_launch_batch(frg_ctx *ctx, const DeviceBatch &db, int nseg, int ntiles, cudaStream_t stream);
// Plain launch over a contiguous batch (HostBatch::whole).
cudaError_t frg_launch_whole(frg_ctx *ctx, const frg_traj &whole, cudaStream_t stream);
bool frg_offsets_to_trajs(int n_traj, const int64_t *offsets, const float *q, const float *qd, const float *u,
                          float *dqdd, float *qdd, float *minv, std::vector<frg_traj> &out);

namespace frg {
// Launch shape used until the autotuner or the caller picks one: 2-warp CTAs,
// 4 per SM.  The knot-per-lane kernels use up to 255 registers, so each
// quadrant of the register file holds two of their warps (8 per SM); 3-warp
// CTAs would leave only 2 CTAs, 6 warps, resident.
inline LaunchShape default_shape() {
    LaunchShape s;
    s.warps_per_cta = 2;
    s.ctas_per_sm = 4;
    return s;
}
}  // namespace frg
