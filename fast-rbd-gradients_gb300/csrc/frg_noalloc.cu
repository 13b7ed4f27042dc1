// Batched gradient over a ragged offset list that allocates no memory.
//
// Who needs it: callers that must not call cudaMalloc / cudaFree after their
// start-up -- a real-time MPC loop that runs the gradient every control period
// (cudaFree synchronizes the whole device and cudaMalloc can block for an
// unbounded time, which breaks a hard period), and plug-ins living inside a
// host application that owns every byte of device memory and hands them only
// input and output buffers.  The regular batched call allocates its descriptor
// lists on first use (and grows them); this one keeps them in a fixed device
// array that exists from library load until process exit.
//
// The scratch is the file-scope array g_noalloc_scratch below (512 KiB on
// every GPU that loads the library): the persistent kernel's work counter, the
// trajectory descriptors (at most kMaxTraj) and the per-tile segment index (at
// most kMaxTiles 32-knot tiles, i.e. 2,097,152 knots).  Every call shares it
// and it keeps the last call's contents, so each call zeroes the counter
// before its launch, and calls whose launches overlap on the GPU (different
// streams, no ordering between them) race on it: order them on one stream or
// synchronize between them.
#include <cuda_runtime.h>

#include <climits>
#include <mutex>
#include <string>

#include "frg.h"
#include "frg_internal.h"
#include "frg_kernels.cuh"

namespace {

constexpr int kMaxTraj = FRG_NOALLOC_MAX_TRAJ;
constexpr int kMaxTiles = FRG_NOALLOC_MAX_KNOTS / 32;
constexpr size_t kCounterBytes = 256;
constexpr size_t kSegBytes = sizeof(frg::Segment) * (kMaxTraj + 1);
constexpr size_t kSegOffset = kCounterBytes;
constexpr size_t kTileOffset = (kSegOffset + kSegBytes + 255) / 256 * 256;
constexpr size_t kScratchBytes = kTileOffset + sizeof(int) * kMaxTiles;
static_assert(kScratchBytes <= 512 * 1024, "the no-alloc scratch must stay at 512 KiB");

// Device scratch of the no-alloc entry point.  Host code must not use this
// name as an address (it is a host-side stand-in); it uses the address that
// cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[512 * 1024];

// Host-side descriptor staging (static, so building a call allocates nothing).
frg::Segment h_segs[kMaxTraj + 1];
int h_tile_seg[kMaxTiles];
std::mutex g_mu;  // guards the host staging and the per-device set-up table

constexpr int kMaxDevices = 64;
unsigned char *g_dev_scratch[kMaxDevices] = {};

// Once per device, with that device current: the scratch's device address.
// (The persistent kernels' shared-memory opt-in is part of frg_create.)
// Caller holds g_mu.
cudaError_t device_setup(int device, unsigned char **out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    if (!g_dev_scratch[device]) {
        unsigned char *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void **>(&ptr), g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_dev_scratch[device] = ptr;
    }
    *out = g_dev_scratch[device];
    return cudaSuccess;
}

}  // namespace

extern "C" frg_status frg_gradient_ragged_noalloc(frg_ctx *ctx, int n_traj, const int64_t *offsets,
                                                  const float *q, const float *qd, const float *u, float *dqdd,
                                                  float *qdd, float *minv, frg_stream stream) {
    if (!ctx) return FRG_ERR_INVALID_ARGUMENT;
    if (n_traj < 0 || (n_traj > 0 && !offsets)) {
        frg_set_error(ctx, "frg_gradient_ragged_noalloc: bad offset list");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_traj > kMaxTraj) {
        frg_set_error(ctx, "frg_gradient_ragged_noalloc: " + std::to_string(n_traj) +
                               " trajectories exceed the fixed scratch limit of " + std::to_string(kMaxTraj) +
                               " (FRG_NOALLOC_MAX_TRAJ); use frg_gradient_ragged or a plan");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (n_traj > 0 && offsets[0] != 0) {
        frg_set_error(ctx, "frg_gradient_ragged_noalloc: offsets[0] must be 0");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    for (int t = 0; t < n_traj; t++)
        if (offsets[t + 1] < offsets[t]) {
            frg_set_error(ctx, "frg_gradient_ragged_noalloc: offsets must be non-decreasing");
            return FRG_ERR_INVALID_ARGUMENT;
        }
    const int64_t total = n_traj > 0 ? offsets[n_traj] : 0;
    if (total > FRG_NOALLOC_MAX_KNOTS) {
        frg_set_error(ctx, "frg_gradient_ragged_noalloc: " + std::to_string(total) +
                               " knots exceed the fixed scratch limit of " + std::to_string(FRG_NOALLOC_MAX_KNOTS) +
                               " (FRG_NOALLOC_MAX_KNOTS); use frg_gradient_ragged or a plan");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    if (total == 0) return FRG_OK;
    if (!(q && qd && u && dqdd && qdd && minv)) {
        frg_set_error(ctx, "frg_gradient_ragged_noalloc: null array");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    DeviceGuard g(ctx->device);
    std::lock_guard<std::mutex> lock(g_mu);
    unsigned char *base = nullptr;
    cudaError_t e = device_setup(ctx->device, &base);
    if (e != cudaSuccess) {
        cudaGetLastError();
        frg_set_error(ctx, std::string("frg_gradient_ragged_noalloc set-up: ") + cudaGetErrorString(e));
        return FRG_ERR_CUDA;
    }
    // descriptors of the trajectories (same layout as the batched path)
    for (int t = 0; t < n_traj; t++) {
        const int64_t o = offsets[t];
        h_segs[t] = frg::Segment{q + frg::kN * o, qd + frg::kN * o, u + frg::kN * o, dqdd + frg::kDqddN * o, qdd + frg::kN * o, minv + frg::kMinvN * o, o};
    }
    h_segs[n_traj] = frg::Segment{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, total};
    const int ntiles = static_cast<int>((total + 31) / 32);
    int s = 0;
    for (int tile = 0; tile < ntiles; tile++) {
        const long long gk = static_cast<long long>(tile) * 32;
        while (s + 1 < n_traj && h_segs[s + 1].knot_begin <= gk) s++;
        h_tile_seg[tile] = s;
    }
    unsigned int *counter = reinterpret_cast<unsigned int *>(base);
    frg::Segment *segs = reinterpret_cast<frg::Segment *>(base + kSegOffset);
    int *tile_seg = reinterpret_cast<int *>(base + kTileOffset);
    cudaStream_t st = stream;
    // pageable sources: each copy returns once its source has been staged, so
    // the host arrays can be rebuilt by the next call
    if ((e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(segs, h_segs, sizeof(frg::Segment) * (n_traj + 1), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(tile_seg, h_tile_seg, sizeof(int) * ntiles, cudaMemcpyHostToDevice, st)) != cudaSuccess) {
        frg_set_error(ctx, std::string("frg_gradient_ragged_noalloc upload: ") + cudaGetErrorString(e));
        return FRG_ERR_CUDA;
    }
    // the batched path's persistent kernels, at the context's tuned persistent
    // shape and mapping, with descriptors and counter in the static scratch
    e = frg::launch_ragged(ctx->damping, ctx->mpc, ctx->ragged_shape, ctx->num_sms, segs, n_traj, tile_seg, ntiles,
                           counter, st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        frg_set_error(ctx, std::string("frg_gradient_ragged_noalloc launch: ") + cudaGetErrorString(e));
        return FRG_ERR_CUDA;
    }
    return FRG_OK;
}
