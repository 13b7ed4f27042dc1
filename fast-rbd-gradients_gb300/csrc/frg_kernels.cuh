// Kernel launch interface shared by the C ABI and the server (host side).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "frg_dims.h"

namespace frg {

// One trajectory (or any contiguous run of knots) of a ragged batch.  Inputs
// q/qd/u are [n][N], outputs dqdd [n][2N^2], qdd [n][N], minv [n][N^2] (N =
// kN joints, frg_dims.h); knot k
// of the batch is segment s's knot (k - knot_begin).
struct Segment {
    const float *q, *qd, *u;
    float *dqdd, *qdd, *minv;
    long long knot_begin;
};

// One served call: a trajectory of h knots whose device pool slot holds
// [q | qd | u | dqdd | qdd | minv] (kSlotN h floats).  The call's inputs are
// read from q, qd, u ([h][N] each): the trajectory's pinned host slot (copied there
// by submit), its device slot (resident inputs), or the caller's device
// arrays.  Results always go to the device slot, and also to the pinned host
// slot (same layout) when host != nullptr.  Inputs read from anywhere but the
// device slot are mirrored into it, so the next resident call finds them.
struct ServeSegment {
    const float *q, *qd, *u;
    float *dev;
    float *host;
    long long h;
    long long knot_begin;
};

// Launch shape: warps per CTA (each warp owns 32 knots at a time) and, for the
// persistent kernel, resident CTAs per SM.
struct LaunchShape {
    int warps_per_cta = 2;
    int ctas_per_sm = 4;
    int lanes_per_knot = 1;  // 1: knot per lane (throughput), 8: knot per 8 lanes (latency)
};

size_t warp_smem_bytes();
// Opt every kernel variant into the dynamic shared memory it needs (call once
// per device, with that device current).
cudaError_t init_kernels();
int max_warps_per_cta();
// Resident CTAs per SM of the batched kernel at `warps` warps per CTA.
int max_ctas_per_sm(int warps, int lanes_per_knot = 1);

// Plain path: n knots, contiguous arrays, grid over 32-knot tiles.
cudaError_t launch_plain(bool damping, bool mpc, const LaunchShape &shape, int n, const float *q, const float *qd,
                         const float *u, float *dqdd, float *qdd, float *minv, cudaStream_t stream);

// Plain path for results in host memory (pinned, mapped): q, qd, u, qdd and
// minv are read and written in place across the host link; dqdd is computed
// into dqdd_dev (device, [n][2N^2]) and each finished tile is copied to dqdd as
// whole lines.  The latency mapping writes every result in place directly.
// minv_packed (throughput mapping only): minv receives Minv's upper triangle,
// kMinvPackedN floats per knot.
cudaError_t launch_host_out(bool damping, bool mpc, const LaunchShape &shape, int n, const float *q, const float *qd,
                            const float *u, float *dqdd_dev, float *dqdd, float *qdd, float *minv,
                            cudaStream_t stream, bool minv_packed = false);

// Ragged batch: one persistent launch walking 32-knot tiles of the
// concatenated knot list.  segs[nseg + 1] (last = end sentinel with
// knot_begin = total knots), tile_seg[ntiles] = segment of each tile's first
// knot, counter = one device word, zero before the first launch (the kernel
// leaves it zero again).
cudaError_t launch_ragged(bool damping, bool mpc, const LaunchShape &shape, int num_sms, const Segment *segs,
                          int nseg, const int *tile_seg, int ntiles, unsigned int *counter, cudaStream_t stream);

// Server batch: like launch_ragged over ServeSegments (segs[nseg] = end
// sentinel).
cudaError_t launch_serve(bool damping, bool mpc, const LaunchShape &shape, int num_sms, const ServeSegment *segs,
                         int nseg, const int *tile_seg, int ntiles, unsigned int *counter, cudaStream_t stream);
cudaError_t init_serve_kernels();

// Single-knot latency: one warp repeats the whole path over ONE knot `iters`
// times in one launch (lanes_per_knot 1 or 8 selects the thread mapping).
cudaError_t launch_single_knot(bool damping, bool mpc, int lanes_per_knot, int iters, const float *q,
                               const float *qd, const float *u, float *dqdd, float *qdd, float *minv,
                               cudaStream_t stream);

// Latency mapping (8 lanes per knot), same arguments as the launches above.
cudaError_t init_group_kernels();
size_t group_warp_smem_bytes();
int max_group_ctas_per_sm(int warps);
cudaError_t launch_group_plain(bool damping, bool mpc, const LaunchShape &shape, int n, const float *q,
                               const float *qd, const float *u, float *dqdd, float *qdd, float *minv,
                               cudaStream_t stream);
cudaError_t launch_group_single_knot(bool damping, bool mpc, int iters, const float *q, const float *qd,
                                     const float *u, float *dqdd, float *qdd, float *minv, cudaStream_t stream);
cudaError_t launch_group_ragged(bool damping, bool mpc, const LaunchShape &shape, int num_sms, const Segment *segs,
                                int nseg, const int *tile_seg, int ntiles, unsigned int *counter, cudaStream_t stream);
cudaError_t launch_group_serve(bool damping, bool mpc, const LaunchShape &shape, int num_sms, const ServeSegment *segs,
                               int nseg, const int *tile_seg, int ntiles, unsigned int *counter, cudaStream_t stream);

// Plain-path variants (frg_ext_kernels.cu): gradient with external forces
// (fext [n][N][6], link frames), forward dynamics only (fd_only: q̈, optional
// Minv), and the explicit-Euler discrete Jacobians A [n][4N^2], B [n][2N^2].
cudaError_t init_ext_kernels();
cudaError_t launch_ext(bool damping, bool mpc, const LaunchShape &shape, int n, const float *q, const float *qd,
                       const float *u, const float *fext, float *dqdd, float *qdd, float *minv, bool fd_only,
                       cudaStream_t stream);
cudaError_t launch_discretize(int n, const float *dqdd, const float *minv, float dt, float *A, float *B,
                              cudaStream_t stream);
// The reference's packed knot records [n][kKnotRecordFloats]: q, qd, u in;
// q̈ and Minv written into the records; the gradient to dqdd [n][2N^2].
constexpr int kKnotRecordFloats = kRecordN;
cudaError_t launch_knots(bool damping, bool mpc, const LaunchShape &shape, int n, float *knots, float *dqdd,
                         cudaStream_t stream);
// Per-knot non-finite flags (bit 0 inputs, bit 1 outputs; NULL arrays skipped).
cudaError_t launch_knot_status(int num_sms, int n, const float *q, const float *qd, const float *u,
                               const float *dqdd, const float *qdd, const float *minv, unsigned int *status,
                               cudaStream_t stream);

// FP64 verification build (frg_f64_kernels.cu): the plain path in double, and
// the two helpers of the sampled check of FP32 results (float inputs widened to
// out [3][n][N]; per-knot Frobenius-relative errors err [n][3] of FP32 dqdd,
// qdd, minv against FP64 results).
cudaError_t init_f64_kernels();
size_t f64_warp_smem_bytes();
cudaError_t launch_plain_f64(bool damping, bool mpc, int num_sms, long long n, const double *q, const double *qd,
                             const double *u, double *dqdd, double *qdd, double *minv, cudaStream_t stream);
cudaError_t launch_widen_inputs(int num_sms, long long n, const float *q, const float *qd, const float *u,
                                double *out, cudaStream_t stream);
cudaError_t launch_compare_f64(int num_sms, long long n, const float *dqdd, const float *qdd, const float *minv,
                               const double *rdqdd, const double *rqdd, const double *rminv, double *err,
                               cudaStream_t stream);

}  // namespace frg
