// Kernels of the latency mapping (8 lanes per knot, frg_knot_group.cuh).
// They take the same launch arguments as the knot-per-lane kernels; a warp's
// work item is a 4-knot slice, 8 slices per 32-knot tile, so a small batch is
// spread over 8x more warps.
#include "frg_kernels.cuh"
#include "frg_knot_group.cuh"
#include "frg_launch.cuh"
#include "frg_serve.cuh"

namespace frg {

namespace {

constexpr int kMaxWarps = 8;

__device__ __forceinline__ KnotPtrs plain_group_knot(const float *q, const float *qd, const float *u, float *dqdd,
                                                     float *qdd, float *minv, int n, long long item, int lane) {
    const long long g = item * kGroupKnots + (lane >> 3);
    if (g >= n) return KnotPtrs{};
    return KnotPtrs{q + kN * g, qd + kN * g, u + kN * g, dqdd + kDqddN * g, qdd + kN * g, minv + kMinvN * g};
}

template <bool DAMP, bool MPC>
__global__ void __launch_bounds__(kMaxWarps * 32)
    grad_group_plain_kernel(const float *q, const float *qd, const float *u, float *dqdd, float *qdd, float *minv,
                            int n) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    GroupSmem *gs = reinterpret_cast<GroupSmem *>(smem_raw) + warp;
    const long long items = (static_cast<long long>(n) + kGroupKnots - 1) / kGroupKnots;
    const int wpc = blockDim.x >> 5;
    // the first slice's inputs into L2 while the work ahead finishes (prefetch_l2)
    if (static_cast<long long>(blockIdx.x) * wpc + warp < items)
        prefetch_knot_inputs(plain_group_knot(q, qd, u, dqdd, qdd, minv, n, static_cast<long long>(blockIdx.x) * wpc + warp,
                                              lane));
    dependent_launch_begin();
    for (long long it = static_cast<long long>(blockIdx.x) * wpc + warp; it < items;
         it += static_cast<long long>(gridDim.x) * wpc)
        process_group<DAMP, MPC>(gs, lane, plain_group_knot(q, qd, u, dqdd, qdd, minv, n, it, lane));
}

// Single-knot latency in this mapping: one warp, knot slot 0 (lanes 0-7)
// carries one knot through the whole path `iters` times; the (i & zero) knot
// offset keeps every repetition in the loop (see grad_single_knot_kernel).
template <bool DAMP, bool MPC>
__global__ void __launch_bounds__(32)
    grad_group_single_knot_kernel(const float *q, const float *qd, const float *u, float *dqdd, float *qdd,
                                  float *minv, int iters, int zero) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & 31;
    GroupSmem *gs = reinterpret_cast<GroupSmem *>(smem_raw);
    for (int i = 0; i < iters; i++) {
        const long long o = static_cast<long long>(i & zero);
        process_group<DAMP, MPC>(gs, lane, plain_group_knot(q + kN * o, qd + kN * o, u + kN * o, dqdd + kDqddN * o,
                                                            qdd + kN * o, minv + kMinvN * o, 1, 0, lane));
    }
}

// persistent (next_ticket): ticket -> (32-knot tile t, 4-knot slice s)
template <bool DAMP, bool MPC, bool SERVE, typename Seg>
__device__ __forceinline__ void group_persistent(const Seg *segs, int nseg, const int *tile_seg, int ntiles,
                                                 unsigned int *counter) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    GroupSmem *gs = reinterpret_cast<GroupSmem *>(smem_raw) + warp;
    const unsigned int items = static_cast<unsigned int>(ntiles) * 8u;
    if constexpr (!SERVE) {
        // the slice this warp is likely to draw first: its inputs into L2 while
        // the work ahead finishes (descriptors are written only by host copies
        // that the launch waits for in full; see grad_ragged_kernel)
        const unsigned int first = blockIdx.x * (blockDim.x >> 5) + warp;
        if (first < items) {
            const int tile = static_cast<int>(first >> 3), slice = static_cast<int>(first & 7u);
            const long long g = static_cast<long long>(tile) * 32 + slice * kGroupKnots + (lane >> 3);
            if (g < segs[nseg].knot_begin) {
                const Seg &sg = segs[segment_of(segs, nseg, tile_seg[tile], g)];
                const long long i = g - sg.knot_begin;
                prefetch_knot_inputs(KnotPtrs{sg.q + kN * i, sg.qd + kN * i, sg.u + kN * i, nullptr, nullptr, nullptr});
            }
        }
    }
    dependent_launch_begin();
    for (unsigned int ticket; next_ticket(items, counter, lane, ticket);) {
        const int tile = static_cast<int>(ticket >> 3), slice = static_cast<int>(ticket & 7u);
        const long long g = static_cast<long long>(tile) * 32 + slice * kGroupKnots + (lane >> 3);
        KnotPtrs kp{}, mr{};
        if (g < segs[nseg].knot_begin) {
            const Seg &sg = segs[segment_of(segs, nseg, tile_seg[tile], g)];
            const long long i = g - sg.knot_begin;
            if constexpr (SERVE) {
                serve_knot(sg, i, kp, mr);
            } else {
                kp = KnotPtrs{sg.q + kN * i, sg.qd + kN * i, sg.u + kN * i, sg.dqdd + kDqddN * i, sg.qdd + kN * i,
                              sg.minv + kMinvN * i};
            }
        }
        process_group<DAMP, MPC, SERVE>(gs, lane, kp, mr);
    }
}

template <bool DAMP, bool MPC>
__global__ void __launch_bounds__(kMaxWarps * 32)
    grad_group_ragged_kernel(const Segment *segs, int nseg, const int *tile_seg, int ntiles, unsigned int *counter) {
    group_persistent<DAMP, MPC, false>(segs, nseg, tile_seg, ntiles, counter);
}

template <bool DAMP, bool MPC>
__global__ void __launch_bounds__(kMaxWarps * 32)
    grad_group_serve_kernel(const ServeSegment *segs, int nseg, const int *tile_seg, int ntiles,
                            unsigned int *counter) {
    group_persistent<DAMP, MPC, true>(segs, nseg, tile_seg, ntiles, counter);
}

template <typename K>
cudaError_t opt_in(K kernel) {
    static_assert(sizeof(GroupSmem) % 16 == 0, "group smem must keep float4 alignment");
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(sizeof(GroupSmem)) * kMaxWarps);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
}

int persistent_grid(const LaunchShape &sh, int num_sms, long long items) {
    long long grid = static_cast<long long>(num_sms) * sh.ctas_per_sm;
    const long long needed = (items + sh.warps_per_cta - 1) / sh.warps_per_cta;
    if (grid > needed) grid = needed;
    return grid < 1 ? 1 : static_cast<int>(grid);
}

}  // namespace

cudaError_t init_group_kernels() {
    cudaError_t e = cudaSuccess;
    for (cudaError_t r : {opt_in(grad_group_plain_kernel<false, false>), opt_in(grad_group_plain_kernel<true, false>),
                          opt_in(grad_group_plain_kernel<false, true>), opt_in(grad_group_plain_kernel<true, true>),
                          opt_in(grad_group_ragged_kernel<false, false>), opt_in(grad_group_ragged_kernel<true, false>),
                          opt_in(grad_group_ragged_kernel<false, true>), opt_in(grad_group_ragged_kernel<true, true>),
                          opt_in(grad_group_serve_kernel<false, false>), opt_in(grad_group_serve_kernel<true, false>),
                          opt_in(grad_group_serve_kernel<false, true>), opt_in(grad_group_serve_kernel<true, true>)})
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    return e;
}

size_t group_warp_smem_bytes() { return sizeof(GroupSmem); }

int max_group_ctas_per_sm(int warps) {
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, grad_group_ragged_kernel<false, false>, warps * 32,
                                                      sizeof(GroupSmem) * warps) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return blocks;
}

#define FRG_DISPATCH(D, M, CALL) \
    if (!(D) && !(M)) CALL(false, false) else if ((D) && !(M)) CALL(true, false) else if (!(D) && (M)) CALL(false, true) else CALL(true, true)

cudaError_t launch_group_plain(bool damping, bool mpc, const LaunchShape &sh, int n, const float *q, const float *qd,
                               const float *u, float *dqdd, float *qdd, float *minv, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int w = sh.warps_per_cta;
    const long long items = (static_cast<long long>(n) + kGroupKnots - 1) / kGroupKnots;
    const int grid = static_cast<int>((items + w - 1) / w);
    const size_t smem = sizeof(GroupSmem) * w;
#define FRG_CALL(D, M) \
    return launch_dependent(grad_group_plain_kernel<D, M>, dim3(grid), dim3(w * 32), smem, st, q, qd, u, dqdd, qdd, minv, n);
    FRG_DISPATCH(damping, mpc, FRG_CALL)
#undef FRG_CALL
}

cudaError_t launch_group_single_knot(bool damping, bool mpc, int iters, const float *q, const float *qd,
                                     const float *u, float *dqdd, float *qdd, float *minv, cudaStream_t st) {
    if (iters <= 0) return cudaSuccess;
    const size_t smem = sizeof(GroupSmem);
#define FRG_CALL(D, M) grad_group_single_knot_kernel<D, M><<<1, 32, smem, st>>>(q, qd, u, dqdd, qdd, minv, iters, 0);
    FRG_DISPATCH(damping, mpc, FRG_CALL)
#undef FRG_CALL
    return cudaGetLastError();
}

cudaError_t launch_group_ragged(bool damping, bool mpc, const LaunchShape &sh, int num_sms, const Segment *segs,
                                int nseg, const int *tile_seg, int ntiles, unsigned int *counter, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    const int w = sh.warps_per_cta, grid = persistent_grid(sh, num_sms, static_cast<long long>(ntiles) * 8);
    const size_t smem = sizeof(GroupSmem) * w;
#define FRG_CALL(D, M) \
    return launch_dependent(grad_group_ragged_kernel<D, M>, dim3(grid), dim3(w * 32), smem, st, segs, nseg, tile_seg, \
                            ntiles, counter);
    FRG_DISPATCH(damping, mpc, FRG_CALL)
#undef FRG_CALL
}

cudaError_t launch_group_serve(bool damping, bool mpc, const LaunchShape &sh, int num_sms, const ServeSegment *segs,
                               int nseg, const int *tile_seg, int ntiles, unsigned int *counter, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    const int w = sh.warps_per_cta, grid = persistent_grid(sh, num_sms, static_cast<long long>(ntiles) * 8);
    const size_t smem = sizeof(GroupSmem) * w;
#define FRG_CALL(D, M) \
    return launch_dependent(grad_group_serve_kernel<D, M>, dim3(grid), dim3(w * 32), smem, st, segs, nseg, tile_seg, \
                            ntiles, counter);
    FRG_DISPATCH(damping, mpc, FRG_CALL)
#undef FRG_CALL
}

}  // namespace frg
