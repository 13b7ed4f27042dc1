// Server kernel: the batched persistent kernel over served calls.  Each
// call's inputs come from where the call has them -- its pinned host slot
// (read over the host link, coalesced), its resident device slot, or the
// caller's device arrays -- and its results go to the device slot and, when
// asked for, to the host slot, so a batch needs no per-call copy.
#include "frg_kernels.cuh"
#include "frg_knot.cuh"
#include "frg_launch.cuh"
#include "frg_serve.cuh"

namespace frg {

namespace {

template <bool DAMP, bool MPC>
__global__ void __launch_bounds__(8 * 32)
    grad_serve_kernel(const ServeSegment *segs, int nseg, const int *tile_seg, int ntiles, unsigned int *counter) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpSmem *ws = reinterpret_cast<WarpSmem *>(smem_raw) + warp;
    dependent_launch_begin();
    for (unsigned int tile; next_ticket(static_cast<unsigned int>(ntiles), counter, lane, tile);) {
        const long long g = static_cast<long long>(tile) * 32 + lane;
        KnotPtrs kp{}, mr{};
        if (g < segs[nseg].knot_begin) {
            const int s = segment_of(segs, nseg, tile_seg[tile], g);
            serve_knot(segs[s], g - segs[s].knot_begin, kp, mr);
        }
        process_tile<DAMP, MPC, true>(ws, lane, kp, mr);
    }
}

template <bool D, bool M>
cudaError_t set_smem() {
    cudaError_t e = cudaFuncSetAttribute(grad_serve_kernel<D, M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(sizeof(WarpSmem)) * 8);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(grad_serve_kernel<D, M>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                cudaSharedmemCarveoutMaxShared);
}

template <bool D, bool M>
cudaError_t serve_impl(const LaunchShape &sh, int num_sms, const ServeSegment *segs, int nseg, const int *tile_seg,
                       int ntiles, unsigned int *counter, cudaStream_t st) {
    const int warps = sh.warps_per_cta;
    int grid = num_sms * sh.ctas_per_sm;
    const int needed = (ntiles + warps - 1) / warps;
    if (grid > needed) grid = needed;
    if (grid < 1) grid = 1;
    return launch_dependent(grad_serve_kernel<D, M>, dim3(grid), dim3(warps * 32), sizeof(WarpSmem) * warps, st, segs,
                            nseg, tile_seg, ntiles, counter);
}

}  // namespace

cudaError_t init_serve_kernels() {
    cudaError_t e = cudaSuccess;
    for (cudaError_t r : {set_smem<false, false>(), set_smem<true, false>(), set_smem<false, true>(),
                          set_smem<true, true>()})
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    return e;
}

cudaError_t launch_serve(bool damping, bool mpc, const LaunchShape &shape, int num_sms, const ServeSegment *segs,
                         int nseg, const int *tile_seg, int ntiles, unsigned int *counter, cudaStream_t stream) {
    if (ntiles <= 0) return cudaSuccess;
    if (shape.warps_per_cta < 1 || shape.warps_per_cta > 8 || shape.ctas_per_sm < 1) return cudaErrorInvalidValue;
    if (shape.lanes_per_knot == 8)
        return launch_group_serve(damping, mpc, shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
    if (!damping && !mpc) return serve_impl<false, false>(shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
    if (damping && !mpc) return serve_impl<true, false>(shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
    if (!damping && mpc) return serve_impl<false, true>(shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
    return serve_impl<true, true>(shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
}

}  // namespace frg
