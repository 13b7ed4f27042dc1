// sm_103a kernels for the iiwa_14 forward-dynamics gradient.
//
// Replaces the reference's dynamicsGradientKernel (helpers_GPU/
// dynamicsGradient.cuh:1259-1290: one knot per 224-thread CTA, ~50 block
// barriers per knot, q̈ and Minv computed on the host) with one knot per lane,
// q̈ and Minv computed on the device, and no block barrier at all.
#include "frg_kernels.cuh"
#include "frg_knot.cuh"
#include "frg_launch.cuh"

namespace frg {

namespace {

constexpr int kMaxWarpsPerCta = 8;
// 227 KB of shared memory per CTA: eight warps' staging fits for every
// supported joint count (28.9 KB per warp at 8 joints, 24.4 KB at 7)
static_assert(kMaxWarpsPerCta * sizeof(WarpSmem) <= 227 * 1024, "eight warps must fit one CTA");

struct PlainArgs {
    const float *q, *qd, *u;
    float *dqdd, *qdd, *minv;
    int n;
    float *dqdd_relay = nullptr;  // RELAY: final dqdd destination (host memory)
};

template <bool MINV_PACKED = false>
__device__ __forceinline__ KnotPtrs plain_knot(const PlainArgs &a, int tile, int lane) {
    const long long g = static_cast<long long>(tile) * 32 + lane;
    if (g >= a.n) return KnotPtrs{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    constexpr int minv_stride = MINV_PACKED ? kMinvPackedN : kMinvN;
    return KnotPtrs{a.q + kN * g,       a.qd + kN * g,  a.u + kN * g,
                    a.dqdd + kDqddN * g, a.qdd + kN * g, a.minv + minv_stride * g};
}
static_assert(kMinvPackedN == kMinvPackedFloats, "host and kernel agree on the packed Minv width");

// Floats of `p` that precede it in its 128-byte line.  A warp loop over
// e = lane - line_shift(p) + 32 m stores exactly one whole line per step,
// which keeps stores to memory that is off 16-byte alignment at full rate
// over the host link (partial lines cost about 30 % there).
__device__ __forceinline__ int line_shift(const float *p) {
    return static_cast<int>((reinterpret_cast<unsigned long long>(p) & 127ull) / sizeof(float));
}

// Copies a finished tile's dqdd rows (2N^2 floats per knot, contiguous) from
// the device array to their final place.  Over the host link only whole
// aligned lines write at full rate: the two N^2-float halves at a 2N^2-float
// stride that process_tile stores run at about 60 % of it, so host results go
// through device memory (where the tile is still in L2) and leave as one
// contiguous 12.5 KB run of 16-byte stores.
__device__ __forceinline__ void relay_dqdd(const PlainArgs &a, int tile, int lane) {
    const long long k0 = static_cast<long long>(tile) * 32;
    const int m = a.n - k0 < 32 ? static_cast<int>(a.n - k0) : 32;
    const float *src = a.dqdd + kDqddN * k0;  // written by this warp: plain loads, not the read-only path
    float *dst = a.dqdd_relay + kDqddN * k0;
    if (m == 32 && aligned16(src) && aligned16(dst)) {
        const float4 *s4 = reinterpret_cast<const float4 *>(src);
        float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll 5
        for (int e = lane; e < kDqddN * 32 / 4; e += 32) d4[e] = s4[e];
    } else {
        for (int e = lane - line_shift(dst); e < kDqddN * m; e += 32)
            if (e >= 0) dst[e] = src[e];
    }
    __syncwarp();
}

// MINV_PACKED (host-buffer batches only): a.minv receives Minv's packed
// upper triangle, kMinvPackedN floats per knot.
template <bool DAMP, bool MPC, bool RELAY = false, bool MINV_PACKED = false>
__global__ void __launch_bounds__(kMaxWarpsPerCta * 32) grad_plain_kernel(PlainArgs a) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpSmem *ws = reinterpret_cast<WarpSmem *>(smem_raw) + warp;
    const int warps_per_cta = blockDim.x >> 5;
    const int ntiles = (a.n + 31) / 32;
    // inputs in device memory: the first tile's into L2 while the work ahead finishes
    if (!RELAY && blockIdx.x * warps_per_cta + warp < ntiles)
        prefetch_knot_inputs(plain_knot<MINV_PACKED>(a, blockIdx.x * warps_per_cta + warp, lane));
    dependent_launch_begin();
    for (int tile = blockIdx.x * warps_per_cta + warp; tile < ntiles; tile += gridDim.x * warps_per_cta) {
        const KnotPtrs kp = plain_knot<MINV_PACKED>(a, tile, lane);
        process_tile<DAMP, MPC, false, false, false, MINV_PACKED>(ws, lane, kp);
        // scatter_out ended with __syncwarp: every lane's dqdd stores are visible to the warp
        if constexpr (RELAY) relay_dqdd(a, tile, lane);
    }
}

__device__ __forceinline__ KnotPtrs ragged_knot(const Segment *segs, int nseg, const int *tile_seg, int tile,
                                                int lane) {
    const long long g = static_cast<long long>(tile) * 32 + lane;
    if (g >= segs[nseg].knot_begin) return KnotPtrs{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const Segment &sg = segs[segment_of(segs, nseg, tile_seg[tile], g)];
    const long long i = g - sg.knot_begin;
    return KnotPtrs{sg.q + kN * i, sg.qd + kN * i, sg.u + kN * i, sg.dqdd + kDqddN * i, sg.qdd + kN * i, sg.minv + kMinvN * i};
}

// Persistent: each warp takes 32-knot tiles from a device work counter until
// the list is exhausted (next_ticket).
template <bool DAMP, bool MPC>
__global__ void __launch_bounds__(kMaxWarpsPerCta * 32)
    grad_ragged_kernel(const Segment *segs, int nseg, const int *tile_seg, int ntiles, unsigned int *counter) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpSmem *ws = reinterpret_cast<WarpSmem *>(smem_raw) + warp;
    // The tile this warp is likely to draw first (warps draw their first
    // tickets in about this order) has its inputs brought into L2 while the
    // work ahead finishes.  The descriptors it reads are written only by the
    // host, by copies that the launch waits for in full.
    const int first = blockIdx.x * (blockDim.x >> 5) + warp;
    if (first < ntiles) prefetch_knot_inputs(ragged_knot(segs, nseg, tile_seg, first, lane));
    dependent_launch_begin();  // before the first ticket: the previous launch of this list resets the counter
    for (unsigned int tile; next_ticket(static_cast<unsigned int>(ntiles), counter, lane, tile);)
        process_tile<DAMP, MPC>(ws, lane, ragged_knot(segs, nseg, tile_seg, static_cast<int>(tile), lane));
}

// Single-knot latency (the reference's kern_single_full, time_GPU.cu:23-51,
// which repeats one knot TEST_ITERS times inside one CTA): one warp carries
// one knot (lane 0) through the whole path `iters` times in a row, each time
// exactly as a one-knot launch does -- gather, arithmetic, scatter of every
// result.  Repetition i reads the knot at an offset of (i & zero) knots;
// `zero` is 0 at run time, but the compiler cannot know it, so no repetition
// can be hoisted out of the loop.
template <bool DAMP, bool MPC>
__global__ void __launch_bounds__(32) grad_single_knot_kernel(PlainArgs a, int iters, int zero) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & 31;
    WarpSmem *ws = reinterpret_cast<WarpSmem *>(smem_raw);
    for (int i = 0; i < iters; i++) {
        const long long o = static_cast<long long>(i & zero);
        const KnotPtrs kp = lane == 0 ? KnotPtrs{a.q + kN * o, a.qd + kN * o, a.u + kN * o, a.dqdd + kDqddN * o,
                                                 a.qdd + kN * o, a.minv + kMinvN * o}
                                      : KnotPtrs{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
        process_tile<DAMP, MPC>(ws, lane, kp);
    }
}

template <typename K>
cudaError_t prepare(K kernel) {
    static_assert(sizeof(WarpSmem) % 16 == 0, "warp smem must keep float4 alignment");
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(sizeof(WarpSmem)) * kMaxWarpsPerCta);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                cudaSharedmemCarveoutMaxShared);
}

template <bool D, bool M, bool R = false, bool P = false>
cudaError_t plain_impl(const LaunchShape &sh, const PlainArgs &a, cudaStream_t st) {
    const int warps = sh.warps_per_cta;
    const int ntiles = (a.n + 31) / 32;
    const int grid = (ntiles + warps - 1) / warps;
    return launch_dependent(grad_plain_kernel<D, M, R, P>, dim3(grid), dim3(warps * 32), sizeof(WarpSmem) * warps, st,
                            a);
}

template <bool D, bool M>
cudaError_t ragged_impl(const LaunchShape &sh, int num_sms, const Segment *segs, int nseg, const int *tile_seg,
                        int ntiles, unsigned int *counter, cudaStream_t st) {
    const int warps = sh.warps_per_cta;
    int grid = num_sms * sh.ctas_per_sm;
    const int needed = (ntiles + warps - 1) / warps;
    if (grid > needed) grid = needed;
    if (grid < 1) grid = 1;
    return launch_dependent(grad_ragged_kernel<D, M>, dim3(grid), dim3(warps * 32), sizeof(WarpSmem) * warps, st, segs,
                            nseg, tile_seg, ntiles, counter);
}

}  // namespace

size_t warp_smem_bytes() { return sizeof(WarpSmem); }

cudaError_t init_kernels() {
    cudaError_t e = cudaSuccess;
    for (cudaError_t r : {prepare(grad_plain_kernel<false, false>), prepare(grad_plain_kernel<true, false>),
                          prepare(grad_plain_kernel<false, true>), prepare(grad_plain_kernel<true, true>),
                          prepare(grad_plain_kernel<false, false, true>), prepare(grad_plain_kernel<true, false, true>),
                          prepare(grad_plain_kernel<false, true, true>), prepare(grad_plain_kernel<true, true, true>),
                          prepare(grad_plain_kernel<false, false, true, true>),
                          prepare(grad_plain_kernel<true, false, true, true>),
                          prepare(grad_plain_kernel<false, true, true, true>),
                          prepare(grad_plain_kernel<true, true, true, true>),
                          prepare(grad_ragged_kernel<false, false>), prepare(grad_ragged_kernel<true, false>),
                          prepare(grad_ragged_kernel<false, true>), prepare(grad_ragged_kernel<true, true>)})
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    return e;
}
int max_warps_per_cta() { return kMaxWarpsPerCta; }

int max_ctas_per_sm(int warps, int lanes_per_knot) {
    if (lanes_per_knot == 8) return max_group_ctas_per_sm(warps);
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, grad_ragged_kernel<false, false>, warps * 32,
                                                      sizeof(WarpSmem) * warps) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return blocks;
}

cudaError_t launch_plain(bool damping, bool mpc, const LaunchShape &shape, int n, const float *q, const float *qd,
                         const float *u, float *dqdd, float *qdd, float *minv, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    if (shape.warps_per_cta < 1 || shape.warps_per_cta > kMaxWarpsPerCta) return cudaErrorInvalidValue;
    if (shape.lanes_per_knot == 8) return launch_group_plain(damping, mpc, shape, n, q, qd, u, dqdd, qdd, minv, stream);
    const PlainArgs a{q, qd, u, dqdd, qdd, minv, n};
    if (!damping && !mpc) return plain_impl<false, false>(shape, a, stream);
    if (damping && !mpc) return plain_impl<true, false>(shape, a, stream);
    if (!damping && mpc) return plain_impl<false, true>(shape, a, stream);
    return plain_impl<true, true>(shape, a, stream);
}

cudaError_t launch_host_out(bool damping, bool mpc, const LaunchShape &shape, int n, const float *q, const float *qd,
                            const float *u, float *dqdd_dev, float *dqdd, float *qdd, float *minv,
                            cudaStream_t stream, bool minv_packed) {
    if (n <= 0) return cudaSuccess;
    if (shape.warps_per_cta < 1 || shape.warps_per_cta > kMaxWarpsPerCta) return cudaErrorInvalidValue;
    if (shape.lanes_per_knot == 8) {  // small batches: latency first, every result straight to its destination
        if (minv_packed) return cudaErrorInvalidValue;
        return launch_group_plain(damping, mpc, shape, n, q, qd, u, dqdd, qdd, minv, stream);
    }
    PlainArgs a{q, qd, u, dqdd_dev, qdd, minv, n};
    a.dqdd_relay = dqdd;
    if (minv_packed) {
        if (!damping && !mpc) return plain_impl<false, false, true, true>(shape, a, stream);
        if (damping && !mpc) return plain_impl<true, false, true, true>(shape, a, stream);
        if (!damping && mpc) return plain_impl<false, true, true, true>(shape, a, stream);
        return plain_impl<true, true, true, true>(shape, a, stream);
    }
    if (!damping && !mpc) return plain_impl<false, false, true>(shape, a, stream);
    if (damping && !mpc) return plain_impl<true, false, true>(shape, a, stream);
    if (!damping && mpc) return plain_impl<false, true, true>(shape, a, stream);
    return plain_impl<true, true, true>(shape, a, stream);
}

cudaError_t launch_single_knot(bool damping, bool mpc, int lanes_per_knot, int iters, const float *q,
                               const float *qd, const float *u, float *dqdd, float *qdd, float *minv,
                               cudaStream_t stream) {
    if (iters <= 0) return cudaSuccess;
    if (lanes_per_knot == 8) return launch_group_single_knot(damping, mpc, iters, q, qd, u, dqdd, qdd, minv, stream);
    if (lanes_per_knot != 1) return cudaErrorInvalidValue;
    const PlainArgs a{q, qd, u, dqdd, qdd, minv, 1};
    const size_t smem = sizeof(WarpSmem);
    if (!damping && !mpc) grad_single_knot_kernel<false, false><<<1, 32, smem, stream>>>(a, iters, 0);
    else if (damping && !mpc) grad_single_knot_kernel<true, false><<<1, 32, smem, stream>>>(a, iters, 0);
    else if (!damping && mpc) grad_single_knot_kernel<false, true><<<1, 32, smem, stream>>>(a, iters, 0);
    else grad_single_knot_kernel<true, true><<<1, 32, smem, stream>>>(a, iters, 0);
    return cudaGetLastError();
}

cudaError_t launch_ragged(bool damping, bool mpc, const LaunchShape &shape, int num_sms, const Segment *segs,
                          int nseg, const int *tile_seg, int ntiles, unsigned int *counter, cudaStream_t stream) {
    if (ntiles <= 0) return cudaSuccess;
    if (shape.warps_per_cta < 1 || shape.warps_per_cta > kMaxWarpsPerCta || shape.ctas_per_sm < 1)
        return cudaErrorInvalidValue;
    if (shape.lanes_per_knot == 8)
        return launch_group_ragged(damping, mpc, shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
    if (!damping && !mpc) return ragged_impl<false, false>(shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
    if (damping && !mpc) return ragged_impl<true, false>(shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
    if (!damping && mpc) return ragged_impl<false, true>(shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
    return ragged_impl<true, true>(shape, num_sms, segs, nseg, tile_seg, ntiles, counter, stream);
}

}  // namespace frg
