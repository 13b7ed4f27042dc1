// Plain-path variants either side of the gradient:
//   - the gradient with external link forces (fext, the s_fext of the
//     reference's RNEA_fp, helpers_CPU/dynamicsGradient.h:654-657);
//   - forward dynamics only: q̈ and Minv (forwardDynamics, :686-706);
//   - discrete-time Jacobians of one explicit-Euler step from the gradient:
//       x = [q; qd],  x+ = x + dt [qd; q̈(q, qd, u)]
//       A = dx+/dx = I + dt [0 I; dq̈/dq dq̈/dqd]   (2N x 2N, column-major)
//       B = dx+/du = dt [0; Minv]                 (2N x N, column-major)
//   - the gradient over the reference's packed knot records (knot<T>,
//     helpers_CPU/dynamicsGradient.h:19-25): [q | qd | u | qdd | Minv],
//     4N + N^2 floats per knot (77 for 7 joints), q̈ and Minv written back
//     into the records.
// N = kN joints (frg_dims.h).
#include "frg_kernels.cuh"
#include "frg_knot.cuh"
#include "frg_launch.cuh"

namespace frg {

namespace {

template <bool DAMP, bool MPC, bool FEXT, bool FDONLY>
__global__ void __launch_bounds__(8 * 32)
    grad_ext_kernel(const float *q, const float *qd, const float *u, const float *fext, float *dqdd, float *qdd,
                    float *minv, int n) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpSmem *ws = reinterpret_cast<WarpSmem *>(smem_raw) + warp;
    const int wpc = blockDim.x >> 5, ntiles = (n + 31) / 32;
    auto knot = [&](int tile) {
        const long long g = static_cast<long long>(tile) * 32 + lane;
        if (g >= n) return KnotPtrs{};
        return KnotPtrs{q + kN * g, qd + kN * g, u + kN * g, dqdd ? dqdd + kDqddN * g : nullptr, qdd + kN * g,
                        minv ? minv + kMinvN * g : nullptr, FEXT ? fext + kFextN * g : nullptr};
    };
    if (blockIdx.x * wpc + warp < ntiles) {  // the first tile's inputs into L2 while the work ahead finishes
        const KnotPtrs kp = knot(blockIdx.x * wpc + warp);
        prefetch_knot_inputs(kp);
        if (FEXT && kp.fext) {
            prefetch_l2(kp.fext);
            prefetch_l2(kp.fext + kFextN - 1);
        }
    }
    dependent_launch_begin();
    for (int tile = blockIdx.x * wpc + warp; tile < ntiles; tile += gridDim.x * wpc)
        process_tile<DAMP, MPC, false, FEXT, FDONLY>(ws, lane, knot(tile));
}

// Knot records [n][4N + N^2]: q, qd, u read from each record, q̈ and Minv
// written into its qdd and Minv fields, the gradient to dqdd [n][2N^2].  The records are
// not tile-contiguous per array, so gather and scatter resolve every knot's
// address; inputs are staged before any output is written, and the fields do
// not overlap.
template <bool DAMP, bool MPC>
__global__ void __launch_bounds__(8 * 32) grad_knots_kernel(float *knots, float *dqdd, int n) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpSmem *ws = reinterpret_cast<WarpSmem *>(smem_raw) + warp;
    const int wpc = blockDim.x >> 5, ntiles = (n + 31) / 32;
    auto knot = [&](int tile) {
        const long long g = static_cast<long long>(tile) * 32 + lane;
        if (g >= n) return KnotPtrs{};
        float *rec = knots + kKnotRecordFloats * g;
        return KnotPtrs{rec, rec + kN, rec + 2 * kN, dqdd + kDqddN * g, rec + 3 * kN, rec + 4 * kN};
    };
    if (blockIdx.x * wpc + warp < ntiles)  // the first tile's inputs into L2 while the work ahead finishes
        prefetch_knot_inputs(knot(blockIdx.x * wpc + warp));
    dependent_launch_begin();
    for (int tile = blockIdx.x * wpc + warp; tile < ntiles; tile += gridDim.x * wpc)
        process_tile<DAMP, MPC>(ws, lane, knot(tile));
}

// One thread per output float: A [n][4N^2] then B [n][2N^2].
__global__ void discretize_kernel(int n, const float *dqdd, const float *minv, float dt, float *A, float *B) {
    constexpr int N2 = 2 * kN, NA = N2 * N2, NB = N2 * kN;  // 2N rows; A and B floats per knot
    const long long total = static_cast<long long>(n) * (NA + NB);
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (e < static_cast<long long>(n) * NA) {
            const long long k = e / NA;
            const int idx = static_cast<int>(e - k * NA), r = idx % N2, c = idx / N2;
            float v;
            if (r < kN) v = (c == r + kN) ? dt : 0.0f;  // dq+/dqd = dt I
            else v = dt * dqdd[kDqddN * k + (r - kN) + kN * c];
            A[e] = v + (r == c ? 1.0f : 0.0f);
        } else {
            const long long e2 = e - static_cast<long long>(n) * NA, k = e2 / NB;
            const int idx = static_cast<int>(e2 - k * NB), r = idx % N2, c = idx / N2;
            B[e2] = r < kN ? 0.0f : dt * minv[kMinvN * k + (r - kN) + kN * c];
        }
    }
}

// The same per 64-knot chunk, for 16-byte-aligned arrays.  The chunk's dqdd
// and Minv (25,088 B and 12,544 B for 7 joints) are staged in shared memory
// with 16-byte loads; A and B leave as 16-byte stores, coalesced.  A knot's A
// and a knot pair's B are N^2 float4 each (49 for 7 joints); each thread owns
// one float4 position j of both, so the element arithmetic is done once per
// thread and the loops over the chunk's knots only load, scale and store.
// The expressions per element are those of discretize_kernel, so the bits are
// too.
constexpr int kDiscKnots = 64;
__global__ void __launch_bounds__(256) discretize_chunks_kernel(int nchunks, const float *dqdd, const float *minv,
                                                                float dt, float *A, float *B) {
    constexpr int N2 = 2 * kN, Q = kN * kN;  // float4 per knot's A and per knot pair's B
    __shared__ float4 s_dqdd4[kDiscKnots * kDqddN / 4];
    __shared__ float4 s_minv4[kDiscKnots * kMinvN / 4];
    const float *s_dqdd = reinterpret_cast<const float *>(s_dqdd4);
    const float *s_minv = reinterpret_cast<const float *>(s_minv4);
    const int ngroups = blockDim.x / Q;  // groups of Q threads
    const int g = threadIdx.x / Q, j = threadIdx.x - g * Q;
    int asrc[4], bsrc[4];  // offset into the knot's dqdd / the knot pair's Minv, or -1
    float aconst[4], aone[4];
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const int idx = 4 * j + t, r = idx % N2, c = idx / N2;  // A element (r, c) of 2N x 2N
        asrc[t] = r < kN ? -1 : (r - kN) + kN * c;
        aconst[t] = r < kN && c == r + kN ? dt : 0.0f;
        aone[t] = r == c ? 1.0f : 0.0f;
        const int kp = idx / kDqddN, bi = idx - kp * kDqddN, br = bi % N2, bc = bi / N2;  // B element of knot kp
        bsrc[t] = br < kN ? -1 : kMinvN * kp + (br - kN) + kN * bc;
    }
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const long long k0 = static_cast<long long>(ch) * kDiscKnots;
        const float4 *gd = reinterpret_cast<const float4 *>(dqdd + kDqddN * k0);
        const float4 *gm = reinterpret_cast<const float4 *>(minv + kMinvN * k0);
        for (int i = threadIdx.x; i < kDiscKnots * kDqddN / 4; i += blockDim.x) s_dqdd4[i] = __ldg(gd + i);
        for (int i = threadIdx.x; i < kDiscKnots * kMinvN / 4; i += blockDim.x) s_minv4[i] = __ldg(gm + i);
        __syncthreads();
        if (g < ngroups) {
            float4 *gA = reinterpret_cast<float4 *>(A + 4 * Q * k0);
            for (int kk = g; kk < kDiscKnots; kk += ngroups) {
                float v[4];
#pragma unroll
                for (int t = 0; t < 4; t++)
                    v[t] = (asrc[t] >= 0 ? dt * s_dqdd[kDqddN * kk + asrc[t]] : aconst[t]) + aone[t];
                gA[Q * kk + j] = make_float4(v[0], v[1], v[2], v[3]);
            }
            float4 *gB = reinterpret_cast<float4 *>(B + kDqddN * k0);
            for (int kp = g; kp < kDiscKnots / 2; kp += ngroups) {
                float v[4];
#pragma unroll
                for (int t = 0; t < 4; t++) v[t] = bsrc[t] >= 0 ? dt * s_minv[kDqddN * kp + bsrc[t]] : 0.0f;
                gB[Q * kp + j] = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
        __syncthreads();  // the next chunk overwrites the staging
    }
}

// status[k] |= bit for every non-finite element of a knot-major array of W
// floats per knot (element-parallel and coalesced; atomics only on hits).
template <int W>
__device__ __forceinline__ void flag_nonfinite(const float *a, long long n, unsigned int bit, unsigned int *status) {
    if (!a) return;
    const long long total = n * W;
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x)
        if (!isfinite(a[e])) atomicOr(status + e / W, bit);
}

__global__ void knot_status_kernel(long long n, const float *q, const float *qd, const float *u, const float *dqdd,
                                   const float *qdd, const float *minv, unsigned int *status) {
    flag_nonfinite<kN>(q, n, 1u, status);
    flag_nonfinite<kN>(qd, n, 1u, status);
    flag_nonfinite<kN>(u, n, 1u, status);
    flag_nonfinite<kDqddN>(dqdd, n, 2u, status);
    flag_nonfinite<kN>(qdd, n, 2u, status);
    flag_nonfinite<kMinvN>(minv, n, 2u, status);
}

template <typename K>
cudaError_t opt_in(K kernel) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(sizeof(WarpSmem)) * 8);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
}

template <bool D, bool M, bool F, bool O>
cudaError_t launch_one(const LaunchShape &sh, int n, const float *q, const float *qd, const float *u,
                       const float *fext, float *dqdd, float *qdd, float *minv, cudaStream_t st) {
    const int w = sh.warps_per_cta, ntiles = (n + 31) / 32, grid = (ntiles + w - 1) / w;
    return launch_dependent(grad_ext_kernel<D, M, F, O>, dim3(grid), dim3(w * 32), sizeof(WarpSmem) * w, st, q, qd, u,
                            fext, dqdd, qdd, minv, n);
}

template <bool F, bool O>
cudaError_t dispatch(bool d, bool m, const LaunchShape &sh, int n, const float *q, const float *qd, const float *u,
                     const float *fext, float *dqdd, float *qdd, float *minv, cudaStream_t st) {
    if (!d && !m) return launch_one<false, false, F, O>(sh, n, q, qd, u, fext, dqdd, qdd, minv, st);
    if (d && !m) return launch_one<true, false, F, O>(sh, n, q, qd, u, fext, dqdd, qdd, minv, st);
    if (!d && m) return launch_one<false, true, F, O>(sh, n, q, qd, u, fext, dqdd, qdd, minv, st);
    return launch_one<true, true, F, O>(sh, n, q, qd, u, fext, dqdd, qdd, minv, st);
}

}  // namespace

cudaError_t init_ext_kernels() {
    cudaError_t e = cudaSuccess;
    for (cudaError_t r : {opt_in(grad_knots_kernel<false, false>), opt_in(grad_knots_kernel<true, false>),
                          opt_in(grad_knots_kernel<false, true>), opt_in(grad_knots_kernel<true, true>)})
        if (r != cudaSuccess && e == cudaSuccess) e = r;
#define FRG_OPT(F, O)                                                                                        \
    for (cudaError_t r : {opt_in(grad_ext_kernel<false, false, F, O>), opt_in(grad_ext_kernel<true, false, F, O>), \
                          opt_in(grad_ext_kernel<false, true, F, O>), opt_in(grad_ext_kernel<true, true, F, O>)})  \
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    FRG_OPT(true, false)
    FRG_OPT(false, true)
    FRG_OPT(true, true)
#undef FRG_OPT
    return e;
}

cudaError_t launch_ext(bool damping, bool mpc, const LaunchShape &shape, int n, const float *q, const float *qd,
                       const float *u, const float *fext, float *dqdd, float *qdd, float *minv, bool fd_only,
                       cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    if (shape.warps_per_cta < 1 || shape.warps_per_cta > 8) return cudaErrorInvalidValue;
    LaunchShape sh = shape;
    if (fd_only) {
        return fext ? dispatch<true, true>(damping, mpc, sh, n, q, qd, u, fext, nullptr, qdd, minv, stream)
                    : dispatch<false, true>(damping, mpc, sh, n, q, qd, u, nullptr, nullptr, qdd, minv, stream);
    }
    return dispatch<true, false>(damping, mpc, sh, n, q, qd, u, fext, dqdd, qdd, minv, stream);
}

cudaError_t launch_discretize(int n, const float *dqdd, const float *minv, float dt, float *A, float *B,
                              cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    auto al16 = [](const void *p) { return (reinterpret_cast<unsigned long long>(p) & 15ull) == 0; };
    int done = 0;  // knots handled by the chunked kernel
    if (al16(dqdd) && al16(minv) && al16(A) && al16(B) && n >= kDiscKnots) {
        const int nchunks = n / kDiscKnots;
        const int grid = nchunks < 152 * 64 ? nchunks : 152 * 64;
        discretize_chunks_kernel<<<grid, 256, 0, stream>>>(nchunks, dqdd, minv, dt, A, B);
        done = nchunks * kDiscKnots;
    }
    const int rest = n - done;
    if (rest > 0) {
        const long long d = done;
        const long long total = static_cast<long long>(rest) * (6 * kMinvN);
        long long blocks = (total + 255) / 256;
        if (blocks > 152 * 16) blocks = 152 * 16;
        discretize_kernel<<<static_cast<int>(blocks), 256, 0, stream>>>(rest, dqdd + kDqddN * d, minv + kMinvN * d,
                                                                        dt, A + 4 * kMinvN * d, B + kDqddN * d);
    }
    return cudaGetLastError();
}

cudaError_t launch_knots(bool damping, bool mpc, const LaunchShape &shape, int n, float *knots, float *dqdd,
                         cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    if (shape.warps_per_cta < 1 || shape.warps_per_cta > 8) return cudaErrorInvalidValue;
    const int w = shape.warps_per_cta, ntiles = (n + 31) / 32, grid = (ntiles + w - 1) / w;
    const size_t smem = sizeof(WarpSmem) * w;
    auto kernel = !damping && !mpc  ? grad_knots_kernel<false, false>
                  : damping && !mpc ? grad_knots_kernel<true, false>
                  : !damping && mpc ? grad_knots_kernel<false, true>
                                    : grad_knots_kernel<true, true>;
    return launch_dependent(kernel, dim3(grid), dim3(w * 32), smem, stream, knots, dqdd, n);
}

cudaError_t launch_knot_status(int num_sms, int n, const float *q, const float *qd, const float *u,
                               const float *dqdd, const float *qdd, const float *minv, unsigned int *status,
                               cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(unsigned int) * static_cast<size_t>(n), stream);
    if (e != cudaSuccess) return e;
    long long blocks = (static_cast<long long>(n) * kDqddN + 255) / 256;
    if (blocks > static_cast<long long>(num_sms) * 8) blocks = static_cast<long long>(num_sms) * 8;
    knot_status_kernel<<<static_cast<int>(blocks), 256, 0, stream>>>(n, q, qd, u, dqdd, qdd, minv, status);
    return cudaGetLastError();
}

}  // namespace frg
