// FP64 verification build of the gradient.
//
// The knot-per-lane device code of frg_knot.cuh / frg_model.cuh compiled a
// second time with double as its scalar type (namespace frg64): the same
// sweeps, the same Minv recursion and the same -Minv dtau finish, with the
// model constants rounded once to double instead of float and the library
// double-precision sincos.  It serves as an on-device FP64 check of the FP32
// engine (sampled verification of served results) and as an FP64 gradient
// for callers that want one; the reference's FP64 path is its CPU code
// (helpers_CPU/dynamicsGradient.h:916-934 with T = double).
//
// Shared memory per warp doubles to 48,384 B, so a CTA is one warp; the
// double-precision registers exceed the 255-register file and part of each
// knot's state lives in local memory.  This path is not the throughput path.
#define FRG_REAL double
#define FRG_NS frg64
#include "frg_knot.cuh"
#undef FRG_REAL
#undef FRG_NS

#include "frg_kernels.cuh"

namespace frg64 {
namespace {

struct Args {
    const double *q, *qd, *u;
    double *dqdd, *qdd, *minv;
    long long n;
};

template <bool DAMP, bool MPC>
__global__ void __launch_bounds__(32) grad_plain_f64_kernel(Args a) {
    extern __shared__ double2 smem_f64[];
    const int lane = threadIdx.x & 31;
    WarpSmem *ws = reinterpret_cast<WarpSmem *>(smem_f64);
    const long long ntiles = (a.n + 31) / 32;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long g = tile * 32 + lane;
        KnotPtrs kp{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
        if (g < a.n)
            kp = KnotPtrs{a.q + frg::kN * g, a.qd + frg::kN * g, a.u + frg::kN * g, a.dqdd + frg::kDqddN * g,
                          a.qdd + frg::kN * g, a.minv + frg::kMinvN * g};
        process_tile<DAMP, MPC>(ws, lane, kp);
    }
}

// q, qd, u (float, [n][N] each) -> out [3][n][N] (double)
__global__ void widen_inputs_kernel(long long n, const float *q, const float *qd, const float *u, double *out) {
    const long long m = frg::kN * n;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < 3 * m;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long a = i / m, j = i - a * m;
        const float *src = a == 0 ? q : (a == 1 ? qd : u);
        out[i] = static_cast<double>(src[j]);
    }
}

// ||x - r||_F / ||r||_F over one knot's W values (r the FP64 result).
template <int W>
__device__ __forceinline__ double frob_rel(const float *x, const double *r) {
    double num = 0.0, den = 0.0;
    for (int j = 0; j < W; j++) {
        const double d = static_cast<double>(x[j]) - r[j];
        num = fma(d, d, num);
        den = fma(r[j], r[j], den);
    }
    return sqrt(num) / fmax(sqrt(den), 1e-300);
}

// err[i] = (dqdd, qdd, minv) Frobenius-relative errors of knot i.  A NaN in
// either operand propagates to the error.
__global__ void compare_kernel(long long n, const float *dqdd, const float *qdd, const float *minv,
                               const double *rdqdd, const double *rqdd, const double *rminv, double *err) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        constexpr int D = frg::kDqddN, N = frg::kN, M = frg::kMinvN;
        err[3 * i + 0] = frob_rel<D>(dqdd + D * i, rdqdd + D * i);
        err[3 * i + 1] = frob_rel<N>(qdd + N * i, rqdd + N * i);
        err[3 * i + 2] = frob_rel<M>(minv + M * i, rminv + M * i);
    }
}

int g_ctas_per_sm = 0;

template <bool D, bool M>
cudaError_t plain_impl(int num_sms, const Args &a, cudaStream_t st) {
    const long long ntiles = (a.n + 31) / 32;
    long long grid = static_cast<long long>(num_sms) * (g_ctas_per_sm > 0 ? g_ctas_per_sm : 1);
    if (grid > ntiles) grid = ntiles;
    grad_plain_f64_kernel<D, M><<<static_cast<int>(grid), 32, sizeof(WarpSmem), st>>>(a);
    return cudaGetLastError();
}

int stride_grid(int num_sms, long long work) {
    long long g = (work + 255) / 256;
    const long long cap = static_cast<long long>(num_sms) * 8;
    if (g > cap) g = cap;
    return static_cast<int>(g < 1 ? 1 : g);
}

}  // namespace
}  // namespace frg64

namespace frg {

size_t f64_warp_smem_bytes() { return sizeof(frg64::WarpSmem); }

cudaError_t init_f64_kernels() {
    using namespace frg64;
    cudaError_t e = cudaSuccess;
    for (auto k : {grad_plain_f64_kernel<false, false>, grad_plain_f64_kernel<true, false>,
                   grad_plain_f64_kernel<false, true>, grad_plain_f64_kernel<true, true>}) {
        const cudaError_t r = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   static_cast<int>(sizeof(WarpSmem)));
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    }
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, grad_plain_f64_kernel<false, false>, 32,
                                                      sizeof(WarpSmem));
    if (e == cudaSuccess) frg64::g_ctas_per_sm = blocks;
    return e;
}

cudaError_t launch_plain_f64(bool damping, bool mpc, int num_sms, long long n, const double *q, const double *qd,
                             const double *u, double *dqdd, double *qdd, double *minv, cudaStream_t stream) {
    using namespace frg64;
    if (n <= 0) return cudaSuccess;
    const Args a{q, qd, u, dqdd, qdd, minv, n};
    if (!damping && !mpc) return plain_impl<false, false>(num_sms, a, stream);
    if (damping && !mpc) return plain_impl<true, false>(num_sms, a, stream);
    if (!damping && mpc) return plain_impl<false, true>(num_sms, a, stream);
    return plain_impl<true, true>(num_sms, a, stream);
}

cudaError_t launch_widen_inputs(int num_sms, long long n, const float *q, const float *qd, const float *u,
                                double *out, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    frg64::widen_inputs_kernel<<<frg64::stride_grid(num_sms, 3 * frg::kN * n), 256, 0, stream>>>(n, q, qd, u, out);
    return cudaGetLastError();
}

cudaError_t launch_compare_f64(int num_sms, long long n, const float *dqdd, const float *qdd, const float *minv,
                               const double *rdqdd, const double *rqdd, const double *rminv, double *err,
                               cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    frg64::compare_kernel<<<frg64::stride_grid(num_sms, n), 256, 0, stream>>>(n, dqdd, qdd, minv, rdqdd, rqdd,
                                                                                rminv, err);
    return cudaGetLastError();
}

}  // namespace frg
