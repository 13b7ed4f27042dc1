// FP32 CUDA-core peak of one GPU, the denominator of the gradient kernels'
// FP32 roofline: every thread of 2 x 1024-thread CTAs per SM runs 8
// independent FMA chains, once as scalar fmaf (FFMA) and once as packed pairs
// (__ffma2_rn, FFMA2); FLOP = 2 per FMA.  Prints the best of `reps` launches
// of each (CUDA events) as
//   FFMA_TFLOPS <x>
//   FFMA2_TFLOPS <y>
// Usage: frg_fp32_peak [device] [reps]
#include <cstdio>
#include <cstdlib>

#include <cuda_runtime.h>

namespace {

constexpr int kThreads = 1024, kChains = 8, kUnroll = 16, kIters = 20000;

__global__ void __launch_bounds__(kThreads) ffma_chains(float *out, int iters, float b, float c) {
    float a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) a[k] = threadIdx.x * 1e-7f + k * 1e-3f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < kUnroll; j++)
#pragma unroll
            for (int k = 0; k < kChains; k++) a[k] = fmaf(a[k], b, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kChains; k++) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps every chain live
}

__global__ void __launch_bounds__(kThreads) ffma2_chains(float2 *out, int iters, float b, float c) {
    const float2 bb = make_float2(b, b), cc = make_float2(c, c);
    float2 a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) a[k] = make_float2(threadIdx.x * 1e-7f + k * 1e-3f, threadIdx.x * 1e-7f - k * 1e-3f);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < kUnroll; j++)
#pragma unroll
            for (int k = 0; k < kChains; k++) a[k] = __ffma2_rn(a[k], bb, cc);
    }
    float2 s = a[0];
#pragma unroll
    for (int k = 1; k < kChains; k++) s = __fadd2_rn(s, a[k]);
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename L>
double best_tflops(L launch, double flop_per_launch, int reps) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int r = 0; r < reps; r++) {
        cudaEventRecord(e0);
        launch();
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double tf = flop_per_launch / (ms * 1e-3) / 1e12;
        if (tf > best) best = tf;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return best;
}

}  // namespace

int main(int argc, char **argv) {
    const int device = argc > 1 ? std::atoi(argv[1]) : 0;
    const int reps = argc > 2 ? std::atoi(argv[2]) : 10;
    if (cudaSetDevice(device) != cudaSuccess) return 1;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = 2 * sms;
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float2) * kThreads * blocks) != cudaSuccess) return 1;
    const double fmas = static_cast<double>(kChains) * kUnroll * kIters * kThreads * blocks;
    ffma_chains<<<blocks, kThreads>>>(out, kIters / 10, 0.999999f, 1e-6f);  // warm-up
    const double t1 = best_tflops([&] { ffma_chains<<<blocks, kThreads>>>(out, kIters, 0.999999f, 1e-6f); },
                                  2.0 * fmas, reps);
    float2 *out2 = reinterpret_cast<float2 *>(out);
    ffma2_chains<<<blocks, kThreads>>>(out2, kIters / 10, 0.999999f, 1e-6f);
    const double t2 = best_tflops([&] { ffma2_chains<<<blocks, kThreads>>>(out2, kIters, 0.999999f, 1e-6f); },
                                  4.0 * fmas, reps);
    const cudaError_t e = cudaDeviceSynchronize();
    cudaFree(out);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "frg_fp32_peak: %s\n", cudaGetErrorString(e));
        return 1;
    }
    std::printf("SMS %d\nFFMA_TFLOPS %.2f\nFFMA2_TFLOPS %.2f\n", sms, t1, t2);
    return 0;
}
