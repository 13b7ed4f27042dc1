// Instruction-fetch probe of one GPU: how fast warps issue from a loop whose
// body is NI instructions long, as the body outgrows the instruction caches.
//
// Each warp runs 8 independent FFMA chains (enough to keep the FMA pipe fed
// from a warp's own dependencies), unrolled into a loop body of NI FFMA
// instructions (16 bytes each), repeated until every warp has issued 2^22
// FFMAs.  The launch puts W warps on every SM (one CTA of W warps per SM), so
// W / 4 warps share each of the SM's four schedulers.  The time of the launch
// (CUDA events) gives the FFMA instructions issued per scheduler per cycle at
// the clock passed on the command line.  The gradient kernels' unrolled link
// sweeps are about 110 KB of code; this shows what body sizes a warp can
// stream at which rate.
//
// Usage: frg_ifetch_probe [device] [sm_mhz]
// Prints one line per (warps per SM, body size):
//   IFETCH warps_per_sm=<W> body_kb=<KB> ms=<t> ipc_per_scheduler=<x>
#include <cstdio>
#include <cstdlib>

#include <cuda_runtime.h>

namespace {

constexpr long long kFfmaPerWarp = 1LL << 22;
constexpr int kChains = 8;

template <int NI>
__global__ void __launch_bounds__(256) ffma_body(float *out, int iters) {
    float a[kChains];
#pragma unroll
    for (int j = 0; j < kChains; j++) a[j] = threadIdx.x * 1e-3f + j;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < NI / kChains; i++)
#pragma unroll
            for (int j = 0; j < kChains; j++) a[j] = fmaf(a[j], 0.9999f, 1e-4f * (i + 1));
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < kChains; j++) s += a[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps every chain live
}

template <int NI>
bool run(float *out, int sms, int warps_per_sm, double sm_mhz) {
    const int iters = static_cast<int>(kFfmaPerWarp / NI);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return false;
    ffma_body<NI><<<sms, 32 * warps_per_sm>>>(out, 2);  // warm-up: code into the caches, clocks up
    cudaEventRecord(e0);
    ffma_body<NI><<<sms, 32 * warps_per_sm>>>(out, iters);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) return false;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double cycles = ms * 1e-3 * sm_mhz * 1e6;
    const double per_scheduler = static_cast<double>(iters) * NI * warps_per_sm / 4.0;
    printf("IFETCH warps_per_sm=%d body_kb=%d ms=%.3f ipc_per_scheduler=%.3f\n", warps_per_sm, NI * 16 / 1024, ms,
           per_scheduler / cycles);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return true;
}

}  // namespace

int main(int argc, char **argv) {
    const int dev = argc > 1 ? atoi(argv[1]) : 0;
    const double sm_mhz = argc > 2 ? atof(argv[2]) : 2070.0;
    if (cudaSetDevice(dev) != cudaSuccess) {
        fprintf(stderr, "no device %d\n", dev);
        return 1;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * sms * 256) != cudaSuccess) return 1;
    bool ok = true;
    for (int w : {8, 4}) {
        ok = ok && run<256>(out, sms, w, sm_mhz) && run<1024>(out, sms, w, sm_mhz) && run<1536>(out, sms, w, sm_mhz) &&
             run<2048>(out, sms, w, sm_mhz) && run<3072>(out, sms, w, sm_mhz) && run<4096>(out, sms, w, sm_mhz) &&
             run<8192>(out, sms, w, sm_mhz) && run<12288>(out, sms, w, sm_mhz);
    }
    const cudaError_t e = cudaDeviceSynchronize();
    cudaFree(out);
    if (!ok || e != cudaSuccess) {
        fprintf(stderr, "probe failed: %s\n", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}
