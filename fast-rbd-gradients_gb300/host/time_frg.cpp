// time_frg: C++ timing driver over the C ABI, the counterpart of the
// reference's time_GPU.cu (its "Completely Fused" rows, time_GPU.cu:307-331)
// with q̈ and Minv computed on the device instead of on the host.
//
//   time_frg [--iters K] [--equivalence] [--damping] [--mpc] [N ...]
//
// For every batch size N (default 16 32 64 128 1024 65536) it prints, like
// time_GPU.cu: "GPU Compute + I/O" (host arrays in, host arrays out:
// frg_gradient_host) and "GPU Compute" (device-resident arrays: frg_gradient +
// stream sync), each as printStats-style statistics over K calls (mean, std,
// min, max, percentiles; utils/experiment_helpers.h:42-99).  --equivalence
// runs the reference's TEST_FOR_EQUIVALENCE point (q = qd = u = 0.1, N = 1;
// experiment_helpers.h:11, time_GPU.cu:199-211) and prints q, qd, qdd, u,
// Minv, dqdd/dq and dqdd/dqd in the reference's printMat layout.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "frg.h"

namespace {

void die(frg_ctx *ctx, frg_status s, const char *what) {
    std::fprintf(stderr, "%s failed: %s (%s)\n", what, frg_status_string(s), frg_last_error(ctx));
    std::exit(1);
}

void print_stats(const char *label, int n, std::vector<double> t) {
    const double mean = std::accumulate(t.begin(), t.end(), 0.0) / t.size();
    double sq = 0;
    for (double x : t) sq += (x - mean) * (x - mean);
    const double sd = std::sqrt(sq / t.size());
    std::sort(t.begin(), t.end());
    auto pct = [&](double p) { return t[std::min(t.size() - 1, static_cast<size_t>(p * t.size()))]; };
    std::printf("[N:%d] %s: Average[%fus] Std Dev [%fus] Min [%fus] Max [%fus] knots/s [%.3e]\n", n, label, mean, sd,
                t.front(), t.back(), n / (mean * 1e-6));
    std::printf("    Percentiles |  50   |  75   |  90   |  95   |  99   |\n");
    std::printf("                | %.2f | %.2f | %.2f | %.2f | %.2f |\n", pct(0.5), pct(0.75), pct(0.9), pct(0.95),
                pct(0.99));
}

void print_mat(const float *A, int rows, int cols, int lda) {
    for (int i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) std::printf("%.6f ", static_cast<double>(A[i + lda * j]));
        std::printf("\n");
    }
}

}  // namespace

int main(int argc, char **argv) {
    int iters = 1000;
    bool equivalence = false;
    frg_options opt;
    frg_options_default(&opt);
    std::vector<int> sizes;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--iters") && i + 1 < argc) iters = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--equivalence")) equivalence = true;
        else if (!std::strcmp(argv[i], "--damping")) opt.vel_damping = 1;
        else if (!std::strcmp(argv[i], "--mpc")) opt.mpc_mode = 1;
        else sizes.push_back(std::atoi(argv[i]));
    }
    if (sizes.empty()) sizes = {16, 32, 64, 128, 1024, 65536};
    frg_ctx *ctx = nullptr;
    frg_status s = frg_create(&ctx, &opt);
    if (s != FRG_OK) die(nullptr, s, "frg_create");

    if (equivalence) {
        float q[7], qd[7], u[7], dqdd[98], qdd[7], minv[49];
        for (int i = 0; i < 7; i++) q[i] = qd[i] = u[i] = 0.1f;
        if ((s = frg_gradient_host(ctx, 1, q, qd, u, dqdd, qdd, minv)) != FRG_OK) die(ctx, s, "frg_gradient_host");
        std::printf("q,qd,qdd,u\n");
        print_mat(q, 1, 7, 1);
        print_mat(qd, 1, 7, 1);
        print_mat(qdd, 1, 7, 1);
        print_mat(u, 1, 7, 1);
        std::printf("Minv\n");
        print_mat(minv, 7, 7, 7);
        std::printf("dqdd/dq\n");
        print_mat(dqdd, 7, 7, 7);
        std::printf("dqdd/dqd\n");
        print_mat(dqdd + 49, 7, 7, 7);
        frg_destroy(ctx);
        return 0;
    }

    const float lim[7] = {2.96706f, 2.09440f, 2.96706f, 2.09440f, 2.96706f, 2.09440f, 3.05433f};
    std::mt19937_64 rng(2021);
    std::uniform_real_distribution<float> unit(-1.0f, 1.0f);
    for (int n : sizes) {
        const size_t N = static_cast<size_t>(n);
        float *h = static_cast<float *>(frg_host_alloc(sizeof(float) * 175 * N));
        if (!h) die(ctx, FRG_ERR_OUT_OF_MEMORY, "frg_host_alloc");
        float *hq = h, *hqd = h + 7 * N, *hu = h + 14 * N, *hdqdd = h + 21 * N, *hqdd = h + 119 * N, *hminv = h + 126 * N;
        for (size_t k = 0; k < N; k++)
            for (int j = 0; j < 7; j++) {
                hq[7 * k + j] = lim[j] * unit(rng);
                hqd[7 * k + j] = 2.0f * unit(rng);
                hu[7 * k + j] = 20.0f * unit(rng);
            }
        float *d = nullptr;
        if (cudaMalloc(&d, sizeof(float) * 175 * N) != cudaSuccess) die(ctx, FRG_ERR_OUT_OF_MEMORY, "cudaMalloc");
        cudaMemcpy(d, h, sizeof(float) * 21 * N, cudaMemcpyHostToDevice);
        cudaStream_t st;
        cudaStreamCreate(&st);
        std::vector<double> io, comp;
        for (int it = 0; it < iters + 10; it++) {
            auto t0 = std::chrono::steady_clock::now();
            if ((s = frg_gradient_host(ctx, n, hq, hqd, hu, hdqdd, hqdd, hminv)) != FRG_OK) die(ctx, s, "frg_gradient_host");
            auto t1 = std::chrono::steady_clock::now();
            if (it >= 10) io.push_back(std::chrono::duration<double, std::micro>(t1 - t0).count());
        }
        for (int it = 0; it < iters + 10; it++) {
            auto t0 = std::chrono::steady_clock::now();
            if ((s = frg_gradient(ctx, n, d, d + 7 * N, d + 14 * N, d + 21 * N, d + 119 * N, d + 126 * N, st)) != FRG_OK)
                die(ctx, s, "frg_gradient");
            cudaStreamSynchronize(st);
            auto t1 = std::chrono::steady_clock::now();
            if (it >= 10) comp.push_back(std::chrono::duration<double, std::micro>(t1 - t0).count());
        }
        print_stats("Completely Fused - GPU Compute + I/O", n, io);
        print_stats("Completely Fused - GPU Compute", n, comp);
        std::printf("----------------------------------------\n");
        cudaStreamDestroy(st);
        cudaFree(d);
        frg_host_free(h);
    }
    frg_destroy(ctx);
    return 0;
}
