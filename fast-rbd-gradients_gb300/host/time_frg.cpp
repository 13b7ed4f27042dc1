// time_frg: C++ timing driver over the C ABI, the counterpart of the
// reference's time_GPU.cu (its "Completely Fused" rows, time_GPU.cu:307-331)
// with q̈ and Minv computed on the device instead of on the host.
//
//   time_frg [--iters K] [--equivalence] [--damping] [--mpc] [--autotune] [N ...]
//   time_frg --ragged T [--iters K] [--autotune]
//
// For every batch size N (default 16 32 64 128 1024 65536) it prints, like
// time_GPU.cu: "GPU Compute + I/O" (host arrays in, host arrays out:
// frg_gradient_host) and "GPU Compute" (device-resident arrays: frg_gradient +
// stream sync), each as printStats-style statistics over K calls (mean, std,
// min, max, percentiles; utils/experiment_helpers.h:42-99).  --equivalence
// runs the reference's TEST_FOR_EQUIVALENCE point (q = qd = u = 0.1, N = 1;
// experiment_helpers.h:11, time_GPU.cu:199-211) and prints q, qd, qdd, u,
// Minv, dqdd/dq and dqdd/dqd in the reference's printMat layout.  --ragged T
// times T trajectories of horizons U{8..256} stored in shuffled order in one
// device buffer (as separately produced trajectories are) in the plain form
// (one launch per trajectory, the only form the reference has), as one
// batched persistent launch, as a plan launch, and as two independent plans
// (a second copy of the batch) in flight together (frg_plan_launch_many).
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

// Wall-clock microseconds of `iters` calls of fn (after 10 untimed), each
// followed by a stream synchronize, as time_GPU.cu times its rows.
template <typename F>
std::vector<double> time_calls(int iters, cudaStream_t st, F fn) {
    std::vector<double> t;
    for (int it = 0; it < iters + 10; it++) {
        auto t0 = std::chrono::steady_clock::now();
        fn();
        cudaStreamSynchronize(st);
        auto t1 = std::chrono::steady_clock::now();
        if (it >= 10) t.push_back(std::chrono::duration<double, std::micro>(t1 - t0).count());
    }
    return t;
}

const float kLim[7] = {2.96706f, 2.09440f, 2.96706f, 2.09440f, 2.96706f, 2.09440f, 3.05433f};

// q ~ U(joint limits), qd ~ U(-2, 2), u ~ U(-20, 20), knot-major [n][7] each.
void fill_knots(std::mt19937_64 &rng, size_t n, float *q, float *qd, float *u) {
    std::uniform_real_distribution<float> unit(-1.0f, 1.0f);
    for (size_t k = 0; k < n; k++)
        for (int j = 0; j < 7; j++) {
            q[7 * k + j] = kLim[j] * unit(rng);
            qd[7 * k + j] = 2.0f * unit(rng);
            u[7 * k + j] = 20.0f * unit(rng);
        }
}

int run_ragged(frg_ctx *ctx, int ntraj, int iters) {
    std::mt19937_64 rng(2021);
    std::uniform_int_distribution<int> hz(8, 256);
    std::vector<int64_t> h(ntraj);
    size_t total = 0;
    for (int t = 0; t < ntraj; t++) total += static_cast<size_t>(h[t] = hz(rng));
    std::vector<int> order(ntraj);
    std::iota(order.begin(), order.end(), 0);
    std::shuffle(order.begin(), order.end(), rng);
    std::vector<size_t> mem(ntraj);
    size_t pos = 0;
    for (int t : order) {
        mem[t] = pos;
        pos += static_cast<size_t>(h[t]);
    }
    std::vector<float> hin(21 * total);
    fill_knots(rng, total, hin.data(), hin.data() + 7 * total, hin.data() + 14 * total);
    // two copies of the batch (inputs and outputs), the second for the
    // independent plan that runs beside the first
    float *d = nullptr;
    if (cudaMalloc(&d, sizeof(float) * 2 * 175 * total) != cudaSuccess) die(ctx, FRG_ERR_OUT_OF_MEMORY, "cudaMalloc");
    cudaMemcpy(d, hin.data(), sizeof(float) * 21 * total, cudaMemcpyHostToDevice);
    cudaMemcpy(d + 175 * total, hin.data(), sizeof(float) * 21 * total, cudaMemcpyHostToDevice);
    const size_t N = total;
    std::vector<frg_traj> trajs(ntraj), trajs2(ntraj);
    for (int t = 0; t < ntraj; t++) {
        const size_t m = mem[t];
        trajs[t] = frg_traj{h[t], d + 7 * m, d + 7 * N + 7 * m, d + 14 * N + 7 * m, d + 21 * N + 98 * m,
                            d + 119 * N + 7 * m, d + 126 * N + 49 * m};
        float *d2 = d + 175 * N;
        trajs2[t] = frg_traj{h[t], d2 + 7 * m, d2 + 7 * N + 7 * m, d2 + 14 * N + 7 * m, d2 + 21 * N + 98 * m,
                             d2 + 119 * N + 7 * m, d2 + 126 * N + 49 * m};
    }
    cudaStream_t st;
    cudaStreamCreate(&st);
    frg_status s;
    frg_plan *plan = nullptr, *plan2 = nullptr;
    if ((s = frg_plan_create(ctx, ntraj, trajs.data(), &plan)) != FRG_OK) die(ctx, s, "frg_plan_create");
    if ((s = frg_plan_create(ctx, ntraj, trajs2.data(), &plan2)) != FRG_OK) die(ctx, s, "frg_plan_create");
    const int n = static_cast<int>(total);
    auto plain = time_calls(iters, st, [&] {
        if ((s = frg_gradient_per_trajectory(ctx, ntraj, trajs.data(), st)) != FRG_OK)
            die(ctx, s, "frg_gradient_per_trajectory");
    });
    auto batched = time_calls(iters, st, [&] {
        if ((s = frg_gradient_batched(ctx, ntraj, trajs.data(), st)) != FRG_OK) die(ctx, s, "frg_gradient_batched");
    });
    auto replay = time_calls(iters, st, [&] {
        if ((s = frg_plan_launch(plan, st)) != FRG_OK) die(ctx, s, "frg_plan_launch");
    });
    frg_plan *pair[2] = {plan, plan2};
    auto two = time_calls(iters, st, [&] {
        if ((s = frg_plan_launch_many(ctx, 2, pair, 2, st)) != FRG_OK) die(ctx, s, "frg_plan_launch_many");
    });
    std::printf("%d trajectories, horizons U{8..256}, %d knots, stored in shuffled order\n", ntraj, n);
    print_stats("Plain - one launch per trajectory", n, plain);
    print_stats("Batched - one persistent launch", n, batched);
    print_stats("Batched - plan launch", n, replay);
    print_stats("Batched - two independent plans in flight (per call: both batches)", 2 * n, two);
    frg_plan_destroy(plan);
    frg_plan_destroy(plan2);
    cudaStreamDestroy(st);
    cudaFree(d);
    return 0;
}

void print_mat(const float *A, int rows, int cols, int lda) {
    for (int i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) std::printf("%.6f ", static_cast<double>(A[i + lda * j]));
        std::printf("\n");
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (frg_model_dofs() != 7) {  // this driver mirrors time_GPU.cu, whose model is the 7-joint iiwa_14
        std::fprintf(stderr, "time_frg drives the iiwa_14 build; this library is %s with %d joints\n",
                     frg_model_name(), frg_model_dofs());
        return 2;
    }
    int iters = 1000;
    bool equivalence = false, autotune = false;
    int ragged = 0;
    frg_options opt;
    frg_options_default(&opt);
    std::vector<int> sizes;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--iters") && i + 1 < argc) iters = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--equivalence")) equivalence = true;
        else if (!std::strcmp(argv[i], "--damping")) opt.vel_damping = 1;
        else if (!std::strcmp(argv[i], "--mpc")) opt.mpc_mode = 1;
        else if (!std::strcmp(argv[i], "--autotune")) autotune = true;
        else if (!std::strcmp(argv[i], "--ragged") && i + 1 < argc) ragged = std::atoi(argv[++i]);
        else sizes.push_back(std::atoi(argv[i]));
    }
    if (sizes.empty()) sizes = {16, 32, 64, 128, 1024, 65536};
    frg_ctx *ctx = nullptr;
    frg_status s = frg_create(&ctx, &opt);
    if (s != FRG_OK) die(nullptr, s, "frg_create");
    if (autotune && (s = frg_autotune(ctx, 65536, nullptr)) != FRG_OK) die(ctx, s, "frg_autotune");
    if (ragged > 0) {
        const int rc = run_ragged(ctx, ragged, iters);
        frg_destroy(ctx);
        return rc;
    }

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

    std::mt19937_64 rng(2021);
    for (int n : sizes) {
        const size_t N = static_cast<size_t>(n);
        // one pinned allocation per array, as a caller's separate buffers
        float *hq = static_cast<float *>(frg_host_alloc(sizeof(float) * 7 * N));
        float *hqd = static_cast<float *>(frg_host_alloc(sizeof(float) * 7 * N));
        float *hu = static_cast<float *>(frg_host_alloc(sizeof(float) * 7 * N));
        float *hdqdd = static_cast<float *>(frg_host_alloc(sizeof(float) * 98 * N));
        float *hqdd = static_cast<float *>(frg_host_alloc(sizeof(float) * 7 * N));
        float *hminv = static_cast<float *>(frg_host_alloc(sizeof(float) * 49 * N));
        if (!(hq && hqd && hu && hdqdd && hqdd && hminv)) die(ctx, FRG_ERR_OUT_OF_MEMORY, "frg_host_alloc");
        fill_knots(rng, N, hq, hqd, hu);
        float *d = nullptr;
        if (cudaMalloc(&d, sizeof(float) * 175 * N) != cudaSuccess) die(ctx, FRG_ERR_OUT_OF_MEMORY, "cudaMalloc");
        cudaMemcpy(d, hq, sizeof(float) * 7 * N, cudaMemcpyHostToDevice);
        cudaMemcpy(d + 7 * N, hqd, sizeof(float) * 7 * N, cudaMemcpyHostToDevice);
        cudaMemcpy(d + 14 * N, hu, sizeof(float) * 7 * N, cudaMemcpyHostToDevice);
        cudaStream_t st;
        cudaStreamCreate(&st);
        auto io = time_calls(iters, st, [&] {
            if ((s = frg_gradient_host(ctx, n, hq, hqd, hu, hdqdd, hqdd, hminv)) != FRG_OK) die(ctx, s, "frg_gradient_host");
        });
        auto comp = time_calls(iters, st, [&] {
            if ((s = frg_gradient(ctx, n, d, d + 7 * N, d + 14 * N, d + 21 * N, d + 119 * N, d + 126 * N, st)) != FRG_OK)
                die(ctx, s, "frg_gradient");
        });
        print_stats("Completely Fused - GPU Compute + I/O", n, io);
        print_stats("Completely Fused - GPU Compute", n, comp);
        std::printf("----------------------------------------\n");
        cudaStreamDestroy(st);
        cudaFree(d);
        for (float *p : {hq, hqd, hu, hdqdd, hqdd, hminv}) frg_host_free(p);
    }
    frg_destroy(ctx);
    return 0;
}
