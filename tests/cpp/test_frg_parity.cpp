// C++ parity test over the C ABI (include/frg.h), checked against the oracle
// (oracle/libfrg_oracle.so: the reference's CPU path restated in C, FP64).
// Built and run by tests/test_gpu_cpp.py.
//
// Inputs follow the reference's experiment distributions with one seeded
// std::mt19937_64: q ~ U(joint limits of utils/iiwa_14.urdf), qd ~ U(-2, 2),
// u ~ U(-20, 20).  Checked, in every (damping, mpc) mode:
//   - frg_gradient (device arrays) against the FP64 oracle: max per-knot
//     Frobenius-relative error of dqdd, qdd, Minv <= 1e-4;
//   - frg_gradient_host on pinned and on pageable host arrays: the same bits
//     as the device path;
//   - frg_gradient_batched and a replayed plan over trajectories stored in
//     shuffled order: the same bits as the device path.
// Exit status 0 when every check passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "frg.h"

extern "C" int frg_oracle_gradient_f64(int n, const double *q, const double *qd, const double *u, const double *fext,
                                       int damping, int mpc, double *dqdd, double *qdd, double *minv);

namespace {

const double kTol = 1e-4;
int g_failures = 0;

void check(bool ok, const char *what, int damping, int mpc) {
    if (!ok) {
        std::printf("FAIL [damping %d, mpc %d] %s\n", damping, mpc, what);
        g_failures++;
    }
}

bool ok_status(frg_ctx *ctx, frg_status s, const char *what) {
    if (s == FRG_OK) return true;
    std::printf("FAIL %s: %s (%s)\n", what, frg_status_string(s), frg_last_error(ctx));
    g_failures++;
    return false;
}

// max over knots of ||a_k - b_k|| / ||b_k|| for n knots of w values
double max_frob_rel(const float *a, const double *b, size_t n, int w) {
    double worst = 0;
    for (size_t k = 0; k < n; k++) {
        double num = 0, den = 0;
        for (int j = 0; j < w; j++) {
            const double d = static_cast<double>(a[w * k + j]) - b[w * k + j];
            num += d * d;
            den += b[w * k + j] * b[w * k + j];
        }
        const double e = std::sqrt(num) / std::max(std::sqrt(den), 1e-300);
        if (!(e <= worst)) worst = e;  // NaN propagates
    }
    return worst;
}

struct Outputs {
    std::vector<float> dqdd, qdd, minv;
    explicit Outputs(size_t n) : dqdd(98 * n), qdd(7 * n), minv(49 * n) {}
    bool operator==(const Outputs &o) const {
        return !std::memcmp(dqdd.data(), o.dqdd.data(), 4 * dqdd.size()) &&
               !std::memcmp(qdd.data(), o.qdd.data(), 4 * qdd.size()) &&
               !std::memcmp(minv.data(), o.minv.data(), 4 * minv.size());
    }
};

void run_mode(int damping, int mpc, const std::vector<float> &q, const std::vector<float> &qd,
              const std::vector<float> &u, const std::vector<int64_t> &horizons) {
    const size_t n = q.size() / 7;
    frg_options opt;
    frg_options_default(&opt);
    opt.vel_damping = damping;
    opt.mpc_mode = mpc;
    frg_ctx *ctx = nullptr;
    if (!ok_status(nullptr, frg_create(&ctx, &opt), "frg_create")) return;

    // FP64 oracle on the same (FP32) inputs
    std::vector<double> q64(q.begin(), q.end()), qd64(qd.begin(), qd.end()), u64(u.begin(), u.end());
    std::vector<double> rd(98 * n), rq(7 * n), rm(49 * n);
    frg_oracle_gradient_f64(static_cast<int>(n), q64.data(), qd64.data(), u64.data(), nullptr, damping, mpc,
                            rd.data(), rq.data(), rm.data());

    // device path
    float *d = nullptr;
    cudaMalloc(&d, sizeof(float) * 175 * n);
    float *dq = d, *dqd = d + 7 * n, *du = d + 14 * n, *ddqdd = d + 21 * n, *dqdd_ = d + 119 * n, *dminv = d + 126 * n;
    cudaMemcpy(dq, q.data(), 28 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dqd, qd.data(), 28 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(du, u.data(), 28 * n, cudaMemcpyHostToDevice);
    Outputs dev(n);
    if (ok_status(ctx, frg_gradient(ctx, static_cast<int>(n), dq, dqd, du, ddqdd, dqdd_, dminv, nullptr), "frg_gradient")) {
        cudaDeviceSynchronize();
        cudaMemcpy(dev.dqdd.data(), ddqdd, 392 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(dev.qdd.data(), dqdd_, 28 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(dev.minv.data(), dminv, 196 * n, cudaMemcpyDeviceToHost);
    }
    const double ed = max_frob_rel(dev.dqdd.data(), rd.data(), n, 98);
    const double eq = max_frob_rel(dev.qdd.data(), rq.data(), n, 7);
    const double em = max_frob_rel(dev.minv.data(), rm.data(), n, 49);
    std::printf("[damping %d, mpc %d] %zu knots vs FP64 oracle: dqdd %.3e  qdd %.3e  minv %.3e\n", damping, mpc, n,
                ed, eq, em);
    check(ed <= kTol && eq <= kTol && em <= kTol, "device path vs FP64 oracle", damping, mpc);

    // host paths: pageable and pinned
    Outputs pageable(n);
    ok_status(ctx, frg_gradient_host(ctx, static_cast<int>(n), q.data(), qd.data(), u.data(), pageable.dqdd.data(),
                                     pageable.qdd.data(), pageable.minv.data()),
              "frg_gradient_host (pageable)");
    check(pageable == dev, "host path, pageable arrays == device path", damping, mpc);
    {
        float *hp[6];
        const int w[6] = {7, 7, 7, 98, 7, 49};
        for (int i = 0; i < 6; i++) hp[i] = static_cast<float *>(frg_host_alloc(sizeof(float) * w[i] * n));
        std::memcpy(hp[0], q.data(), 28 * n);
        std::memcpy(hp[1], qd.data(), 28 * n);
        std::memcpy(hp[2], u.data(), 28 * n);
        ok_status(ctx, frg_gradient_host(ctx, static_cast<int>(n), hp[0], hp[1], hp[2], hp[3], hp[4], hp[5]),
                  "frg_gradient_host (pinned)");
        Outputs pinned(n);
        std::memcpy(pinned.dqdd.data(), hp[3], 392 * n);
        std::memcpy(pinned.qdd.data(), hp[4], 28 * n);
        std::memcpy(pinned.minv.data(), hp[5], 196 * n);
        check(pinned == dev, "host path, pinned arrays == device path", damping, mpc);
        for (float *p : hp) frg_host_free(p);
    }

    // batched and plan over the same knots cut into trajectories stored in shuffled order
    const size_t T = horizons.size();
    std::vector<size_t> begin(T + 1, 0);
    for (size_t t = 0; t < T; t++) begin[t + 1] = begin[t] + static_cast<size_t>(horizons[t]);
    std::vector<size_t> order(T), mem(T);
    std::iota(order.begin(), order.end(), size_t(0));
    std::mt19937_64 shuf(7);
    std::shuffle(order.begin(), order.end(), shuf);
    size_t pos = 0;
    for (size_t t : order) {
        mem[t] = pos;
        pos += static_cast<size_t>(horizons[t]);
    }
    float *s = nullptr;
    cudaMalloc(&s, sizeof(float) * 175 * n);
    std::vector<frg_traj> trajs(T);
    for (size_t t = 0; t < T; t++) {
        const size_t m = mem[t], b = begin[t], h = static_cast<size_t>(horizons[t]);
        cudaMemcpy(s + 7 * m, q.data() + 7 * b, 28 * h, cudaMemcpyHostToDevice);
        cudaMemcpy(s + 7 * n + 7 * m, qd.data() + 7 * b, 28 * h, cudaMemcpyHostToDevice);
        cudaMemcpy(s + 14 * n + 7 * m, u.data() + 7 * b, 28 * h, cudaMemcpyHostToDevice);
        trajs[t] = frg_traj{horizons[t], s + 7 * m, s + 7 * n + 7 * m, s + 14 * n + 7 * m, s + 21 * n + 98 * m,
                            s + 119 * n + 7 * m, s + 126 * n + 49 * m};
    }
    auto gather = [&](Outputs &o) {
        cudaDeviceSynchronize();
        for (size_t t = 0; t < T; t++) {
            const size_t m = mem[t], b = begin[t], h = static_cast<size_t>(horizons[t]);
            cudaMemcpy(o.dqdd.data() + 98 * b, s + 21 * n + 98 * m, 392 * h, cudaMemcpyDeviceToHost);
            cudaMemcpy(o.qdd.data() + 7 * b, s + 119 * n + 7 * m, 28 * h, cudaMemcpyDeviceToHost);
            cudaMemcpy(o.minv.data() + 49 * b, s + 126 * n + 49 * m, 196 * h, cudaMemcpyDeviceToHost);
        }
    };
    Outputs batched(n), replayed(n);
    cudaMemset(s + 21 * n, 0xff, sizeof(float) * 154 * n);  // NaN fill: every result must be written
    ok_status(ctx, frg_gradient_batched(ctx, static_cast<int>(T), trajs.data(), nullptr), "frg_gradient_batched");
    gather(batched);
    check(batched == dev, "batched launch == device path", damping, mpc);
    frg_plan *plan = nullptr;
    if (ok_status(ctx, frg_plan_create(ctx, static_cast<int>(T), trajs.data(), &plan), "frg_plan_create")) {
        cudaMemset(s + 21 * n, 0xff, sizeof(float) * 154 * n);
        ok_status(ctx, frg_plan_launch(plan, nullptr), "frg_plan_launch");
        ok_status(ctx, frg_plan_launch(plan, nullptr), "frg_plan_launch (replay)");
        gather(replayed);
        check(replayed == dev, "plan replay == device path", damping, mpc);
        frg_plan_destroy(plan);
    }
    check(cudaGetLastError() == cudaSuccess, "no CUDA error", damping, mpc);
    cudaFree(s);
    cudaFree(d);
    frg_destroy(ctx);
}

}  // namespace

int main() {
    const float lim[7] = {2.96706f, 2.09440f, 2.96706f, 2.09440f, 2.96706f, 2.09440f, 3.05433f};
    std::mt19937_64 rng(2021);
    std::uniform_real_distribution<float> unit(-1.0f, 1.0f);
    std::uniform_int_distribution<int> hz(1, 96);
    std::vector<int64_t> horizons;
    size_t n = 0;
    while (n < 3000) {
        horizons.push_back(hz(rng));
        n += static_cast<size_t>(horizons.back());
    }
    std::vector<float> q(7 * n), qd(7 * n), u(7 * n);
    for (size_t k = 0; k < n; k++)
        for (int j = 0; j < 7; j++) {
            q[7 * k + j] = lim[j] * unit(rng);
            qd[7 * k + j] = 2.0f * unit(rng);
            u[7 * k + j] = 20.0f * unit(rng);
        }
    for (int j = 0; j < 7; j++) q[j] = qd[j] = u[j] = 0.1f;  // knot 0: the reference's equivalence point
    for (int damping = 0; damping < 2; damping++)
        for (int mpc = 0; mpc < 2; mpc++) run_mode(damping, mpc, q, qd, u, horizons);
    std::printf("%s: %d failure(s)\n", g_failures ? "FAILED" : "PASSED", g_failures);
    return g_failures ? 1 : 0;
}
