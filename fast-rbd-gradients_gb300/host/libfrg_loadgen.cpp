// Load generator for the gradient server (C++ host code over the C ABI).
//
// A session is one trajectory that makes `calls` successive gradient calls
// (iLQR / line-search style): each call waits for the previous one, perturbs
// q, qd, u by N(0, sigma) and submits again; after the last call the session
// releases its slot.  Sessions start either
//   - open loop: Poisson arrivals at `rate` sessions/s for `duration_s`, or
//   - closed loop: `concurrency` sessions kept active for `duration_s`, or
//   - queued: `total_sessions` sessions submitted at once (admission test).
// `threads` client threads share the session table: each takes the next
// completion (frg_server_wait_any), perturbs that session's inputs and submits
// its next call; thread 0 also starts sessions.  Latencies are the server's
// submit -> results-visible times.
//
// With `source` 1 the sessions model a solver whose iterates live on the GPU:
// before the run, kPoolSets sets of `calls` perturbed iterates each are
// generated and copied to the device in one copy; session s takes set
// s % kPoolSets (the first h knots of each iterate), each call submits its
// iterate with frg_server_submit_device, and its results stay in the
// trajectory's device slot (sampled calls copy them out afterwards).  Starting
// a session thus makes no CUDA call.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "frg.h"

extern "C" {

typedef struct frg_loadgen_cfg {
    int mode;               /* 0 open loop (Poisson), 1 closed loop, 2 queued */
    double rate;            /* sessions/s (mode 0) */
    int concurrency;        /* active sessions (mode 1) */
    int total_sessions;     /* sessions (mode 2); 0 = unlimited in modes 0/1 */
    double duration_s;      /* arrival window (modes 0/1) */
    int calls;              /* calls per session */
    const int *horizons;    /* horizon choices, sampled uniformly ... */
    int n_horizons;
    int horizon_lo, horizon_hi; /* ... or, if n_horizons == 0, uniform in [lo, hi] */
    double sigma;           /* perturbation std of every call after the first */
    uint64_t seed;
    double sample_frac;     /* fraction of calls whose inputs/results are copied out */
    int sample_cap;         /* capacity of the sample buffers, in knots */
    float *sample_q, *sample_qd, *sample_u, *sample_dqdd, *sample_qdd, *sample_minv;
    int64_t *sample_h;      /* horizon of each sampled call (sample_cap entries) */
    int threads;            /* client threads (>= 1) */
    int source;             /* 0: host inputs, results to the host (frg_server_submit);
                               1: device inputs, results kept on the device (frg_server_submit_device) */
} frg_loadgen_cfg;

typedef struct frg_loadgen_result {
    uint64_t calls, knots, sessions, errors, samples, sample_knots;
    double elapsed_s;
    double calls_per_s, knots_per_s;
    double p50_us, p90_us, p99_us, max_us, mean_us;
    double p50_h64_us, p99_h64_us;  /* 64-knot calls only (0 if none) */
    double mean_batch_requests;
} frg_loadgen_result;

}  // extern "C"

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kPoolSets = 1024;

struct Session {
    uint64_t id;
    int64_t h;
    int call = 0;
    std::vector<float> q, qd, u;
};

double pct(std::vector<double> &v, double p) {
    if (v.empty()) return 0.0;
    const size_t k = std::min(v.size() - 1, static_cast<size_t>(p * static_cast<double>(v.size())));
    std::nth_element(v.begin(), v.begin() + static_cast<long>(k), v.end());
    return v[k];
}

}  // namespace

extern "C" int frg_loadgen_run(frg_server *srv, const frg_loadgen_cfg *cfg, frg_loadgen_result *res) {
    if (!srv || !cfg || !res || cfg->calls < 1 || cfg->threads < 1) return 1;
    if (frg_model_dofs() != 7) return 1;  // the sessions sample the iiwa_14's joint limits
    std::memset(res, 0, sizeof(*res));
    const float lim[7] = {2.96705972839f, 2.09439510239f, 2.96705972839f, 2.09439510239f,
                          2.96705972839f, 2.09439510239f, 3.05432619099f};
    std::mutex mu;  // sessions, req_to_session, samples, result counters
    std::unordered_map<uint64_t, Session> sessions;  // key = session id = the server's traj_id
    std::vector<std::vector<double>> lat(cfg->threads), lat64(cfg->threads);
    std::vector<double> batch_sum(cfg->threads, 0.0);
    std::atomic<uint64_t> next_id{1}, started{0}, active{0}, calls{0}, knots{0}, done_sessions{0}, errors{0};
    std::atomic<bool> window_open{true};
    int sampled_knots = 0;
    const uint64_t limit = cfg->total_sessions > 0 ? static_cast<uint64_t>(cfg->total_sessions) : UINT64_MAX;
    const bool on_device = cfg->source == 1;
    int max_h = cfg->n_horizons > 0 ? 0 : cfg->horizon_hi;
    for (int i = 0; i < cfg->n_horizons; i++) max_h = std::max(max_h, cfg->horizons[i]);
    // source 1: iterate j of set s is [q | qd | u], each 7 * max_h floats, at
    // (s * calls + j) * 3 * n_max
    const size_t n_max = 7 * static_cast<size_t>(std::max(max_h, 1));
    std::vector<float> pool_host;
    float *pool_dev = nullptr;
    auto iterate = [&](const float *base, uint64_t sid, int j) {
        return base + (static_cast<size_t>(sid % kPoolSets) * cfg->calls + j) * 3 * n_max;
    };
    if (on_device) {
        std::mt19937_64 prng(cfg->seed ^ 0x9e3779b97f4a7c15ull);
        std::uniform_real_distribution<float> unit(-1.0f, 1.0f);
        std::normal_distribution<float> noise(0.0f, static_cast<float>(cfg->sigma));
        pool_host.resize(static_cast<size_t>(kPoolSets) * cfg->calls * 3 * n_max);
        for (int set = 0; set < kPoolSets; set++) {
            float *it0 = pool_host.data() + static_cast<size_t>(set) * cfg->calls * 3 * n_max;
            for (size_t i = 0; i < n_max; i++) {
                it0[i] = lim[i % 7] * unit(prng);
                it0[n_max + i] = 2.0f * unit(prng);
                it0[2 * n_max + i] = 20.0f * unit(prng);
            }
            for (int j = 1; j < cfg->calls; j++)  // iterate j = iterate j - 1 + N(0, sigma)
                for (size_t i = 0; i < 3 * n_max; i++)
                    it0[j * 3 * n_max + i] = it0[(j - 1) * 3 * n_max + i] + noise(prng);
        }
        if (cudaMalloc(&pool_dev, sizeof(float) * pool_host.size()) != cudaSuccess ||
            cudaMemcpy(pool_dev, pool_host.data(), sizeof(float) * pool_host.size(), cudaMemcpyHostToDevice) !=
                cudaSuccess) {
            cudaFree(pool_dev);
            return 1;
        }
    }
    const auto t0 = Clock::now();  // after the staging: the run's clock
    auto elapsed = [&] { return std::chrono::duration<double>(Clock::now() - t0).count(); };

    auto submit = [&](Session &s) -> bool {
        uint64_t rid = 0;
        frg_status st;
        if (on_device) {
            const float *it = iterate(pool_dev, s.id, s.call);
            st = frg_server_submit_device(srv, s.id, s.h, it, it + n_max, it + 2 * n_max, 0, &rid);
        } else {
            st = frg_server_submit(srv, s.id, s.h, s.q.data(), s.qd.data(), s.u.data(), &rid);
        }
        if (st != FRG_OK) {
            errors++;
            return false;
        }
        return true;
    };
    auto start_session = [&](std::mt19937_64 &rng) {
        std::uniform_real_distribution<float> unit(-1.0f, 1.0f);
        Session s;
        s.id = next_id++;
        s.h = cfg->n_horizons > 0 ? cfg->horizons[rng() % static_cast<uint64_t>(cfg->n_horizons)]
                                  : cfg->horizon_lo + static_cast<int64_t>(
                                        rng() % static_cast<uint64_t>(cfg->horizon_hi - cfg->horizon_lo + 1));
        const size_t n = 7 * static_cast<size_t>(s.h);
        s.q.resize(n);
        s.qd.resize(n);
        s.u.resize(n);
        for (size_t i = 0; i < n; i++) {
            s.q[i] = lim[i % 7] * unit(rng);
            s.qd[i] = 2.0f * unit(rng);
            s.u[i] = 20.0f * unit(rng);
        }
        started++;
        active++;
        Session *sp;
        {
            std::lock_guard<std::mutex> lk(mu);
            sp = &sessions.emplace(s.id, std::move(s)).first->second;
        }
        if (!submit(*sp)) {
            std::lock_guard<std::mutex> lk(mu);
            sessions.erase(sp->id);
            active--;
        }
    };

    auto client = [&](int tid) {
        std::mt19937_64 rng(cfg->seed * 1000003ull + static_cast<uint64_t>(tid));
        std::normal_distribution<float> noise(0.0f, static_cast<float>(cfg->sigma));
        std::uniform_real_distribution<double> u01(0.0, 1.0);
        std::exponential_distribution<double> gap(cfg->mode == 0 && cfg->rate > 0 ? cfg->rate : 1.0);
        double next_arrival = 0.0;
        for (;;) {
            const double now = elapsed();
            const bool window = now < cfg->duration_s && started < limit && cfg->mode != 2;
            if (!window) window_open = false;
            if (tid == 0 && window) {
                if (cfg->mode == 0)
                    while (next_arrival <= now && started < limit) {
                        start_session(rng);
                        next_arrival += gap(rng);
                    }
                else {  // top up to `concurrency` once per pass, so the clock is re-read
                    const uint64_t have = active.load();
                    const uint64_t want = have < static_cast<uint64_t>(cfg->concurrency) ? cfg->concurrency - have : 0;
                    for (uint64_t i = 0; i < want && started < limit; i++) start_session(rng);
                }
            }
            if (!window_open && active == 0) break;
            frg_request_info info;
            const frg_status st = frg_server_wait_any(srv, (tid == 0 && window) ? 100 : 20000, &info);
            if (st == FRG_ERR_TIMEOUT) continue;
            if (st != FRG_OK) {
                errors++;
                break;
            }
            Session *sp = nullptr;
            long long dev_sample = -1;  // knot offset of a sampled device-resident call
            {
                std::lock_guard<std::mutex> lk(mu);
                auto it = sessions.find(info.traj_id);
                if (it == sessions.end()) continue;
                sp = &it->second;
                if (info.status == FRG_OK && cfg->sample_frac > 0 && u01(rng) < cfg->sample_frac &&
                    sampled_knots + sp->h <= cfg->sample_cap && res->samples < static_cast<uint64_t>(cfg->sample_cap)) {
                    const size_t k0 = static_cast<size_t>(sampled_knots), n = static_cast<size_t>(sp->h);
                    const float *in[3] = {sp->q.data(), sp->qd.data(), sp->u.data()};
                    if (on_device) {
                        const float *it = iterate(pool_host.data(), sp->id, sp->call);
                        in[0] = it;
                        in[1] = it + n_max;
                        in[2] = it + 2 * n_max;
                        dev_sample = static_cast<long long>(k0);
                    } else {
                        std::memcpy(cfg->sample_dqdd + 98 * k0, info.dqdd, 392 * n);
                        std::memcpy(cfg->sample_qdd + 7 * k0, info.qdd, 28 * n);
                        std::memcpy(cfg->sample_minv + 49 * k0, info.minv, 196 * n);
                    }
                    std::memcpy(cfg->sample_q + 7 * k0, in[0], 28 * n);
                    std::memcpy(cfg->sample_qd + 7 * k0, in[1], 28 * n);
                    std::memcpy(cfg->sample_u + 7 * k0, in[2], 28 * n);
                    cfg->sample_h[res->samples++] = sp->h;
                    sampled_knots += static_cast<int>(sp->h);
                }
            }
            if (dev_sample >= 0) {  // the call's results are in its device slot until its next call
                const size_t k0 = static_cast<size_t>(dev_sample), n = static_cast<size_t>(sp->h);
                if (cudaMemcpy(cfg->sample_dqdd + 98 * k0, info.dev_dqdd, 392 * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
                    cudaMemcpy(cfg->sample_qdd + 7 * k0, info.dev_qdd, 28 * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
                    cudaMemcpy(cfg->sample_minv + 49 * k0, info.dev_minv, 196 * n, cudaMemcpyDeviceToHost) != cudaSuccess)
                    errors++;
            }
            Session &s = *sp;  // only this thread touches s until its next call completes
            if (info.status != FRG_OK) errors++;
            lat[tid].push_back(info.latency_us);
            if (s.h == 64) lat64[tid].push_back(info.latency_us);
            batch_sum[tid] += info.batch_requests;
            calls++;
            knots += static_cast<uint64_t>(s.h);
            bool finished = ++s.call >= cfg->calls;
            if (!finished) {
                if (!on_device)
                    for (auto *v : {&s.q, &s.qd, &s.u})
                        for (float &x : *v) x += noise(rng);
                finished = !submit(s);
            }
            if (finished) {
                const uint64_t sid = s.id;
                frg_server_release(srv, sid);
                {
                    std::lock_guard<std::mutex> lk(mu);
                    sessions.erase(sid);
                }
                done_sessions++;
                active--;
            }
        }
    };
    if (cfg->mode == 2) {  // every session's first call is queued before any client runs
        std::mt19937_64 rng(cfg->seed);
        while (started < limit) start_session(rng);
    }
    std::vector<std::thread> ths;
    for (int t = 1; t < cfg->threads; t++) ths.emplace_back(client, t);
    client(0);
    for (auto &t : ths) t.join();

    cudaFree(pool_dev);
    res->calls = calls;
    res->knots = knots;
    res->sessions = done_sessions;
    res->errors = errors;
    res->elapsed_s = elapsed();
    res->sample_knots = static_cast<uint64_t>(sampled_knots);
    res->calls_per_s = res->calls / res->elapsed_s;
    res->knots_per_s = res->knots / res->elapsed_s;
    std::vector<double> all, all64;
    double bsum = 0;
    for (int t = 0; t < cfg->threads; t++) {
        all.insert(all.end(), lat[t].begin(), lat[t].end());
        all64.insert(all64.end(), lat64[t].begin(), lat64[t].end());
        bsum += batch_sum[t];
    }
    if (!all.empty()) {
        double sum = 0;
        for (double x : all) sum += x;
        res->mean_us = sum / static_cast<double>(all.size());
        res->max_us = *std::max_element(all.begin(), all.end());
        res->mean_batch_requests = bsum / static_cast<double>(all.size());
        res->p50_us = pct(all, 0.50);
        res->p90_us = pct(all, 0.90);
        res->p99_us = pct(all, 0.99);
    }
    res->p50_h64_us = pct(all64, 0.50);
    res->p99_h64_us = pct(all64, 0.99);
    return res->errors ? 2 : 0;
}
