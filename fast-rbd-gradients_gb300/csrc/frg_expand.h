// Host threads that expand packed Minv (upper triangle, kMinvPackedN floats
// per knot, column by column) into the dense symmetric N x N form the API
// returns.  The pipelined host-buffer call sends Minv over the host link
// packed -- 112 instead of 196 B per knot at 7 joints -- and expands one batch
// here while the next batch's results stream in.
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <mutex>
#include <thread>
#include <vector>

#include "frg_dims.h"

class MinvExpander {
  public:
    explicit MinvExpander(int threads) {
        for (int i = 0; i < threads; i++) workers_.emplace_back([this] { work(); });
    }
    ~MinvExpander() {
        {
            std::lock_guard<std::mutex> l(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : workers_) t.join();
    }
    MinvExpander(const MinvExpander &) = delete;
    MinvExpander &operator=(const MinvExpander &) = delete;

    // Starts expanding n knots from packed into dense (one job at a time:
    // wait() for the previous one first).
    void start(const float *packed, float *dense, size_t n) {
        {
            std::lock_guard<std::mutex> l(m_);
            src_ = packed;
            dst_ = dense;
            n_ = n;
            chunks_ = (n + kChunk - 1) / kChunk;
            done_.store(0);
            job_ = job_ == 0xffffffffull ? 1 : job_ + 1;  // never 0, a worker's initial `seen`
            ticket_.store(job_ << 32);
        }
        cv_.notify_all();
    }
    // Blocks until the current job (if any) is complete.
    void wait() {
        std::unique_lock<std::mutex> l(m_);
        done_cv_.wait(l, [this] { return done_.load() >= chunks_; });
    }

  private:
    static constexpr size_t kChunk = 1024;  // knots per work item

    // One knot, every index a compile-time constant: column c of the dense
    // matrix is packed column c for rows r <= c and packed column r, entry c
    // for rows r > c.
    template <int C = 0>
    static inline void expand_knot(const float *__restrict p, float *__restrict d) {
        if constexpr (C < frg::kN) {
            expand_col<C, 0>(p, d);
            expand_knot<C + 1>(p, d);
        }
    }
    template <int C, int R>
    static inline void expand_col(const float *__restrict p, float *__restrict d) {
        if constexpr (R < frg::kN) {
            constexpr int lo = R < C ? R : C, hi = R < C ? C : R;
            d[R + frg::kN * C] = p[hi * (hi + 1) / 2 + lo];
            expand_col<C, R + 1>(p, d);
        }
    }

    void work() {
        unsigned long long seen = 0;
        for (;;) {
            const float *src;
            float *dst;
            size_t n, chunks;
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return stop_ || job_ != seen; });
                if (stop_) return;
                seen = job_;
                src = src_;
                dst = dst_;
                n = n_;
                chunks = chunks_;
            }
            // Chunks are claimed with a compare-and-swap on (job, next chunk): a
            // worker still in an earlier job can never take a chunk of this one.
            for (;;) {
                unsigned long long v = ticket_.load();
                size_t c = 0;
                bool claimed = false;
                while ((v >> 32) == seen && (c = static_cast<size_t>(v & 0xffffffffull)) < chunks)
                    if (ticket_.compare_exchange_weak(v, v + 1)) {
                        claimed = true;
                        break;
                    }
                if (!claimed) break;
                const size_t k0 = c * kChunk, k1 = std::min(n, k0 + kChunk);
                for (size_t k = k0; k < k1; k++) expand_knot(src + frg::kMinvPackedN * k, dst + frg::kMinvN * k);
                if (done_.fetch_add(1) + 1 == chunks) {
                    std::lock_guard<std::mutex> l(m_);
                    done_cv_.notify_all();
                }
            }
        }
    }

    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    const float *src_ = nullptr;
    float *dst_ = nullptr;
    size_t n_ = 0, chunks_ = 0;
    std::atomic<unsigned long long> ticket_{0};  // job << 32 | next chunk
    std::atomic<size_t> done_{0};
    unsigned long long job_ = 0;
    bool stop_ = false;
};
