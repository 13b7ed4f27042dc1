// Continuous-batching gradient server (include/frg.h frg_server_*).
//
// Requests are gradient calls of trajectories (MPC / iLQR style: one
// trajectory makes many calls).  Each trajectory holds, from its first call to
// frg_server_release, a slot of 4N + 3N^2 floats per knot (175 for 7 joints:
// [q | qd | u | dqdd | qdd | minv]) in a capped device pool, mirrored at the same offset in a pinned
// host arena.  Admission is by free pool bytes: a trajectory whose slot does
// not fit waits (an admission stall) until releases free enough of the pool.
//
// A dispatcher thread folds every ready request into the next batch (up to
// max_batch_knots knots), uploads the batch's descriptor list with one copy
// and launches the persistent server kernel.  The kernel reads each call's
// inputs where the call has them: the pinned host slot (frg_server_submit
// copies host inputs there), the caller's device arrays
// (frg_server_submit_device), or the trajectory's device slot
// (frg_server_submit_resident: the inputs of its previous call, or what the
// caller wrote there in place).  Inputs from elsewhere are mirrored into the
// device slot; results go to the device slot, and to the host slot when the
// caller wants them there.  Up to max_inflight batches run at once on their
// own streams, so requests that arrive while others are on the GPU start
// without waiting for them.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "frg.h"
#include "frg_internal.h"
#include "frg_kernels.cuh"

namespace {

using Clock = std::chrono::steady_clock;
constexpr size_t kGranule = 256;
constexpr size_t kFloatsPerKnot = frg::kSlotN;
constexpr int kIdleSpinUs = 200;

double us_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::micro>(b - a).count();
}

// First-fit allocator of [0, cap) in 256-byte granules, with coalescing.
class ArenaAllocator {
public:
    void init(size_t cap) {
        cap_ = cap / kGranule * kGranule;
        free_.clear();
        if (cap_) free_[0] = cap_;
        used_ = peak_ = 0;
    }
    bool alloc(size_t bytes, size_t *off) {
        bytes = (bytes + kGranule - 1) / kGranule * kGranule;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            *off = it->first;
            const size_t rest = it->second - bytes;
            const size_t at = it->first + bytes;
            free_.erase(it);
            if (rest) free_[at] = rest;
            used_ += bytes;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + kGranule - 1) / kGranule * kGranule;
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t cap() const { return cap_; }
    size_t used() const { return used_; }
    size_t peak() const { return peak_; }

private:
    std::map<size_t, size_t> free_;
    size_t cap_ = 0, used_ = 0, peak_ = 0;
};

struct Traj {
    uint64_t id = 0;
    int64_t h = 0;
    size_t off = 0, bytes = 0;
    bool admitted = false;
    bool busy = false;             // a call queued or in flight
    bool inputs_resident = false;  // the device slot holds a complete q, qd, u
};

enum class ReqState { Admission, Ready, InFlight, Done };
// Where a call's inputs are: copied to the pinned host slot, the caller's
// device arrays, or the trajectory's device slot.
enum class Source { Host, Device, Resident };

struct Request {
    uint64_t id = 0, traj = 0;
    int64_t h = 0;
    ReqState state = ReqState::Admission;
    Source src = Source::Host;
    const float *dq = nullptr, *dqd = nullptr, *du = nullptr;  // Source::Device
    bool host_results = true;
    frg_status status = FRG_OK;
    std::vector<float> staged;  // inputs of a request waiting for admission
    Clock::time_point t_submit, t_launch, t_done;
    uint64_t batch = 0;
    int batch_requests = 0;
    bool consumed = false;
};

struct Batch {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    // one descriptor block, pinned on the host and mirrored on the device:
    // the batch's segments, then (16-byte aligned) its tile list, uploaded by
    // one copy
    unsigned char *h_desc = nullptr, *d_desc = nullptr;
    unsigned int *d_counter = nullptr;
    std::vector<Request *> reqs;
    bool busy = false;
    uint64_t id = 0;
};

}  // namespace

struct frg_server {
    frg_ctx *ctx = nullptr;
    frg_server_options opt{};
    frg::LaunchShape shape;          // batches above latency_mapping_max_knots
    frg::LaunchShape latency_shape;  // 8 lanes per knot, for small batches
    float *dev_pool = nullptr;
    float *host_pool = nullptr;
    ArenaAllocator arena;
    int max_reqs_per_batch = 0, max_tiles_per_batch = 0;

    std::mutex mu;
    std::condition_variable cv_dispatch, cv_done;
    std::unordered_map<uint64_t, Traj> trajs;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::deque<Request *> admission, ready;
    std::deque<uint64_t> completions;
    std::vector<Batch> batches;
    uint64_t next_req = 1, next_batch = 1;
    bool stop = false;
    std::atomic<bool> kick{false};  // set by submit/release: work for the dispatcher
    std::string fatal;
    frg_server_stats st{};
    std::thread dispatcher;

    void run();
    void launch_batch(Batch &b, std::unique_lock<std::mutex> &lk);
    void complete_batch(Batch &b, cudaError_t err, Clock::time_point now);
    bool admit(Traj &t, int64_t h);
    float *host_slot(const Traj &t) const { return host_pool + t.off / sizeof(float); }
    float *dev_slot(const Traj &t) const { return dev_pool + t.off / sizeof(float); }
};

namespace {

void fill_info(const frg_server *s, const Request &r, frg_request_info *info) {
    if (!info) return;
    std::memset(info, 0, sizeof(*info));
    info->request_id = r.id;
    info->traj_id = r.traj;
    info->horizon = r.h;
    info->status = r.status;
    info->batch_id = r.batch;
    info->batch_requests = r.batch_requests;
    if (r.state == ReqState::Done) {
        info->latency_us = us_between(r.t_submit, r.t_done);
        info->queue_us = us_between(r.t_submit, r.t_launch);
        auto it = s->trajs.find(r.traj);
        if (r.status == FRG_OK && it != s->trajs.end() && it->second.admitted) {
            const Traj &t = it->second;
            const float *hs = s->host_slot(t), *ds = s->dev_slot(t);
            const int64_t h = t.h;
            if (r.host_results) {
                info->dqdd = hs + frg::kSlotDqdd * h;
                info->qdd = hs + frg::kSlotQdd * h;
                info->minv = hs + frg::kSlotMinv * h;
            }
            info->dev_q = ds;
            info->dev_qd = ds + frg::kSlotQd * h;
            info->dev_u = ds + frg::kSlotU * h;
            info->dev_dqdd = ds + frg::kSlotDqdd * h;
            info->dev_qdd = ds + frg::kSlotQdd * h;
            info->dev_minv = ds + frg::kSlotMinv * h;
        }
    }
}

}  // namespace

bool frg_server::admit(Traj &t, int64_t h) {
    size_t off = 0;
    const size_t bytes = kFloatsPerKnot * sizeof(float) * static_cast<size_t>(h);
    if (!arena.alloc(bytes, &off)) return false;
    t.off = off;
    t.bytes = bytes;
    t.h = h;
    t.admitted = true;
    st.pool_bytes_used = arena.used();
    st.pool_bytes_peak = arena.peak();
    return true;
}

void frg_server::complete_batch(Batch &b, cudaError_t err, Clock::time_point now) {
    for (Request *r : b.reqs) {
        r->state = ReqState::Done;
        r->t_done = now;
        r->status = err == cudaSuccess ? FRG_OK : FRG_ERR_CUDA;
        auto it = trajs.find(r->traj);
        if (it != trajs.end()) {
            it->second.busy = false;
            it->second.inputs_resident = err == cudaSuccess;  // the kernel left this call's inputs in the slot
        }
        completions.push_back(r->id);
        st.completed++;
        st.knots += static_cast<uint64_t>(r->h);
    }
    if (completions.size() > 4 * reqs.size() + 4096) {  // drop ids already taken by wait/poll
        std::deque<uint64_t> keep;
        for (uint64_t id : completions)
            if (reqs.count(id)) keep.push_back(id);
        completions.swap(keep);
    }
    if (err != cudaSuccess && fatal.empty()) fatal = std::string("server batch failed: ") + cudaGetErrorString(err);
    b.reqs.clear();
    b.busy = false;
}

void frg_server::run() {
    DeviceGuard g(ctx->device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        // completions of batches in flight
        bool inflight = false, done_any = false;
        const auto now = Clock::now();
        for (Batch &b : batches) {
            if (!b.busy) continue;
            const cudaError_t q = cudaEventQuery(b.done);
            if (q == cudaErrorNotReady) {
                inflight = true;
                continue;
            }
            complete_batch(b, q, now);
            done_any = true;
        }
        if (done_any) cv_done.notify_all();
        // admission, FIFO: a trajectory that does not fit blocks the ones behind it
        while (!admission.empty()) {
            Request *r = admission.front();
            Traj &t = trajs[r->traj];
            if (!admit(t, r->h)) break;
            if (r->src == Source::Host)
                std::memcpy(host_slot(t), r->staged.data(), sizeof(float) * 3 * frg::kN * static_cast<size_t>(r->h));
            r->staged.clear();
            r->staged.shrink_to_fit();
            r->state = ReqState::Ready;
            ready.push_back(r);
            admission.pop_front();
        }
        if (stop && !inflight && ready.empty()) break;
        Batch *free_b = nullptr;
        for (Batch &b : batches)
            if (!b.busy) {
                free_b = &b;
                break;
            }
        if (free_b && !ready.empty()) {
            launch_batch(*free_b, lk);
            continue;
        }
        if (inflight) {  // poll the batches in flight again shortly
            lk.unlock();
            std::this_thread::yield();
            lk.lock();
            continue;
        }
        // idle: spin briefly for new work (a sleeping dispatcher costs a
        // thread wake-up on the next submit), then block
        kick.store(false);
        lk.unlock();
        const auto spin_until = Clock::now() + std::chrono::microseconds(kIdleSpinUs);
        while (!kick.load(std::memory_order_acquire) && Clock::now() < spin_until) std::this_thread::yield();
        lk.lock();
        if (!kick.load() && ready.empty() && !stop) cv_dispatch.wait(lk);
    }
}

// Folds ready requests into batch b and launches it (called with mu held;
// releases it around the CUDA calls).
void frg_server::launch_batch(Batch &b, std::unique_lock<std::mutex> &lk) {
    int64_t knots = 0;
    while (!ready.empty() && static_cast<int>(b.reqs.size()) < max_reqs_per_batch) {
        Request *r = ready.front();
        if (!b.reqs.empty() && knots + r->h > opt.max_batch_knots) break;
        ready.pop_front();
        b.reqs.push_back(r);
        knots += r->h;
    }
    b.id = next_batch++;
    const auto t_launch = Clock::now();
    const int nseg = static_cast<int>(b.reqs.size());
    frg::ServeSegment *h_segs = reinterpret_cast<frg::ServeSegment *>(b.h_desc);
    long long begin = 0;
    for (int i = 0; i < nseg; i++) {
        Request *r = b.reqs[i];
        const Traj &t = trajs[r->traj];
        float *hs = host_slot(t), *ds = dev_slot(t);
        const long long h = r->h;
        const float *q = r->dq, *qd = r->dqd, *u = r->du;  // Source::Device
        if (r->src == Source::Host) {
            q = hs;
            qd = hs + frg::kSlotQd * h;
            u = hs + frg::kSlotU * h;
        } else if (r->src == Source::Resident) {
            q = ds;
            qd = ds + frg::kSlotQd * h;
            u = ds + frg::kSlotU * h;
        }
        h_segs[i] = frg::ServeSegment{q, qd, u, ds, r->host_results ? hs : nullptr, h, begin};
        begin += r->h;
        r->state = ReqState::InFlight;
        r->t_launch = t_launch;
        r->batch = b.id;
        r->batch_requests = nseg;
    }
    h_segs[nseg] = frg::ServeSegment{nullptr, nullptr, nullptr, nullptr, nullptr, 0, begin};
    const size_t tiles_off = (sizeof(frg::ServeSegment) * (nseg + 1) + 15) / 16 * 16;
    int *h_tiles = reinterpret_cast<int *>(b.h_desc + tiles_off);
    const int ntiles = static_cast<int>((begin + 31) / 32);
    int s = 0;
    for (int tile = 0; tile < ntiles; tile++) {
        while (s + 1 < nseg && h_segs[s + 1].knot_begin <= static_cast<long long>(tile) * 32) s++;
        h_tiles[tile] = s;
    }
    b.busy = true;
    st.launches++;
    lk.unlock();
    cudaError_t e = cudaMemcpyAsync(b.d_desc, b.h_desc, tiles_off + sizeof(int) * ntiles, cudaMemcpyHostToDevice,
                                    b.stream);
    frg::LaunchShape sh = shape;
    if (begin <= opt.latency_mapping_max_knots) sh = latency_shape;
    if (e == cudaSuccess)
        e = frg::launch_serve(ctx->damping, ctx->mpc, sh, ctx->num_sms,
                              reinterpret_cast<const frg::ServeSegment *>(b.d_desc), nseg,
                              reinterpret_cast<const int *>(b.d_desc + tiles_off), ntiles, b.d_counter, b.stream);
    if (e == cudaSuccess) e = cudaEventRecord(b.done, b.stream);
    lk.lock();
    if (e != cudaSuccess) {
        complete_batch(b, e, Clock::now());
        cv_done.notify_all();
    }
}

extern "C" {

void frg_server_options_default(frg_server_options *opt) {
    if (!opt) return;
    opt->pool_bytes = size_t(1) << 30;
    opt->max_batch_knots = 1 << 16;
    opt->max_inflight = 3;
    opt->warps_per_cta = 0;
    opt->ctas_per_sm = 0;
    opt->latency_mapping_max_knots = 4096;
}

frg_status frg_server_create(frg_ctx *ctx, const frg_server_options *opt_in, frg_server **out) {
    if (!ctx || !out) return FRG_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    frg_server_options opt;
    frg_server_options_default(&opt);
    if (opt_in) opt = *opt_in;
    if (opt.pool_bytes < kGranule || opt.max_batch_knots < 32 || opt.max_inflight < 1 || opt.max_inflight > 16 ||
        opt.warps_per_cta < 0 || opt.warps_per_cta > 8 || opt.ctas_per_sm < 0) {
        frg_set_error(ctx, "frg_server_create: invalid options");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    frg_server *s = new (std::nothrow) frg_server();
    if (!s) return FRG_ERR_OUT_OF_MEMORY;
    s->ctx = ctx;
    s->opt = opt;
    s->shape = ctx->ragged_shape;
    if (opt.warps_per_cta) s->shape.warps_per_cta = opt.warps_per_cta;
    if (opt.ctas_per_sm) s->shape.ctas_per_sm = opt.ctas_per_sm;
    if (s->shape.lanes_per_knot == 8) s->shape.lanes_per_knot = 1;  // big batches: throughput mapping
    s->latency_shape.warps_per_cta = 4;
    s->latency_shape.ctas_per_sm = std::max(1, frg::max_ctas_per_sm(4, 8));
    s->latency_shape.lanes_per_knot = 8;
    s->max_tiles_per_batch = opt.max_batch_knots / 32 + 2;
    s->max_reqs_per_batch = std::min(opt.max_batch_knots, 8192);
    DeviceGuard g(ctx->device);
    auto fail = [&](const char *what, cudaError_t e) {
        cudaGetLastError();
        frg_set_error(ctx, std::string("frg_server_create: ") + what + ": " + cudaGetErrorString(e));
        frg_server_destroy(s);
        return e == cudaErrorMemoryAllocation ? FRG_ERR_OUT_OF_MEMORY : FRG_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = frg::init_serve_kernels()) != cudaSuccess) return fail("kernel set-up", e);
    if ((e = frg::init_group_kernels()) != cudaSuccess) return fail("latency kernel set-up", e);
    if ((e = cudaMalloc(&s->dev_pool, opt.pool_bytes)) != cudaSuccess) return fail("device pool", e);
    if ((e = cudaHostAlloc(&s->host_pool, opt.pool_bytes, cudaHostAllocMapped | cudaHostAllocPortable)) != cudaSuccess)
        return fail("host arena", e);
    s->arena.init(opt.pool_bytes);
    s->batches.resize(static_cast<size_t>(opt.max_inflight));
    for (Batch &b : s->batches) {
        if ((e = cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream", e);
        if ((e = cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming)) != cudaSuccess) return fail("event", e);
        const size_t desc_bytes = sizeof(frg::ServeSegment) * (s->max_reqs_per_batch + 1) + 16 +
                                  sizeof(int) * s->max_tiles_per_batch;
        if ((e = cudaHostAlloc(&b.h_desc, desc_bytes, 0)) != cudaSuccess ||
            (e = cudaMalloc(&b.d_desc, desc_bytes)) != cudaSuccess ||
            (e = cudaMalloc(&b.d_counter, sizeof(unsigned int))) != cudaSuccess ||
            (e = cudaMemset(b.d_counter, 0, sizeof(unsigned int))) != cudaSuccess)
            return fail("batch buffers", e);
    }
    s->dispatcher = std::thread([s] { s->run(); });
    *out = s;
    return FRG_OK;
}

void frg_server_destroy(frg_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        // requests still waiting for admission can never run now
        for (Request *r : s->admission) {
            r->state = ReqState::Done;
            r->status = FRG_ERR_SHUTDOWN;
        }
        s->admission.clear();
    }
    s->kick.store(true);
    s->cv_dispatch.notify_all();
    if (s->dispatcher.joinable()) s->dispatcher.join();
    s->cv_done.notify_all();
    DeviceGuard g(s->ctx->device);
    for (Batch &b : s->batches) {
        if (b.stream) cudaStreamSynchronize(b.stream);
        if (b.stream) cudaStreamDestroy(b.stream);
        if (b.done) cudaEventDestroy(b.done);
        if (b.h_desc) cudaFreeHost(b.h_desc);
        cudaFree(b.d_desc);
        cudaFree(b.d_counter);
    }
    cudaFree(s->dev_pool);
    if (s->host_pool) cudaFreeHost(s->host_pool);
    delete s;
}

}  // extern "C"

namespace {

// One gradient call of trajectory traj_id over `horizon` knots whose inputs
// are at `src` (host arrays, copied before return; the caller's device arrays;
// or the trajectory's device slot, horizon ignored).
frg_status submit_call(frg_server *s, const char *who, uint64_t traj_id, int64_t horizon, Source src,
                       const float *q, const float *qd, const float *u, bool host_results, uint64_t *request_id) {
    if (!s) return FRG_ERR_INVALID_ARGUMENT;
    if (src != Source::Resident && (horizon <= 0 || !q || !qd || !u)) {
        frg_set_error(s->ctx, std::string(who) + ": horizon must be > 0 and q, qd, u non-null");
        return FRG_ERR_INVALID_ARGUMENT;
    }
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop) return FRG_ERR_SHUTDOWN;
    if (src == Source::Resident) {
        auto it = s->trajs.find(traj_id);
        if (it == s->trajs.end() || !it->second.admitted || !it->second.inputs_resident) {
            frg_set_error(s->ctx, std::string(who) + ": the trajectory has no resident inputs (no completed call)");
            return FRG_ERR_NOT_FOUND;
        }
        horizon = it->second.h;
    }
    const size_t bytes = kFloatsPerKnot * sizeof(float) * static_cast<size_t>(horizon);
    const size_t n7 = frg::kN * static_cast<size_t>(horizon);  // floats of one input array
    if (bytes > s->arena.cap()) {
        s->st.rejected++;
        frg_set_error(s->ctx, std::string(who) + ": horizon " + std::to_string(horizon) +
                                  " needs more than the whole device pool");
        return FRG_ERR_ADMISSION;
    }
    if (horizon / 32 + 2 > s->max_tiles_per_batch) {
        s->st.rejected++;
        frg_set_error(s->ctx, std::string(who) + ": horizon exceeds max_batch_knots");
        return FRG_ERR_ADMISSION;
    }
    Traj &t = s->trajs[traj_id];
    t.id = traj_id;
    if (t.busy) {
        frg_set_error(s->ctx, std::string(who) + ": trajectory has a call in flight");
        return FRG_ERR_NOT_READY;
    }
    if (t.admitted && t.h != horizon) {  // horizon changed: new slot
        s->arena.release(t.off, t.bytes);
        t.admitted = false;
        t.inputs_resident = false;
    }
    auto req = std::make_unique<Request>();
    Request *r = req.get();
    r->id = s->next_req++;
    r->traj = traj_id;
    r->h = horizon;
    r->src = src;
    r->host_results = host_results;
    if (src == Source::Device) {
        r->dq = q;
        r->dqd = qd;
        r->du = u;
    }
    r->t_submit = Clock::now();
    s->st.submitted++;
    t.busy = true;
    bool admitted = t.admitted || (s->admission.empty() && s->admit(t, horizon));
    if (admitted) {
        if (src == Source::Host) {
            float *slot = s->host_slot(t);
            lk.unlock();  // the slot belongs to this trajectory and no call of it is in flight
            std::memcpy(slot, q, sizeof(float) * n7);
            std::memcpy(slot + n7, qd, sizeof(float) * n7);
            std::memcpy(slot + 2 * n7, u, sizeof(float) * n7);
            lk.lock();
        }
        r->state = ReqState::Ready;
        s->ready.push_back(r);
    } else {
        if (src == Source::Host) {
            r->staged.resize(3 * n7);
            std::memcpy(r->staged.data(), q, sizeof(float) * n7);
            std::memcpy(r->staged.data() + n7, qd, sizeof(float) * n7);
            std::memcpy(r->staged.data() + 2 * n7, u, sizeof(float) * n7);
        }
        r->state = ReqState::Admission;
        s->admission.push_back(r);
        s->st.admission_stalls++;
    }
    s->reqs.emplace(r->id, std::move(req));
    if (request_id) *request_id = r->id;
    lk.unlock();
    s->kick.store(true, std::memory_order_release);
    s->cv_dispatch.notify_one();
    return FRG_OK;
}

}  // namespace

extern "C" {

frg_status frg_server_submit(frg_server *s, uint64_t traj_id, int64_t horizon, const float *q, const float *qd,
                             const float *u, uint64_t *request_id) {
    return submit_call(s, "frg_server_submit", traj_id, horizon, Source::Host, q, qd, u, true, request_id);
}

frg_status frg_server_submit_device(frg_server *s, uint64_t traj_id, int64_t horizon, const float *q,
                                    const float *qd, const float *u, unsigned int flags, uint64_t *request_id) {
    return submit_call(s, "frg_server_submit_device", traj_id, horizon, Source::Device, q, qd, u,
                       (flags & FRG_SERVE_HOST_RESULTS) != 0, request_id);
}

frg_status frg_server_submit_resident(frg_server *s, uint64_t traj_id, unsigned int flags, uint64_t *request_id) {
    return submit_call(s, "frg_server_submit_resident", traj_id, 0, Source::Resident, nullptr, nullptr, nullptr,
                       (flags & FRG_SERVE_HOST_RESULTS) != 0, request_id);
}

frg_status frg_server_slot(frg_server *s, uint64_t traj_id, frg_slot_info *out) {
    if (!s || !out) return FRG_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->trajs.find(traj_id);
    if (it == s->trajs.end() || !it->second.admitted || !it->second.inputs_resident) return FRG_ERR_NOT_FOUND;
    const Traj &t = it->second;
    if (t.busy) {
        frg_set_error(s->ctx, "frg_server_slot: trajectory has a call in flight");
        return FRG_ERR_NOT_READY;
    }
    float *ds = s->dev_slot(t);
    const int64_t h = t.h;
    out->horizon = h;
    out->q = ds;
    out->qd = ds + frg::kSlotQd * h;
    out->u = ds + frg::kSlotU * h;
    out->dqdd = ds + frg::kSlotDqdd * h;
    out->qdd = ds + frg::kSlotQdd * h;
    out->minv = ds + frg::kSlotMinv * h;
    return FRG_OK;
}

frg_status frg_server_poll(frg_server *s, uint64_t request_id, frg_request_info *info) {
    if (!s) return FRG_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end() || it->second->consumed) return FRG_ERR_NOT_FOUND;
    Request &r = *it->second;
    fill_info(s, r, info);
    if (r.state != ReqState::Done) return FRG_ERR_NOT_READY;
    r.consumed = true;
    s->reqs.erase(it);
    return FRG_OK;
}

frg_status frg_server_wait(frg_server *s, uint64_t request_id, int64_t timeout_us, frg_request_info *info) {
    if (!s) return FRG_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    // The request is looked up by id on every wake-up: while this thread
    // sleeps, a concurrent poll / wait_any may take the same completion and
    // free the request, so no pointer to it is held across the wait.
    auto live = [&]() -> Request * {
        auto it = s->reqs.find(request_id);
        return it == s->reqs.end() || it->second->consumed ? nullptr : it->second.get();
    };
    if (!live()) return FRG_ERR_NOT_FOUND;
    auto settled = [&] {
        const Request *r = live();
        return !r || r->state == ReqState::Done;
    };
    if (timeout_us < 0) s->cv_done.wait(lk, settled);
    else if (!s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), settled)) {
        if (const Request *r = live()) fill_info(s, *r, info);
        return FRG_ERR_TIMEOUT;
    }
    Request *r = live();
    if (!r) return FRG_ERR_NOT_FOUND;  // taken by another thread while this one waited
    fill_info(s, *r, info);
    r->consumed = true;
    s->reqs.erase(request_id);
    return FRG_OK;
}

frg_status frg_server_wait_any(frg_server *s, int64_t timeout_us, frg_request_info *info) {
    if (!s) return FRG_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto pending = [&] {
        while (!s->completions.empty()) {
            auto it = s->reqs.find(s->completions.front());
            if (it != s->reqs.end() && !it->second->consumed) return true;
            s->completions.pop_front();  // already taken by wait/poll
        }
        return false;
    };
    if (timeout_us < 0) s->cv_done.wait(lk, pending);
    else if (!s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), pending)) return FRG_ERR_TIMEOUT;
    const uint64_t id = s->completions.front();
    s->completions.pop_front();
    auto it = s->reqs.find(id);
    fill_info(s, *it->second, info);
    s->reqs.erase(it);
    return FRG_OK;
}

frg_status frg_server_release(frg_server *s, uint64_t traj_id) {
    if (!s) return FRG_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->trajs.find(traj_id);
        if (it == s->trajs.end()) return FRG_ERR_NOT_FOUND;
        if (it->second.busy) {
            frg_set_error(s->ctx, "frg_server_release: trajectory has a call in flight");
            return FRG_ERR_NOT_READY;
        }
        if (it->second.admitted) s->arena.release(it->second.off, it->second.bytes);
        s->trajs.erase(it);
        s->st.pool_bytes_used = s->arena.used();
    }
    s->kick.store(true, std::memory_order_release);
    s->cv_dispatch.notify_one();  // admission may proceed
    return FRG_OK;
}

frg_status frg_server_cancel(frg_server *s, uint64_t request_id) {
    if (!s) return FRG_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(request_id);
        if (it == s->reqs.end() || it->second->consumed) return FRG_ERR_NOT_FOUND;
        Request *r = it->second.get();
        if (r->state != ReqState::Admission && r->state != ReqState::Ready) {
            frg_set_error(s->ctx, "frg_server_cancel: the call is already on the GPU or done");
            return FRG_ERR_NOT_READY;
        }
        std::deque<Request *> &q = r->state == ReqState::Admission ? s->admission : s->ready;
        q.erase(std::find(q.begin(), q.end(), r));
        r->staged.clear();
        r->staged.shrink_to_fit();
        r->state = ReqState::Done;  // completed, without results: waiters wake and see the status
        r->status = FRG_ERR_CANCELLED;
        r->t_launch = r->t_done = Clock::now();
        auto t = s->trajs.find(r->traj);
        if (t != s->trajs.end()) t->second.busy = false;
        s->completions.push_back(r->id);
        s->st.cancelled++;
    }
    s->cv_done.notify_all();
    s->kick.store(true, std::memory_order_release);
    s->cv_dispatch.notify_one();  // the head of the admission queue may have changed
    return FRG_OK;
}

frg_status frg_server_get_stats(frg_server *s, frg_server_stats *out) {
    if (!s || !out) return FRG_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->pool_bytes_cap = s->arena.cap();
    out->pool_bytes_used = s->arena.used();
    out->pool_bytes_peak = s->arena.peak();
    out->queued_admission = s->admission.size();
    out->queued_ready = s->ready.size();
    return s->fatal.empty() ? FRG_OK : FRG_ERR_CUDA;
}

}  // extern "C"
