// C entry points around the reference's own CPU recursions
// (helpers_CPU/dynamicsGradient.h, helpers_CPU/minv.h, helpers_CPU/math.h),
// compiled UNMODIFIED from the reference tree behind oracle/eigen_shim.
//
// ORACLE TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into
// oracle/_ref/libfrg_ref.so where the reference sources are present; used to
// validate the C restatement (oracle/frg_oracle.c) and to generate the golden
// fixtures under tests/golden/.  Never linked into the product library.
//
// Per knot this runs the reference's full forward-dynamics-gradient path
// forwardDynamicsGradientThreaded<T, QDD_MINV_PASSED_IN=false, MPC, VD, EXTERNAL_TI=true>
// (helpers_CPU/dynamicsGradient.h:925-934), which computes q̈ and the upper
// triangle of Minv on the way (:881-896) and finishes with -Minv·[dτ/dq|dτ/dq̇]
// (:933).  knot.qdd is zeroed first: the setup reads it as an input (:877, :634).
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <vector>
#include <algorithm>
#include <chrono>
#include "utils/ReusableThreads.h"
#include "helpers_CPU/dynamicsGradient.h"

namespace {

template <typename T, bool MPC, bool VD>
void run_knots(int n, const T *q, const T *qd, const T *u, T *dqdd, T *qdd, T *minv, T *Ts, T *Is) {
    for (int k = 0; k < n; k++) {
        knot<T> kn;
        std::memset(&kn, 0, sizeof(kn));
        for (int i = 0; i < NUM_POS; i++) {
            kn.q[i] = q[NUM_POS * k + i];
            kn.qd[i] = qd[NUM_POS * k + i];
            kn.u[i] = u[NUM_POS * k + i];
        }
        forwardDynamicsGradientThreaded<T, false, MPC, VD, true>(&dqdd[2 * NUM_POS * NUM_POS * k], &kn, Ts, Is);
        for (int i = 0; i < NUM_POS; i++) qdd[NUM_POS * k + i] = kn.qdd[i];
        triangularToDense<T, NUM_POS, true>(kn.Minv);
        for (int i = 0; i < NUM_POS * NUM_POS; i++) minv[NUM_POS * NUM_POS * k + i] = kn.Minv[i];
    }
}

template <typename T>
int dispatch(int n, const T *q, const T *qd, const T *u, int damping, int mpc, T *dqdd, T *qdd, T *minv) {
    std::vector<T> Ts(36 * NUM_POS), Is(36 * NUM_POS);
    initTransforms(Ts.data());
    initInertiaTensors(Is.data());
    if (!mpc && !damping) run_knots<T, false, false>(n, q, qd, u, dqdd, qdd, minv, Ts.data(), Is.data());
    else if (!mpc && damping) run_knots<T, false, true>(n, q, qd, u, dqdd, qdd, minv, Ts.data(), Is.data());
    else if (mpc && !damping) run_knots<T, true, false>(n, q, qd, u, dqdd, qdd, minv, Ts.data(), Is.data());
    else run_knots<T, true, true>(n, q, qd, u, dqdd, qdd, minv, Ts.data(), Is.data());
    return 0;
}

// The time_CPU.cpp:30-54 driver shape: contiguous knot chunks per thread on a
// ReusableThreads pool; reference mode QDD_MINV_PASSED_IN=false (full path).
constexpr int kRefThreads = 8;
template <typename T>
void chunk_task(int n, const T *q, const T *qd, const T *u, T *dqdd, T *qdd, T *minv, int tid) {
    int per = n / kRefThreads, k0 = per * tid, k1 = (tid == kRefThreads - 1) ? n : per * (tid + 1);
    std::vector<T> Ts(36 * NUM_POS), Is(36 * NUM_POS);
    initTransforms(Ts.data());
    initInertiaTensors(Is.data());
    run_knots<T, false, false>(k1 - k0, q + NUM_POS * k0, qd + NUM_POS * k0, u + NUM_POS * k0,
                               dqdd + 98 * k0, qdd + NUM_POS * k0, minv + 49 * k0, Ts.data(), Is.data());
}

}  // namespace

extern "C" {

int frg_ref_gradient_f64(int n, const double *q, const double *qd, const double *u, int damping, int mpc,
                         double *dqdd, double *qdd, double *minv) {
    return dispatch<double>(n, q, qd, u, damping, mpc, dqdd, qdd, minv);
}

int frg_ref_gradient_f32(int n, const float *q, const float *qd, const float *u, int damping, int mpc,
                         float *dqdd, float *qdd, float *minv) {
    return dispatch<float>(n, q, qd, u, damping, mpc, dqdd, qdd, minv);
}

// Wall time in seconds of `iters` passes of the threaded FP32 full path over n knots.
double frg_ref_time_threaded_f32(int n, const float *q, const float *qd, const float *u,
                                 float *dqdd, float *qdd, float *minv, int iters) {
    ReusableThreads<kRefThreads> pool;
    auto t0 = std::chrono::steady_clock::now();
    for (int it = 0; it < iters; it++) {
        for (int tid = 0; tid < kRefThreads; tid++)
            pool.addTask(tid, &chunk_task<float>, n, q, qd, u, dqdd, qdd, minv, tid);
        pool.sync();
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

int frg_ref_threads(void) { return kRefThreads; }

}  // extern "C"
