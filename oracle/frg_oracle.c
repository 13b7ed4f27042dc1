/* frg oracle: CPU restatement of the reference's iiwa_14 forward-dynamics
 * gradient (helpers_CPU/dynamicsGradient.h + helpers_CPU/minv.h), in FP64 and
 * FP32, plus a persistent-thread-pool driver shaped like time_CPU.cpp:30-54.
 *
 * ORACLE TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference arm load it (as oracle/libfrg_oracle.so),
 * and only as the checker or the timed CPU baseline.  The CUDA product path
 * never calls it and never falls back to it.
 *
 * Pinned against the reference itself: tests/golden/ holds outputs of the
 * reference's own helpers_CPU code (built by oracle/Makefile into oracle/_ref/)
 * and tests/test_oracle.py checks this file against them.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* g, as the reference's GRAVITY default (dynamicsGradient.h:7-9). */
static const double kGravity = 9.81;

/* The model: the same tables the kernels compile (FRG_MODEL_TABLES selects a
 * generated robot; default the iiwa_14 of utils/iiwa_14.urdf).
 *  - link inertial (Ixx Ixy Ixz Iyy Iyz Izz at the COM, COM x y z, mass): for
 *    the iiwa the constants the reference code-generates at
 *    dynamicsGradient.h:127-202 (urdf lines 31-37, 47-53, ..., 129-137);
 *  - F = R(rpy)^T of each joint frame, column-major (for the iiwa signed
 *    permutations: rpy (0,0,0) -> identity; (pi/2,0,pi) and (-pi/2,pi,0) ->
 *    w |-> (-w0, w2, w1); (pi/2,0,0) -> w |-> (w0, w2, -w1));
 *  - the joint origin xyz in the parent frame (the reference's tz_j1..ty_j7,
 *    dynamicsGradient.h:223-229). */
#ifdef FRG_MODEL_TABLES
#include FRG_MODEL_TABLES
#else
#include "../fast-rbd-gradients_gb300/csrc/frg_model_iiwa14.h"
#endif
#ifndef FRG_MODEL_NUM_JOINTS
#define FRG_MODEL_NUM_JOINTS 7
#endif
/* per-knot sizes for N joints: q, qd, u, qdd N; dqdd 2N^2; Minv N^2; fext 6N */
#define KN FRG_MODEL_NUM_JOINTS
#define KD (2 * KN * KN)
#define KM (KN * KN)
static const double kLinkInertial[KN][10] = FRG_MODEL_LINK_INERTIAL;
static const double kJointFT[KN][9] = FRG_MODEL_JOINT_F;
static const double kJointOrigin[KN][3] = FRG_MODEL_JOINT_ORIGIN;

#define REAL double
#define FN(name) name##_f64
#include "frg_oracle_impl.h"
#undef REAL
#undef FN
#undef SZ6
#undef NJ
#define REAL float
#define FN(name) name##_f32
#include "frg_oracle_impl.h"
#undef REAL
#undef FN

/* -------------------------------------------------------------- exports ---- */

/* Joint count N of the model compiled in (the per-knot sizes follow it). */
int frg_oracle_dofs(void) { return KN; }

int frg_oracle_gradient_f64(int n, const double *q, const double *qd, const double *u, const double *fext,
                            int damping, int mpc, double *dqdd, double *qdd, double *minv) {
    if (n < 0) return 1;
    for (int k = 0; k < n; k++)
        knot_gradient_f64(&q[KN * k], &qd[KN * k], &u[KN * k], fext ? &fext[6 * KN * k] : NULL, damping, mpc,
                          &dqdd[KD * k], &qdd[KN * k], &minv[KM * k]);
    return 0;
}

int frg_oracle_gradient_f32(int n, const float *q, const float *qd, const float *u, const float *fext,
                            int damping, int mpc, float *dqdd, float *qdd, float *minv) {
    if (n < 0) return 1;
    for (int k = 0; k < n; k++)
        knot_gradient_f32(&q[KN * k], &qd[KN * k], &u[KN * k], fext ? &fext[6 * KN * k] : NULL, damping, mpc,
                          &dqdd[KD * k], &qdd[KN * k], &minv[KM * k]);
    return 0;
}

/* Transforms and inertias alone, for the model-constant checks. */
void frg_oracle_model_f64(const double *q, double *X, double *I) {
    double s[KN], c[KN];
    for (int k = 0; k < KN; k++) { s[k] = sin(q[k]); c[k] = cos(q[k]); }
    model_transforms_f64(X, s, c);
    model_inertias_f64(I);
}

/* ---------------------------------------------- persistent worker pool ---- */
/* Shaped like the reference's ReusableThreads (utils/ReusableThreads.h:26-115):
 * persistent workers each take one task (a contiguous chunk of knots, as
 * time_CPU.cpp:30-36 splits them) per round, and the caller waits for all. */

typedef struct {
    pthread_t th;
    int tid;
} worker_t;

static struct {
    pthread_mutex_t mu;
    pthread_cond_t go, done;
    int nthreads, generation, pending, shutdown;
    int n, given; /* given: q̈ and Minv are inputs (the reference's time_CPU mode) */
    const float *q, *qd, *u;
    float *dqdd, *qdd, *minv;
    worker_t *w;
} g_pool = {.mu = PTHREAD_MUTEX_INITIALIZER, .go = PTHREAD_COND_INITIALIZER, .done = PTHREAD_COND_INITIALIZER};

static void *worker_main(void *arg) {
    worker_t *w = (worker_t *)arg;
    int seen = 0;
    for (;;) {
        pthread_mutex_lock(&g_pool.mu);
        while (!g_pool.shutdown && g_pool.generation == seen) pthread_cond_wait(&g_pool.go, &g_pool.mu);
        if (g_pool.shutdown) { pthread_mutex_unlock(&g_pool.mu); break; }
        seen = g_pool.generation;
        const int n = g_pool.n, T = g_pool.nthreads, given = g_pool.given;
        pthread_mutex_unlock(&g_pool.mu);
        const int per = n / T, k0 = per * w->tid, k1 = (w->tid == T - 1) ? n : per * (w->tid + 1);
        if (k1 > k0 && given) {
            for (int k = k0; k < k1; k++)
                knot_gradient_given_f32(g_pool.q + KN * k, g_pool.qd + KN * k, g_pool.qdd + KN * k,
                                        g_pool.minv + KM * k, 0, 0, g_pool.dqdd + KD * k);
        } else if (k1 > k0) {
            frg_oracle_gradient_f32(k1 - k0, g_pool.q + KN * k0, g_pool.qd + KN * k0, g_pool.u + KN * k0, NULL, 0, 0,
                                    g_pool.dqdd + KD * k0, g_pool.qdd + KN * k0, g_pool.minv + KM * k0);
        }
        pthread_mutex_lock(&g_pool.mu);
        if (--g_pool.pending == 0) pthread_cond_signal(&g_pool.done);
        pthread_mutex_unlock(&g_pool.mu);
    }
    return NULL;
}

static void pool_stop(void) {
    if (!g_pool.w) return;
    pthread_mutex_lock(&g_pool.mu);
    g_pool.shutdown = 1;
    pthread_cond_broadcast(&g_pool.go);
    pthread_mutex_unlock(&g_pool.mu);
    for (int t = 0; t < g_pool.nthreads; t++) pthread_join(g_pool.w[t].th, NULL);
    free(g_pool.w);
    g_pool.w = NULL;
    g_pool.shutdown = 0;
    g_pool.nthreads = 0;
}

static int pool_start(int threads) {
    if (g_pool.w && g_pool.nthreads == threads) return 0;
    pool_stop();
    g_pool.w = (worker_t *)calloc((size_t)threads, sizeof(worker_t));
    if (!g_pool.w) return 1;
    g_pool.nthreads = threads;
    for (int t = 0; t < threads; t++) {
        g_pool.w[t].tid = t;
        if (pthread_create(&g_pool.w[t].th, NULL, worker_main, &g_pool.w[t])) return 1;
    }
    return 0;
}

/* Runs `iters` rounds over n knots on `threads` persistent workers, FP32,
 * DAMPING off / gravity on (the reference's experiment defaults,
 * utils/experiment_helpers.h:19-20).  given == 0: the full path (q̈ and Minv
 * computed and written); given != 0: the reference's time_CPU mode, q̈ and
 * Minv read from qdd / minv (QDD_MINV_PASSED_IN=true, time_CPU.cpp:30-54).
 * Returns the wall seconds of all rounds, or a negative value on error.  Not
 * thread-safe. */
double frg_oracle_time_threaded_mode_f32(int n, const float *q, const float *qd, const float *u, float *dqdd,
                                         float *qdd, float *minv, int threads, int iters, int given) {
    if (threads < 1 || n < 0 || iters < 0 || pool_start(threads)) return -1.0;
    g_pool.given = given != 0;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int it = 0; it < iters; it++) {
        pthread_mutex_lock(&g_pool.mu);
        g_pool.n = n; g_pool.q = q; g_pool.qd = qd; g_pool.u = u;
        g_pool.dqdd = dqdd; g_pool.qdd = qdd; g_pool.minv = minv;
        g_pool.pending = threads;
        g_pool.generation++;
        pthread_cond_broadcast(&g_pool.go);
        while (g_pool.pending > 0) pthread_cond_wait(&g_pool.done, &g_pool.mu);
        pthread_mutex_unlock(&g_pool.mu);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    g_pool.given = 0;
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

double frg_oracle_time_threaded_f32(int n, const float *q, const float *qd, const float *u, float *dqdd,
                                    float *qdd, float *minv, int threads, int iters) {
    return frg_oracle_time_threaded_mode_f32(n, q, qd, u, dqdd, qdd, minv, threads, iters, 0);
}

/* The time_CPU-mode gradient alone, single-threaded (for the parity tests). */
int frg_oracle_gradient_given_f32(int n, const float *q, const float *qd, const float *qdd, const float *minv,
                                  float *dqdd) {
    if (n < 0) return 1;
    for (int k = 0; k < n; k++)
        knot_gradient_given_f32(&q[KN * k], &qd[KN * k], &qdd[KN * k], &minv[KM * k], 0, 0, &dqdd[KD * k]);
    return 0;
}

void frg_oracle_pool_shutdown(void) { pool_stop(); }
