/*
 * frg.h - C ABI of the GB300 (sm_103a) iiwa_14 forward-dynamics-gradient engine.
 *
 * Per knot point (q, qd, u) the engine runs the RNEA forward/backward sweeps,
 * the articulated-body Minv recursion, q̈ = Minv (u - c), the dtau/dq and
 * dtau/dqd recursions and the finish [dq̈/dq | dq̈/dq̇] = -Minv [dtau/dq | dtau/dqd],
 * in FP32 on the CUDA cores.
 *
 * Replaces the host sequence of the reference's time_GPU.cu:137-158,313-316
 * (pack [q|qd|u|qdd|Minv] per knot, cudaMemcpy H2D,
 *  dynamicsGradientKernel<T,N,MPC_MODE,VEL_DAMPING><<<N,(32,7)>>>(d_dqdd,
 *  d_mem_vol, d_mem_const) from helpers_GPU/dynamicsGradient.cuh:1257-1290,
 *  cudaMemcpy D2H) with one call whose inputs are only q, qd, u: q̈ and Minv
 * are produced on the device instead of being computed on the host by
 * forwardDynamics (helpers_CPU/dynamicsGradient.h:686-706, :936-939).
 *
 * Layouts (all float32, knot-major, every matrix column-major as in the
 * reference, helpers_CPU/dynamicsGradient.h:34-41), for a robot of N joints
 * (N = 7 for the iiwa_14; frg_model_dofs() reports the build's N, as the
 * reference's NUM_POS macro fixes it, dynamicsGradient.h:7-12):
 *   q, qd, u  [n][N]
 *   dqdd      [n][2N^2] = N x 2N, column c < N: dq̈/dq_c, column N + c: dq̈/dq̇_c
 *                        (the reference's 2*NUM_POS*NUM_POS block per knot,
 *                        time_CPU.cpp:34, dynamicsGradient.h:921; 98 floats)
 *   qdd       [n][N]
 *   minv      [n][N^2]  dense symmetric (the reference's DENSE_MINV form,
 *                        time_GPU.cu:134; 49 floats)
 * Sizes below quoted as numbers are the iiwa's (N = 7).
 *
 * Conventions: every call returns an frg_status (nothing aborts or exits;
 * the reference's gpuErrchk aborted the process, dynamicsGradient.cuh:28-35);
 * frg_last_error() describes the last failure of a context.  A context is used
 * by one host thread at a time.  Buffers passed in belong to the caller.
 */
#ifndef FRG_H
#define FRG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-knot sizes of the default build (the 7-joint iiwa_14).  A library built
 * for another robot reports its joint count N through frg_model_dofs(); its
 * sizes are those of the layouts above with that N. */
#define FRG_NUM_JOINTS 7
#define FRG_DQDD_FLOATS 98
#define FRG_MINV_FLOATS 49

typedef enum frg_status {
    FRG_OK = 0,
    FRG_ERR_INVALID_ARGUMENT = 1,
    FRG_ERR_CUDA = 2,
    FRG_ERR_OUT_OF_MEMORY = 3,
    FRG_ERR_NOT_READY = 4,  /* a server request is still in flight */
    FRG_ERR_ADMISSION = 5,  /* a server request can never fit the device pool */
    FRG_ERR_TIMEOUT = 6,
    FRG_ERR_SHUTDOWN = 7,
    FRG_ERR_NOT_FOUND = 8,
    FRG_ERR_INTERNAL = 9,
    FRG_ERR_CANCELLED = 10 /* a served call withdrawn by frg_server_cancel */
} frg_status;

/* Same type as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st *frg_stream;

typedef struct frg_ctx frg_ctx;
typedef struct frg_plan frg_plan;

/* Replaces the reference's compile-time switches (utils/experiment_helpers.h:
 * 17-21; template bools MPC_MODE, VEL_DAMPING of dynamicsGradient.h:685,868). */
typedef struct frg_options {
    int device;        /* CUDA device ordinal (default 0) */
    int vel_damping;   /* VEL_DAMPING: adds 0.5 qd to the bias and 0.5 to the
                          dtau/dqd diagonal (default 0, experiment_helpers.h:20) */
    int mpc_mode;      /* MPC_MODE: gravity-compensated arm, base acceleration 0
                          (default 0, dynamicsGradient.h:635-637) */
    int warps_per_cta; /* 0 = engine default (2) */
    int ctas_per_sm;   /* 0 = engine default (4; persistent batched launches) */
    int lanes_per_knot; /* 0 = default (1); 1 = one knot per lane, 32 knots per
                           warp (throughput); 8 = one knot per 8 lanes, 4 knots
                           per warp (latency: small batches finish ~2.5x sooner) */
} frg_options;

void frg_options_default(frg_options *opt);
const char *frg_status_string(frg_status s);
/* The robot this library was built for: "iiwa_14" (the default, the
 * reference's model, code-generated there at helpers_CPU/dynamicsGradient.h:
 * 124-229) or the name in the tables header frg/urdf.py wrote from another
 * URDF of a serial arm of 1 to 8 revolute joints. */
const char *frg_model_name(void);
/* Its joint count N (7 for the iiwa_14): the reference's NUM_POS
 * (helpers_CPU/dynamicsGradient.h:7-12), which sizes every per-knot array. */
int frg_model_dofs(void);

/* Creates a context on opt->device (NULL opt = defaults). */
frg_status frg_create(frg_ctx **out, const frg_options *opt);
void frg_destroy(frg_ctx *ctx);
/* Message of the last failed call on ctx ("" if none).  ctx may be NULL. */
const char *frg_last_error(const frg_ctx *ctx);

/* Launch shape of ctx's launches (sets both the plain and the persistent
 * shape; the autotuner tunes them separately and get returns the plain one). */
frg_status frg_set_launch_shape(frg_ctx *ctx, int warps_per_cta, int ctas_per_sm);
frg_status frg_get_launch_shape(const frg_ctx *ctx, int *warps_per_cta, int *ctas_per_sm);
/* Threads per knot of every launch of ctx: 1 or 8 (the autotuner sets it too). */
frg_status frg_set_lanes_per_knot(frg_ctx *ctx, int lanes_per_knot);
int frg_get_lanes_per_knot(const frg_ctx *ctx);

/*
 * Plain path: one launch over n_knots knots of DEVICE arrays, asynchronous on
 * `stream`.  The drop-in for dynamicsGradientKernel<<<N,(32,7)>>>
 * (helpers_GPU/dynamicsGradient.cuh:1259) with q̈ and Minv produced, not
 * consumed.  n_knots == 0 is a no-op.
 */
frg_status frg_gradient(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u, float *dqdd,
                        float *qdd, float *minv, frg_stream stream);

/*
 * Single-knot latency, the counterpart of the reference's kern_single_full
 * (time_GPU.cu:23-51, timed at :191-195), which repeats one knot TEST_ITERS
 * times inside one CTA so that the time per knot excludes the launch.  Here
 * one warp carries ONE knot (q, qd, u [7], DEVICE) through the whole path
 * `iters` times in a row in one launch -- each repetition exactly as a
 * one-knot frg_gradient does it, results stored to dqdd [98], qdd [7],
 * minv [49] -- in the thread mapping lanes_per_knot (1: one lane; 8: eight
 * lanes share the knot's columns, the mapping small batches use).
 * Asynchronous on `stream`; with us_per_knot != NULL it waits for the launch
 * and writes its CUDA-event time divided by iters (launch included, so use a
 * large iters, or the difference of two iters, to take the launch out).
 */
frg_status frg_single_knot_latency(frg_ctx *ctx, int lanes_per_knot, int iters, const float *q, const float *qd,
                                   const float *u, float *dqdd, float *qdd, float *minv, frg_stream stream,
                                   double *us_per_knot);

/*
 * Same, for HOST arrays, synchronous: returns when the results are in the host
 * arrays (the time_GPU.cu:313-316 "Compute + I/O" sequence).  Pinned arrays
 * (frg_host_alloc, cudaHostAlloc / cudaHostRegister) take a single launch
 * with no copies: the kernel reads the inputs across the host link itself and
 * writes each 32-knot tile's results to the host arrays as soon as the tile
 * finishes, so the transfer overlaps the arithmetic.  Pageable arrays are
 * staged through device buffers owned by ctx.
 *
 * qdd and/or minv may be NULL: that result is then not returned, and none of
 * its bytes cross the host link (the kernel writes it to device memory owned by
 * ctx).  dqdd alone is what the reference's "Completely Fused" call returns
 * (time_GPU.cu:316 copies back d_dqdd only): 392 of the 616 result bytes per
 * knot at 7 joints.
 */
frg_status frg_gradient_host(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                             float *dqdd, float *qdd, float *minv);

/*
 * Many host-buffer batches in one call (a caller streaming batch after batch
 * through host memory): each batch as frg_gradient_host, returning when every
 * result is in its host arrays.  With pinned arrays the batches alternate
 * between two internal streams, two launches in flight at once, so a batch's
 * launch and first tiles -- about 25 us in which no result exists yet -- overlap
 * the previous batch's results streaming over the host link, which then stays
 * busy.  When every batch asks for Minv (and the context runs one lane per
 * knot), Minv crosses the link as its upper triangle -- 112 instead of 196 B
 * per knot at 7 joints -- into pinned staging owned by ctx, and host threads
 * expand each batch into its dense minv array while later batches compute:
 * the same bits, 14 % fewer bytes on the link that bounds the call.  Batches
 * must not share output arrays with other batches of the call that may be in
 * flight (neighbouring ones).  A batch's qdd and minv may be NULL, as in
 * frg_gradient_host.  Pageable arrays are processed one batch after the
 * other.  No counterpart in the reference, whose time_GPU.cu:310-330 loop
 * synchronises after every batch.
 */
typedef struct frg_host_batch {
    int n_knots;
    const float *q, *qd, *u;
    float *dqdd, *qdd, *minv;
} frg_host_batch;
frg_status frg_gradient_host_batches(frg_ctx *ctx, int n_batches, const frg_host_batch *batches);

/*
 * The reference's own per-knot layout, for callers that already pack it: the
 * knot<T> record of helpers_CPU/dynamicsGradient.h:19-25, [q N | qd N | u N |
 * qdd N | Minv N^2] = FRG_KNOT_RECORD_FLOATS (4N + N^2) floats per knot, as time_GPU.cu:
 * 137-158 packs it for dynamicsGradientKernel.  knots [n] (DEVICE) supply q,
 * qd, u; q̈ and dense Minv are written into each record's qdd and Minv fields
 * (the reference fills them on the host first, forwardDynamics at
 * time_GPU.cu:134); the gradient goes to dqdd [n][98].  Asynchronous on
 * `stream`; the same arithmetic and bits as frg_gradient, one knot per lane
 * whatever the lanes-per-knot setting.
 */
#define FRG_KNOT_RECORD_FLOATS 77
frg_status frg_gradient_knots(frg_ctx *ctx, int n_knots, float *knots, float *dqdd, frg_stream stream);

/*
 * Either side of the gradient (plain path, DEVICE arrays, asynchronous):
 *  - frg_gradient_fext: the gradient with external spatial forces on the links,
 *    fext [n][7][6] (link k's force in its own frame, [n, f] order), subtracted
 *    from each link force in both RNEA passes as the reference's s_fext
 *    (helpers_CPU/dynamicsGradient.h:654-657); fext == NULL is frg_gradient.
 *  - frg_forward_dynamics: q̈ [n][7] and, if minv != NULL, Minv [n][49] only
 *    (forwardDynamics, dynamicsGradient.h:686-706); fext may be NULL.
 *  - frg_discrete_jacobians: for the explicit-Euler step x+ = x + dt [qd; q̈]
 *    of the state x = [q; qd], A = I + dt [0 I; dq̈/dq dq̈/dqd] [n][14x14] and
 *    B = dt [0; Minv] [n][14x7], column-major, from dqdd and minv (the solver
 *    step that consumes the gradient; MPC/iLQR callers).
 */
frg_status frg_gradient_fext(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                             const float *fext, float *dqdd, float *qdd, float *minv, frg_stream stream);
frg_status frg_forward_dynamics(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                                const float *fext, float *qdd, float *minv, frg_stream stream);
frg_status frg_discrete_jacobians(frg_ctx *ctx, int n_knots, const float *dqdd, const float *minv, float dt,
                                  float *A, float *B, frg_stream stream);

/*
 * FP64 verification build (DEVICE arrays, asynchronous on `stream`).  The
 * reference's GPU path is FP32 only and has no counterpart; its FP64 results
 * come from the CPU recursions (helpers_CPU/dynamicsGradient.h:916-934 with
 * T = double), which these calls restate on the device from the same kernel
 * source compiled in double.
 *  - frg_gradient_f64: frg_gradient with double arrays of the same layouts.
 *  - frg_verify_f64: recomputes n_knots knots in FP64 from the FP32 inputs q,
 *    qd, u and writes, per knot, the Frobenius-relative errors
 *    ||x - x64||_F / ||x64||_F of the FP32 results dqdd, qdd, minv to
 *    err [n][3] (doubles, device).  Its scratch (175 doubles per knot) is a
 *    ctx-owned device buffer that grows on demand: a call that grows it
 *    allocates and synchronises the device, so size it once with the largest
 *    batch before timed or captured work.  Calls sharing a ctx must not
 *    overlap on different streams.
 */
frg_status frg_gradient_f64(frg_ctx *ctx, int n_knots, const double *q, const double *qd, const double *u,
                            double *dqdd, double *qdd, double *minv, frg_stream stream);
frg_status frg_verify_f64(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                          const float *dqdd, const float *qdd, const float *minv, double *err, frg_stream stream);

/* One trajectory (a contiguous run of knots) of a batched call; all DEVICE
 * pointers with the layouts above. */
typedef struct frg_traj {
    int64_t n_knots;
    const float *q, *qd, *u;
    float *dqdd, *qdd, *minv;
} frg_traj;

/*
 * Plain form over many trajectories: one launch per trajectory, in order, on
 * `stream` (what a caller of the reference does for a batch of trajectories:
 * one dynamicsGradientKernel launch each).
 */
frg_status frg_gradient_per_trajectory(frg_ctx *ctx, int n_traj, const frg_traj *trajs, frg_stream stream);

/*
 * Batched form: ONE launch over all trajectories' knots, asynchronous on
 * `stream`.  Trajectories scattered in memory run on a persistent kernel that
 * walks the 32-knot tiles of the ragged list; trajectories that lie back to
 * back in memory (e.g. offsets into concatenated arrays) are one contiguous
 * run of knots and take the plain kernel, without per-tile lookups.
 * Builds the launch's descriptor list on every call; for a batch that is run
 * repeatedly, build an frg_plan once instead.
 */
frg_status frg_gradient_batched(frg_ctx *ctx, int n_traj, const frg_traj *trajs, frg_stream stream);

/* Convenience: trajectories as [offsets[t], offsets[t+1]) of contiguous
 * device arrays (offsets: HOST array of n_traj + 1 non-decreasing entries). */
frg_status frg_gradient_ragged(frg_ctx *ctx, int n_traj, const int64_t *offsets, const float *q, const float *qd,
                               const float *u, float *dqdd, float *qdd, float *minv, frg_stream stream);

/*
 * Allocation-free batched call.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc/cudaFree once running -- a real-time
 * MPC loop (cudaFree synchronizes the device, cudaMalloc can block for an
 * unbounded time) or a plug-in whose host application owns all device memory.
 * Same arguments, layouts and results as frg_gradient_ragged, but the launch's
 * descriptor lists and work counter live in one fixed 512 KiB device array
 * that every GPU loading the library holds until process exit, so at most
 * FRG_NOALLOC_MAX_TRAJ trajectories and FRG_NOALLOC_MAX_KNOTS knots per call
 * (larger batches return FRG_ERR_INVALID_ARGUMENT).  The first call on a
 * device looks up that array's device address on that device.  All calls
 * share the array: calls whose launches may overlap on the GPU (different
 * streams, unordered) race -- order them.
 */
#define FRG_NOALLOC_MAX_TRAJ 4096
#define FRG_NOALLOC_MAX_KNOTS (65536 * 32)
frg_status frg_gradient_ragged_noalloc(frg_ctx *ctx, int n_traj, const int64_t *offsets, const float *q,
                                       const float *qd, const float *u, float *dqdd, float *qdd, float *minv,
                                       frg_stream stream);

/*
 * Plans: a batched launch prepared once (descriptor list on the device, the
 * context's launch shape at creation) and repeated by frg_plan_launch, one
 * persistent launch each.  The trajectory pointers are baked in; the data
 * behind them may change between launches.  Launches of one plan must not
 * overlap on the device.  Every launch of the engine's gradient kernels uses
 * programmatic dependent launch: it may be scheduled while the previous work
 * on its stream finishes, and waits for that work to complete before reading
 * its inputs or writing anything (before the wait it reads only its own launch
 * descriptors and asks L2 to fetch its first inputs, a hint), so stream order
 * holds and back-to-back launches (solver iterations, plan repeats) lose no
 * time between them.  Plan launches can be captured into a caller's CUDA graph
 * like any kernel launch.
 */
frg_status frg_plan_create(frg_ctx *ctx, int n_traj, const frg_traj *trajs, frg_plan **out);
frg_status frg_plan_create_ragged(frg_ctx *ctx, int n_traj, const int64_t *offsets, const float *q,
                                  const float *qd, const float *u, float *dqdd, float *qdd, float *minv,
                                  frg_plan **out);
frg_status frg_plan_launch(frg_plan *plan, frg_stream stream);
/*
 * Independent plans, several in flight: plans[i] is launched on stream
 * i mod in_flight, where stream 0 is `stream` and streams 1 to in_flight - 1
 * belong to the context (in_flight 1 to 4), so the launches run side by side.
 * A persistent launch's last wave of tiles leaves part of the GPU idle;
 * launches on the other streams fill it.  On the 512-trajectory mix this takes
 * a launch from 41 us to 33-34 us (two or three in flight).  Stream order is
 * kept against everything else: the launches wait for the work queued on
 * `stream` before the call, and work queued on `stream` after it waits for all
 * n launches.  Launches on different streams may run at the same time in any
 * combination, so the caller guarantees that plans at positions of different
 * residues mod in_flight are independent: none writes memory that another
 * reads or writes.  A plan may appear more than once, but only at positions
 * of one residue (else FRG_ERR_INVALID_ARGUMENT): launches of one plan on two
 * streams would share its work counter.  All plans belong to ctx.  There is
 * no counterpart in the reference, whose launches are synchronous
 * (time_GPU.cu:313-316).
 */
frg_status frg_plan_launch_many(frg_ctx *ctx, int n_plans, frg_plan *const *plans, int in_flight,
                                frg_stream stream);
int64_t frg_plan_knots(const frg_plan *plan);
void frg_plan_destroy(frg_plan *plan);

/*
 * Autotuner: on n_knots synthetic knots, times with CUDA events every shape of
 * the plain kernel (threads per knot x warps per CTA; contiguous batches) and
 * of the persistent kernel (x resident CTAs per SM; trajectories scattered in
 * memory) and keeps the fastest of each in ctx.
 * Writes the best throughput (knots/s) if best_knots_per_s is not NULL.
 */
frg_status frg_autotune(frg_ctx *ctx, int64_t n_knots, double *best_knots_per_s);

/*
 * The tuned launch shapes of ctx as plain values, so that a caller can keep
 * the autotuner's choice (in a file, keyed by GPU model) and restore it at
 * start-up instead of re-tuning.  set validates every field; a shape the GPU
 * cannot launch fails with FRG_ERR_INVALID_ARGUMENT and changes nothing.
 */
typedef struct frg_tuning {
    int warps_per_cta, lanes_per_knot;                             /* plain launches (contiguous knots) */
    int ragged_warps_per_cta, ragged_ctas_per_sm, ragged_lanes_per_knot; /* persistent launches */
} frg_tuning;
frg_status frg_get_tuning(const frg_ctx *ctx, frg_tuning *out);
frg_status frg_set_tuning(frg_ctx *ctx, const frg_tuning *tuning);

/*
 * Per-knot status (DEVICE arrays, asynchronous): status[k] gets
 * FRG_KNOT_NONFINITE_INPUT if any of knot k's q, qd, u is NaN or infinite, and
 * FRG_KNOT_NONFINITE_OUTPUT if any of its dqdd, qdd, minv is (outputs may be
 * NULL: not checked), else 0.  The reference has no such check; its kernel
 * propagates non-finite values silently.  A non-finite input never spreads to
 * other knots here (one knot per lane), so the flags locate the bad knots.
 * One coalesced pass over the arrays, separate from the gradient launch.
 */
#define FRG_KNOT_NONFINITE_INPUT 1u
#define FRG_KNOT_NONFINITE_OUTPUT 2u
frg_status frg_knot_status(frg_ctx *ctx, int n_knots, const float *q, const float *qd, const float *u,
                           const float *dqdd, const float *qdd, const float *minv, uint32_t *status,
                           frg_stream stream);

/*
 * Continuous-batching server (MPC / iLQR callers).  No counterpart in the
 * reference, whose drivers time one synchronous batch at a time
 * (time_GPU.cu:310-330); it serves the gradient calls of many trajectories as
 * they arrive:
 *  - a trajectory (traj_id) keeps a slot of 700 B per knot -- its q, qd, u
 *    and its results -- in a capped device pool, mirrored in pinned host
 *    memory, from its first call until frg_server_release; a call's inputs
 *    may come from the host (frg_server_submit), from the caller's device
 *    arrays (frg_server_submit_device) or from the slot itself
 *    (frg_server_submit_resident), and its results may stay on the device;
 *  - admission is by free pool bytes: a new trajectory that does not fit
 *    waits (an admission stall) until releases make room;
 *  - a dispatcher thread folds all ready calls into the next persistent
 *    launch (up to max_batch_knots) while up to max_inflight earlier launches
 *    still run, each on its own stream;
 *  - results of a call are bit-identical alone or batched with any others:
 *    every knot's arithmetic is the same in both thread mappings, whichever
 *    the batch size selects.
 * One call per trajectory may be in flight; submit copies the inputs.
 */
typedef struct frg_server frg_server;

typedef struct frg_server_options {
    size_t pool_bytes;    /* device pool cap (and pinned host mirror), default 1 GiB */
    int max_batch_knots;  /* knots folded into one launch at most, default 65536 */
    int max_inflight;     /* launches in flight at once (streams), default 3, <= 16 */
    int warps_per_cta;    /* launch shape of larger server launches, 0 = the context's */
    int ctas_per_sm;
    int latency_mapping_max_knots; /* batches up to this many knots use the
                                      8-lanes-per-knot mapping (default 4096;
                                      0: one lane per knot for every batch) */
} frg_server_options;

typedef struct frg_request_info {
    uint64_t request_id, traj_id;
    int64_t horizon;
    frg_status status;
    /* results in pinned host memory, valid until this trajectory's next
     * submit or its release; NULL unless status == FRG_OK and the call wrote
     * results to the host (frg_server_submit, or FRG_SERVE_HOST_RESULTS) */
    const float *dqdd, *qdd, *minv;
    /* the trajectory's resident device copy (inputs and results) */
    const float *dev_q, *dev_qd, *dev_u, *dev_dqdd, *dev_qdd, *dev_minv;
    double latency_us;  /* submit -> results visible in host memory */
    double queue_us;    /* submit -> launch */
    uint64_t batch_id;
    int batch_requests; /* calls folded into the same launch */
} frg_request_info;

typedef struct frg_server_stats {
    uint64_t submitted, completed, launches, knots;
    uint64_t admission_stalls; /* calls that waited for pool space */
    uint64_t rejected;         /* calls that can never fit */
    size_t pool_bytes_cap, pool_bytes_used, pool_bytes_peak;
    size_t queued_admission, queued_ready;
    uint64_t cancelled;        /* calls withdrawn by frg_server_cancel */
} frg_server_stats;

void frg_server_options_default(frg_server_options *opt);
frg_status frg_server_create(frg_ctx *ctx, const frg_server_options *opt, frg_server **out);
/* Finishes queued and in-flight calls (calls still waiting for admission end
 * with FRG_ERR_SHUTDOWN), then frees everything. */
void frg_server_destroy(frg_server *srv);
/* Queues one gradient call of trajectory traj_id over `horizon` knots (host
 * arrays [horizon][7], copied before return).  FRG_ERR_NOT_READY if the
 * trajectory already has a call in flight, FRG_ERR_ADMISSION if its slot can
 * never fit the pool. */
frg_status frg_server_submit(frg_server *srv, uint64_t traj_id, int64_t horizon, const float *q, const float *qd,
                             const float *u, uint64_t *request_id);
/*
 * Device-resident calls.  The reference copies every call's inputs and
 * results across the host link (time_GPU.cu:313-316); these keep a
 * trajectory's state on the GPU across its solver iterations.
 *  - frg_server_submit_device: the call's inputs are already on the GPU (a
 *    solver that computes its next iterate there): q, qd, u [horizon][7] are
 *    the caller's DEVICE arrays, read by the kernel directly and copied into
 *    the trajectory's device slot.  They must stay valid and unchanged until
 *    the call completes.
 *  - frg_server_submit_resident: a call on the inputs resident in the
 *    trajectory's device slot -- those of its previous completed call, or what
 *    the caller wrote there in place through frg_server_slot between calls
 *    (finished before this submit, e.g. by synchronizing the stream that wrote
 *    them).  FRG_ERR_NOT_FOUND if the trajectory has no completed call.
 * Both write results to the device slot (frg_request_info dev_dqdd, dev_qdd,
 * dev_minv) and, with FRG_SERVE_HOST_RESULTS in flags, to the pinned host
 * slot as frg_server_submit does.  Admission, batching, errors, cancellation
 * and determinism are those of frg_server_submit.
 */
#define FRG_SERVE_HOST_RESULTS 1u
frg_status frg_server_submit_device(frg_server *srv, uint64_t traj_id, int64_t horizon, const float *q,
                                    const float *qd, const float *u, unsigned int flags, uint64_t *request_id);
frg_status frg_server_submit_resident(frg_server *srv, uint64_t traj_id, unsigned int flags,
                                      uint64_t *request_id);
/* The trajectory's device slot: q, qd, u (writable between calls, not while
 * one is in flight: FRG_ERR_NOT_READY) and the last call's results.
 * FRG_ERR_NOT_FOUND if the trajectory has no completed call. */
typedef struct frg_slot_info {
    int64_t horizon;
    float *q, *qd, *u;
    const float *dqdd, *qdd, *minv;
} frg_slot_info;
frg_status frg_server_slot(frg_server *srv, uint64_t traj_id, frg_slot_info *out);
/* FRG_OK (done, info filled, request retired), FRG_ERR_NOT_READY, FRG_ERR_NOT_FOUND. */
frg_status frg_server_poll(frg_server *srv, uint64_t request_id, frg_request_info *info);
/* Blocks until the call is done (timeout_us < 0: no limit); FRG_ERR_TIMEOUT otherwise. */
frg_status frg_server_wait(frg_server *srv, uint64_t request_id, int64_t timeout_us, frg_request_info *info);
/* Next completed call not yet taken by poll/wait, in completion order. */
frg_status frg_server_wait_any(frg_server *srv, int64_t timeout_us, frg_request_info *info);
/* Frees the trajectory's slots (FRG_ERR_NOT_READY while a call is in flight). */
frg_status frg_server_release(frg_server *srv, uint64_t traj_id);
/* Withdraws a call that has not reached the GPU (still waiting for admission
 * or for the next launch): it completes at once with status
 * FRG_ERR_CANCELLED and no results (wait / poll / wait_any return it like any
 * completed call), and its trajectory may be submitted again.
 * FRG_ERR_NOT_READY if the call is already on the GPU or done,
 * FRG_ERR_NOT_FOUND if it is unknown or already taken.  No counterpart in the
 * reference, which has no request queue. */
frg_status frg_server_cancel(frg_server *srv, uint64_t request_id);
frg_status frg_server_get_stats(frg_server *srv, frg_server_stats *out);

/* Pinned host memory for the _host calls and the server (NULL on failure). */
void *frg_host_alloc(size_t bytes);
void frg_host_free(void *p);

#ifdef __cplusplus
}
#endif

#endif /* FRG_H */
