"""Benchmark: iiwa_14 forward-dynamics gradients on GB300.

Workload (one "step"): the ragged 512-trajectory mix -- horizons ~ U{8..256}
(seed 2021, 66,809 knots), knots q ~ U(URDF joint limits), qd ~ U(-2, 2),
u ~ U(-20, 20) (seeded synthetic data; the reference ships no dataset) --
through the full path (RNEA, Minv, q̈, dtau/dq, dtau/dqd, -Minv dtau) in FP32.

  value     knot-gradients/s of the batched form: one persistent launch over
            the ragged offset list (a plan launch per step), inputs resident
            in HBM; 6 rotating input/output sets (~280 MB > 129 MB L2).  The
            K steps are independent batches issued by one
            frg_plan_launch_many call with three in flight (step i on stream
            i mod 3), so each launch's partial last wave overlaps the next
            batches.
            single_stream: the same K launches one after another on one
            stream.
  e2e       the same metric through the C ABI's host-buffer calls: H2D of
            q, qd, u from pinned memory, kernel, D2H of dqdd, qdd, Minv
            inside every timed step (frg_gradient_host_batches, two steps in
            flight, Minv over the link as its upper triangle and expanded to
            dense by host threads inside the call; e2e.single_call: one
            synchronous frg_gradient_host per step, dense Minv over the link;
            e2e.gradient_only: dqdd alone returned, as the reference's
            Completely Fused call returns it).
  plain     the plain form of the same mix: one launch per trajectory.
  plain_scaling  one plain launch per batch of N contiguous knots, N in
            {16, 32, 64, 128, 1024, 65536} (L2 warm), plus N = 1 (single-knot
            latency) and N = 65536 over batches larger than L2; the faster
            thread mapping kept.
  entry_points  the calls either side of the gradient (external forces,
            forward dynamics, knot records, discrete Jacobians, the FP64
            build) on 65,536 knots, L2 flushed: time per launch.
  served    p50/p99 request latency of the continuous-batching server, and
            the 2 GiB-pool admission run with 1 % of its calls verified by
            the FP64 GPU build.
  parity    max per-knot Frobenius-relative error of dqdd, qdd, Minv over
            every knot the timed launches produced, against the FP64 GPU
            build (frg_verify_f64).
  roofline  dominant kernel (the batched kernel): algorithmic bytes
            (84 B in + 616 B out per knot) / CUDA-event launch time vs the
            measured HBM copy peak; FP32 work at the reference's 35,257
            FLOP/knot vs the FP32 CUDA-core peak.

--impl reference times the reference algorithm's CPU path (the oracle's C
restatement, threaded like time_CPU.cpp) on this host's cores on the same
workload.  Under torchrun each rank runs its own mix (weak scaling); there is
no collective on the data path.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "fast-rbd-gradients_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "knot-pt gradients/s + p99 request latency, batched/served vs plain, same GB300"
UNIT = "knot-gradients/s"
N_TRAJ, H_LO, H_HI, MIX_SEED = 512, 8, 256, 2021
BYTES_PER_KNOT = 84 + 616          # algorithmic HBM bytes: q, qd, u in; dqdd, qdd, Minv out
D2H_PACKED = 392 + 28 + 112        # bytes per knot over the host link when Minv travels as its upper triangle
FLOP_PER_KNOT_REF = 35257          # the reference's full path as written (op-counted)
ROTATING_SETS = 6
IN_FLIGHT = 3                      # independent batches in flight in the timed steps (divides ROTATING_SETS)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["frg", "reference"], default="frg")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving latency measurement")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n-traj", type=int, default=N_TRAJ, help="trajectories in the ragged mix")
    ap.add_argument("--plain-n", type=int, default=0,
                    help="with --profile: time plain launches of this many contiguous knots instead of the mix")
    ap.add_argument("--plain-lanes", type=int, default=1, choices=(1, 8),
                    help="with --plain-n: threads per knot of those launches")
    ap.add_argument("--profile", action="store_true",
                    help="batched launches only (no autotune, plain form, e2e, serving or CPU baseline): "
                         "the command the ncu summaries in profiles/ capture")
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(rank, n_traj=N_TRAJ):
    from frg import dist as fdist
    return fdist.rank_mix(rank, n_traj, H_LO, H_HI, MIX_SEED)


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return pk, "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


# Figures of one ncu capture of grad_ragged_kernel on this exact workload (the
# 512-trajectory mix, 66,809 knots, --profile shape), per launch; the command
# and its full output summary are in profiles/grad_ragged_kernel_bench_mix.md.
#  - DRAM bytes read + written while the kernel runs: the mix's 41 MB of
#    results stay dirty in the 129 MB L2 when it ends (written back later, by
#    the next launches' evictions), so writes are almost absent here;
#  - FP32 operations executed (2 x FFMA + FADD + FMUL, thread level), which
#    count what the kernel does after dropping the reference's structural zeros.
NCU_MIX = {"dram_read_bytes": 6.019e6, "dram_write_bytes": 0.260e6,
           "l2_write_bytes_all_sources": 77.3e6,
           "executed_flop_per_knot": 13440.0,
           "knots": 66809}
# FP32 CUDA-core peak measured on a GB300 of this machine: every thread of
# 2 x 1024-thread CTAs per SM runs 8 independent FMA chains (CUDA events, best
# of 20 launches of 20 ms, SM clock 2070 MHz, no throttle reason): 78.5 TFLOP/s
# with scalar FFMA, 80.4 with packed FFMA2 (fma.rn.f32x2); the larger is the
# denominator.  Method and figures in profiles/fp32_fma_peak.md.
FP32_PEAK_TFLOPS_MEASURED = 80.4


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms in the background."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.rows, self.proc = gpu, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": len(self.rows)}
        if not self.rows:
            return out

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in self.rows if num(r[1])]
        mx = [num(r[2]) for r in self.rows if num(r[2])]
        if sm:
            out["sm_mhz"] = statistics.median(sm)
        if mx:
            out["sm_max_mhz"] = max(mx)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for i, nm in enumerate(names):
            if any(r[5 + i].lower() == "active" for r in self.rows):
                out["reasons"].append(nm)
        return out


PLAIN_SIZES = (16, 32, 64, 128, 1024, 65536)
FLUSH_SETS = 4  # rotating 65,536-knot sets: 4 x 46 MB > 129 MB L2


def plain_scaling(ctx, torch, dev, stream, peaks, fp32_peak, steps=20):
    """Plain path, one launch per batch of N contiguous device-resident knots
    (the scaling config), in both thread mappings; the faster is kept.  Rows:
    N = 1 (single-knot latency), every N of the config with one batch reused
    (L2 warm), and N = 65,536 again over rotating batches larger than L2."""
    import frg
    out = []
    nmax = max(PLAIN_SIZES)
    sets = []
    for i in range(FLUSH_SETS):
        q, qd, u = frg.sample_knots(nmax, seed=99 + i)
        sets.append([torch.from_numpy(x).to(dev) for x in (q, qd, u)] +
                    [torch.empty((nmax, w), device=dev) for w in (98, 7, 49)])
    saved = ctx.tuning()
    rows = [(1, 1)] + [(n, 1) for n in PLAIN_SIZES] + [(nmax, FLUSH_SETS)]
    for n, nsets in rows:
        best = None
        for lanes in (1, 8):
            ctx.set_lanes_per_knot(lanes)
            for i in range(3):
                ctx.gradient(n, *sets[i % nsets], stream=stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for i in range(steps):
                ctx.gradient(n, *sets[i % nsets], stream=stream)
            e1.record(stream)
            stream.synchronize()
            ms = e0.elapsed_time(e1) / steps
            if best is None or ms < best[0]:
                best = (ms, lanes)
        ms, lanes = best
        out.append({"n": n, "us_per_launch": round(ms * 1e3, 2), "knots_per_s": n / (ms * 1e-3),
                    "lanes_per_knot": lanes,
                    "l2": "warm (one batch reused)" if nsets == 1 else
                          f"flushed ({nsets} rotating batches, {nsets * n * BYTES_PER_KNOT / 1e6:.0f} MB)",
                    "hbm_frac": BYTES_PER_KNOT * n / (ms * 1e-3) / 1e9 / float(peaks["hbm_gbs"]),
                    "fp32_frac": FLOP_PER_KNOT_REF * n / (ms * 1e-3) / 1e12 / fp32_peak})
    ctx.set_tuning(saved)
    return out


def fp32_peak_live(device):
    """FP32 CUDA-core peak measured now on `device` by the committed probe
    frg/bin/frg_fp32_peak (FFMA and packed FFMA2 chains; the larger is the
    peak); the recorded FP32_PEAK_TFLOPS_MEASURED if the probe cannot run."""
    exe = os.path.join(ROOT, "fast-rbd-gradients_gb300", "frg", "bin", "frg_fp32_peak")
    try:
        r = subprocess.run([exe, str(device), "10"], capture_output=True, text=True, timeout=120)
        vals = dict(line.split() for line in r.stdout.splitlines() if len(line.split()) == 2)
        ffma, ffma2 = float(vals["FFMA_TFLOPS"]), float(vals["FFMA2_TFLOPS"])
        if r.returncode == 0 and ffma > 0:
            return {"peak": max(ffma, ffma2), "ffma_tflops": ffma, "ffma2_tflops": ffma2,
                    "source": "measured in this run (frg/bin/frg_fp32_peak: FFMA and FFMA2 chains, best of 10)"}
    except (OSError, KeyError, ValueError, subprocess.SubprocessError):
        pass
    return {"peak": FP32_PEAK_TFLOPS_MEASURED, "source": "recorded FP32_PEAK_TFLOPS_MEASURED (probe unavailable)"}


def host_link_rates(torch, dev, stream, nbytes, reps=10):
    """Host link rates (GB/s) of plain copies between pinned host memory and
    device memory, nbytes each, CUDA events on `stream`: the bound of calls
    whose inputs and results live in host memory."""
    n = nbytes // 4
    h = torch.empty(n, dtype=torch.float32, pin_memory=True)
    d = torch.empty(n, dtype=torch.float32, device=dev)
    out = {}
    for name, (dst, src) in (("h2d_gbs", (d, h)), ("d2h_gbs", (h, d))):
        with torch.cuda.stream(stream):
            for _ in range(2):
                dst.copy_(src, non_blocking=True)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                dst.copy_(src, non_blocking=True)
            e1.record(stream)
        stream.synchronize()
        out[name] = nbytes * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9
    return out


def single_knot(ctx, torch, dev, stream, n1=100, n2=1100, reps=5):
    """Single-knot latency (the reference's kern_single_full, time_GPU.cu:23-51):
    one warp repeats the whole path over one knot inside one launch
    (frg_single_knot_latency).  us_per_knot is the slope of the CUDA-event time
    between n1 and n2 repetitions, so the launch is excluded; us_one_repetition
    is one repetition per launch, launch included."""
    import frg
    q, qd, u = (torch.from_numpy(x).to(dev) for x in frg.sample_knots(1, seed=11))
    outs = [torch.empty((1, w), device=dev) for w in (98, 7, 49)]
    out = {}
    for lanes in (1, 8):
        def per_launch_ms(iters, count):
            for _ in range(2):
                ctx.single_knot_latency(lanes, iters, q, qd, u, *outs, stream=stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(count):
                ctx.single_knot_latency(lanes, iters, q, qd, u, *outs, stream=stream)
            e1.record(stream)
            stream.synchronize()
            return e0.elapsed_time(e1) / count
        t1, t2 = per_launch_ms(n1, reps), per_launch_ms(n2, reps)
        out[f"lanes_per_knot_{lanes}"] = {"us_per_knot": (t2 - t1) * 1e3 / (n2 - n1),
                                          "us_one_repetition": per_launch_ms(1, 50) * 1e3,
                                          "repetitions": [n1, n2]}
    return out


def entry_points(ctx, torch, dev, stream, peaks, n=65536, steps=20):
    """The entry points either side of the gradient, each on n contiguous
    device-resident knots over FLUSH_SETS rotating batches (larger than L2),
    with the context's plain launch shape: CUDA-event time per launch and the
    algorithmic bytes each moves per knot (inputs + outputs)."""
    import frg
    f32, f64 = torch.float32, torch.float64
    sets = []
    for i in range(FLUSH_SETS):
        q, qd, u = frg.sample_knots(n, seed=500 + i)
        t = {k: torch.from_numpy(x).to(dev) for k, x in (("q", q), ("qd", qd), ("u", u))}
        t["fext"] = torch.randn((n, 42), device=dev, dtype=f32)
        for k, w in (("dqdd", 98), ("qdd", 7), ("minv", 49), ("A", 196), ("B", 98)):
            t[k] = torch.empty((n, w), device=dev, dtype=f32)
        t["knots"] = torch.zeros((n, 77), device=dev, dtype=f32)
        t["knots"][:, 0:7], t["knots"][:, 7:14], t["knots"][:, 14:21] = t["q"], t["qd"], t["u"]
        for k in ("q", "qd", "u"):
            t[k + "64"] = t[k].to(f64)
        for k, w in (("dqdd64", 98), ("qdd64", 7), ("minv64", 49)):
            t[k] = torch.empty((n, w), device=dev, dtype=f64)
        sets.append(t)
    calls = {
        "gradient": (700, lambda t: ctx.gradient(n, t["q"], t["qd"], t["u"], t["dqdd"], t["qdd"], t["minv"],
                                                 stream=stream)),
        "gradient_fext": (868, lambda t: ctx.gradient_fext(n, t["q"], t["qd"], t["u"], t["fext"], t["dqdd"],
                                                           t["qdd"], t["minv"], stream=stream)),
        "forward_dynamics (qdd)": (112, lambda t: ctx.forward_dynamics(n, t["q"], t["qd"], t["u"], t["qdd"],
                                                                      stream=stream)),
        "forward_dynamics (qdd, Minv)": (308, lambda t: ctx.forward_dynamics(n, t["q"], t["qd"], t["u"], t["qdd"],
                                                                            t["minv"], stream=stream)),
        "gradient_knots (77-float records)": (84 + 224 + 392, lambda t: ctx.gradient_knots(n, t["knots"], t["dqdd"],
                                                                                         stream=stream)),
        "discrete_jacobians": (392 + 196 + 784 + 392, lambda t: ctx.discrete_jacobians(n, t["dqdd"], t["minv"], 0.01,
                                                                                       t["A"], t["B"],
                                                                                       stream=stream)),
        "gradient_f64 (verification build)": (1400, lambda t: ctx.gradient_f64(n, t["q64"], t["qd64"], t["u64"],
                                                                               t["dqdd64"], t["qdd64"], t["minv64"],
                                                                               stream=stream)),
    }
    out = {}
    for name, (bytes_per_knot, call) in calls.items():
        reps = 4 if "f64" in name else steps
        for i in range(FLUSH_SETS):
            call(sets[i])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(reps):
            call(sets[i % FLUSH_SETS])
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = {"us_per_launch": round(ms * 1e3, 2), "knots_per_s": n / (ms * 1e-3),
                     "bytes_per_knot": bytes_per_knot,
                     "hbm_frac": bytes_per_knot * n / (ms * 1e-3) / 1e9 / float(peaks["hbm_gbs"])}
    return {"n": n, "l2": f"flushed ({FLUSH_SETS} rotating batches)", "calls": out}


def mix_parity(ctx, torch, sets, n, stream):
    """Max per-knot Frobenius-relative error of each output matrix over the
    results of the batched launches, against the FP64 GPU build."""
    err = torch.empty((n, 3), dtype=torch.float64, device=sets[0][0].device)
    worst = torch.zeros(3, dtype=torch.float64, device=err.device)
    with torch.cuda.stream(stream):
        for tq, tqd, tu, outs, _, _ in sets:
            ctx.verify_f64(n, tq, tqd, tu, *outs, err, stream=stream)
            worst = torch.maximum(worst, err.max(dim=0).values)
    stream.synchronize()
    w = worst.cpu().tolist()
    return {"max_frob_rel_dqdd": w[0], "max_frob_rel_qdd": w[1], "max_frob_rel_minv": w[2], "bar": 1e-4,
            "knots": n * len(sets), "checked_by": "FP64 GPU verification build (frg_verify_f64), every knot"}


def cpu_baseline(q, qd, u, budget_s=8.0):
    """The oracle port (C restatement of the reference CPU path) on all host
    threads, on a bounded sample of the workload's knots: the full path
    (q̈, Minv and the gradient timed: the figure comparable with the GPU), and
    the reference's own time_CPU mode (q̈ and Minv passed in, untimed)."""
    import frg_oracle
    threads = os.cpu_count() or 1
    m = min(len(q), 16384)
    qs, qds, us = q[:m], qd[:m], u[:m]
    out = None
    for given in (False, True):
        fn = frg_oracle.time_threaded_given_f32 if given else frg_oracle.time_threaded_f32
        t, _ = fn(qs, qds, us, threads, 1)  # warm
        iters = max(1, int(budget_s / 2 / max(t, 1e-3)))
        t, _ = fn(qs, qds, us, threads, iters)
        sample = f"{m} knots of the mix x {iters} rounds ({t:.1f} s), FP32, damping off, gravity on"
        if not given:
            out = {"value": m * iters / t, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                   "mode": "full path: q̈, Minv and the gradient timed"}
        else:
            out["time_cpu_mode"] = {"value": m * iters / t, "unit": UNIT, "sample": sample,
                                    "mode": "the reference's time_CPU mode: q̈ and Minv passed in, not timed"}
    frg_oracle.shutdown_pool()
    return out


def run_reference(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    import frg_oracle
    h, off, n, q, qd, u = workload(0)
    threads = os.cpu_count() or 1
    for _ in range(max(args.warmup, 1)):
        frg_oracle.time_threaded_f32(q, qd, u, threads, 1)
    t, _ = frg_oracle.time_threaded_f32(q, qd, u, threads, args.steps)
    frg_oracle.shutdown_pool()
    value = n * args.steps / t
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"ragged mix: {N_TRAJ} trajectories, horizons U{{{H_LO}..{H_HI}}}, {n} knots",
                   "knots_per_step": n, "path": "CPU: oracle C restatement of helpers_CPU, persistent thread pool"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"full mix ({n} knots) per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_frg(args):
    import torch
    import frg

    ws, rank, local = dist_setup()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)
    h, off, n, q, qd, u = workload(rank, args.n_traj)
    n_traj = args.n_traj
    peaks, peaks_src = load_peaks()

    ctx = frg.Context(device=dev.index)
    if args.profile and args.plain_n:
        pn = args.plain_n
        pq, pqd, pu = (torch.from_numpy(x).to(dev) for x in frg.sample_knots(pn, seed=99))
        po = [torch.empty((pn, w), device=dev) for w in (98, 7, 49)]
        ctx.set_lanes_per_knot(args.plain_lanes)
        for _ in range(args.warmup + args.steps):
            ctx.gradient(pn, pq, pqd, pu, *po)
        torch.cuda.synchronize()
        print(json.dumps({"profile": True, "plain_n": pn, "lanes_per_knot": args.plain_lanes}))
        ctx.close()
        return 0
    tuned = None if args.profile else ctx.autotune(n)
    shape = ctx.launch_shape()
    tuning = ctx.tuning()  # plain and persistent shapes chosen by frg_autotune

    # Trajectories live in memory in a shuffled order (as separately produced
    # trajectories do), so the batch is a ragged list of scattered runs that
    # the persistent kernel walks; the plain form launches once per trajectory
    # over the same buffers.
    perm = np.random.Generator(np.random.PCG64(MIX_SEED)).permutation(n_traj)
    mem_off = np.zeros(n_traj, np.int64)
    pos = 0
    for t in perm:
        mem_off[t] = pos
        pos += int(off[t + 1] - off[t])
    stream = torch.cuda.Stream(device=dev)
    sets = []
    with torch.cuda.stream(stream):
        for i in range(ROTATING_SETS):
            qq = frg.perturb(q, 1e-3, seed=i) if i else q
            tq, tqd, tu = (torch.from_numpy(x).to(dev) for x in (qq, qd, u))
            outs = (torch.empty((n, 98), device=dev), torch.empty((n, 7), device=dev), torch.empty((n, 49), device=dev))
            o = [int(x) for x in mem_off]
            trajs = [(int(off[t + 1] - off[t]), tq[o[t]:], tqd[o[t]:], tu[o[t]:], outs[0][o[t]:], outs[1][o[t]:],
                      outs[2][o[t]:]) for t in range(n_traj)]
            plan = ctx.plan(trajs)
            sets.append((tq, tqd, tu, outs, plan, trajs))
    stream.synchronize()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    def timed(fn, steps):
        """CUDA-event time (ms) on `stream` of `steps` calls issued back to
        back between one pair of events, as a list of `steps` equal per-step
        shares.  (Bracketing every step with its own events instead adds the
        stream's event processing, about 4 us, to each launch.)"""
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(steps):
            fn(i)
        e1.record(stream)
        stream.synchronize()
        return [e0.elapsed_time(e1) / steps] * steps

    # ---- batched (value) ----
    # clocks are sampled over a load window: >= 1.5 s of back-to-back warm-up
    # launches (at least W of them) followed by the K timed steps
    clocks = ClockSampler(dev.index)
    clocks.start()
    i, tw = 0, time.perf_counter()
    load_window_s = 0.0 if args.profile else 1.5  # profiling: W warm-up launches only
    while i < args.warmup or time.perf_counter() - tw < load_window_s:
        sets[i % ROTATING_SETS][4].launch(stream)
        i += 1
        if i % 64 == 0:
            stream.synchronize()
    # The K steps are K independent batches (the rotating sets).  Timed two
    # ways: back to back on one stream (single_stream), and as one
    # frg_plan_launch_many call with IN_FLIGHT batches in flight (step i on
    # stream i mod IN_FLIGHT), so that a launch's partial last wave of tiles
    # overlaps the next batches (value).  ROTATING_SETS is a multiple of
    # IN_FLIGHT, so each set always runs on the same stream.
    plans = [sets[i % ROTATING_SETS][4] for i in range(args.steps)]
    if not args.profile:
        ctx.plan_launch_many([s[4] for s in sets] * 2, stream, IN_FLIGHT)
    barrier()
    single_ms = timed(lambda i: sets[i % ROTATING_SETS][4].launch(stream), args.steps)
    barrier()
    t0 = time.perf_counter()
    if args.profile:
        step_ms = single_ms
    else:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.plan_launch_many(plans, stream, IN_FLIGHT)
        e1.record(stream)
        stream.synchronize()
        step_ms = [e0.elapsed_time(e1) / args.steps] * args.steps
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    from frg import dist as fdist
    value, total_ms, _ = fdist.aggregate(sum(step_ms), n, args.steps, device=dev)
    ms_per_step = total_ms / args.steps
    single_value, single_total_ms, _ = fdist.aggregate(sum(single_ms), n, args.steps, device=dev)

    # ---- parity of the timed launches' results: every knot of every rotating
    # set against the FP64 GPU verification build ----
    parity = None if args.profile else mix_parity(ctx, torch, sets, n, stream)

    if args.profile:
        if rank == 0:
            print(json.dumps({"profile": True, "knots_per_step": n, "steps": args.steps,
                              "launch_ms": statistics.mean(step_ms), "launch_shape": shape}))
        for s in sets:
            s[4].close()
        ctx.close()
        return 0

    # ---- plain per-trajectory launches ----
    for i in range(args.warmup):
        ctx.per_trajectory(sets[i % ROTATING_SETS][5], stream)
    plain_ms = timed(lambda i: ctx.per_trajectory(sets[i % ROTATING_SETS][5], stream), max(5, args.steps // 5))
    plain_value = n / (statistics.mean(plain_ms) * 1e-3)

    # ---- e2e through the C ABI with host buffers ----
    # two sets of pinned buffers: the pipelined call keeps two batches in
    # flight, and neighbouring batches must not share output arrays
    hsets = []
    for _ in range(2):
        hin = [frg.lib().frg_host_alloc(7 * 4 * n) for _ in range(3)]
        hout = [frg.lib().frg_host_alloc(w * 4 * n) for w in (98, 7, 49)]
        for ptr, arr in zip(hin, (q, qd, u)):
            np.ctypeslib.as_array((ctypes.c_float * (7 * n)).from_address(ptr))[:] = arr.reshape(-1)
        hsets.append(hin + hout)
    e2e_steps = max(5, args.steps)  # K steps, each the whole mix from host buffers to host buffers
    # one frg_gradient_host call per step (synchronous: launch, results, return)
    for _ in range(max(1, args.warmup)):
        ctx.gradient_host_into(n, *hsets[0])
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.gradient_host_into(n, *hsets[0])
    e2e_single_s = (time.perf_counter() - t0) / e2e_steps
    # the same steps as batches of one frg_gradient_host_batches call
    batches = [(n, *hsets[i % 2]) for i in range(e2e_steps)]
    ctx.gradient_host_batches(batches[:max(2, args.warmup)])
    t0 = time.perf_counter()
    ctx.gradient_host_batches(batches)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    # the reference's "Completely Fused" output (time_GPU.cu:316 copies back
    # dqdd only): q̈ and Minv not asked for, so they stay on the device
    grad_only = [(n, *hsets[i % 2][:4], None, None) for i in range(e2e_steps)]
    ctx.gradient_host_batches(grad_only[:max(2, args.warmup)])
    t0 = time.perf_counter()
    ctx.gradient_host_batches(grad_only)
    e2e_grad_s = (time.perf_counter() - t0) / e2e_steps
    for hs in hsets:
        for p in hs:
            frg.lib().frg_host_free(p)

    link = host_link_rates(torch, dev, stream, 616 * n)

    # ---- plain path scaling (one launch per batch of N knots) ----
    fp32 = fp32_peak_live(dev.index)
    fp32_peak = fp32["peak"]
    scaling = plain_scaling(ctx, torch, dev, stream, peaks, fp32_peak)
    entries = entry_points(ctx, torch, dev, stream, peaks)
    latency = single_knot(ctx, torch, dev, stream)

    # ---- serving: latency at 50 % of saturation, and admission under a 2 GiB pool ----
    served = served_adm = None
    if not args.no_serve:
        from frg import serve
        served = serve.bench_latency(ctx, seconds=3.0)
        served_adm = serve.bench_admission(ctx)

    line = None
    if rank == 0:
        launch_ms = statistics.mean(step_ms)
        achieved_gbs = BYTES_PER_KNOT * n / (launch_ms * 1e-3) / 1e9
        traffic_pk = (NCU_MIX["dram_read_bytes"] + NCU_MIX["dram_write_bytes"]) / NCU_MIX["knots"]
        fp32_achieved = FLOP_PER_KNOT_REF * n / (launch_ms * 1e-3) / 1e12
        fp32_peak = fp32["peak"]
        fp32_executed = NCU_MIX["executed_flop_per_knot"] * n / (launch_ms * 1e-3) / 1e12
        d2h_s = 616 * n / (link["d2h_gbs"] * 1e9)
        d2h_packed_s = D2H_PACKED * n / (link["d2h_gbs"] * 1e9)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {
                "workload": f"ragged mix: {n_traj} trajectories, horizons U{{{H_LO}..{H_HI}}} (seed {MIX_SEED}), "
                            f"{n} knots per rank, stored in shuffled order; one persistent launch over the "
                            f"ragged trajectory list, one plan launch per step; the steps are independent "
                            f"batches, {IN_FLIGHT} in flight on {IN_FLIGHT} streams (frg_plan_launch_many)",
                "knots_per_step": n, "l2": f"{ROTATING_SETS} rotating input/output sets "
                                            f"({ROTATING_SETS * n * BYTES_PER_KNOT / 1e6:.0f} MB > 129 MB L2)",
                "launch_shape": tuning,
                "autotune_knots_per_s": tuned, "parallelism": f"replicas x{ws} (knots sharded, no collective)",
            },
            "e2e": {"value": n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 84 * n,
                    "d2h_bytes_per_step": D2H_PACKED * n,
                    "call": f"frg_gradient_host_batches: {e2e_steps} steps, each the whole mix from pinned host "
                            f"buffers to pinned host buffers (dqdd, q̈, dense Minv: 616 B per knot), two "
                            f"batches in flight; Minv crosses the link as its upper triangle (112 of 196 B) "
                            f"and host threads expand it into the dense arrays inside the call",
                    "ms_per_step": e2e_s * 1e3,
                    "host_link": dict(link, bound="d2h: bytes over the link / measured device-to-host copy rate",
                                      bound_ms=d2h_packed_s * 1e3),
                    "host_link_frac": d2h_packed_s / e2e_s,
                    "single_call": {"value": n / e2e_single_s, "ms_per_step": e2e_single_s * 1e3,
                                    "d2h_bytes_per_step": 616 * n,
                                    "host_link_frac": d2h_s / e2e_single_s,
                                    "call": "one synchronous frg_gradient_host per step (dense Minv over the link)"},
                    "gradient_only": {"value": n / e2e_grad_s, "ms_per_step": e2e_grad_s * 1e3,
                                      "d2h_bytes_per_step": 392 * n,
                                      "host_link_frac": d2h_s * 392 / 616 / e2e_grad_s,
                                      "call": "frg_gradient_host_batches with qdd and minv NULL: dqdd alone "
                                              "returned, the output of the reference's Completely Fused call"}},
            "single_stream": {"value": single_value, "unit": UNIT, "ms_per_step": single_total_ms / args.steps,
                              "call": "the same K plan launches back to back on one stream (each launch starts "
                                      "while the one before finishes, programmatic dependent launch)"},
            "plain_per_trajectory": {"value": plain_value, "unit": UNIT, "launches_per_step": n_traj,
                                     "ms_per_step": statistics.mean(plain_ms)},
            "batched_vs_plain": value / ws / plain_value,
            "plain_scaling": scaling,
            "entry_points": entries,
            "single_knot": latency,
            "parity": parity,
            "served": served,
            "served_admission": served_adm,
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": float(peaks["hbm_gbs"]), "unit": "GB/s",
                         "frac": achieved_gbs / float(peaks["hbm_gbs"]),
                         "traffic": traffic_pk * n,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of this kernel on this "
                                           "mix (NCU_MIX); the results stay dirty in L2 when the kernel ends",
                         "peak_source": f"{peaks_src} (MEASURED_PEAKS.json hbm_gbs)" if peaks_src == "measured"
                         else "fallback 6.8 TB/s", "bytes_per_knot": BYTES_PER_KNOT,
                         "kernel": "grad_ragged_kernel", "launch_ms": launch_ms,
                         "launch_ms_note": f"time per batch with {IN_FLIGHT} independent batches in flight; "
                                           "single_stream.ms_per_step is one launch after another"},
            "compute_roofline": {"bound": "fp32", "achieved": fp32_achieved, "unit": "TFLOP/s",
                                 "peak": fp32_peak, "frac": fp32_achieved / fp32_peak,
                                 "flop_per_knot": FLOP_PER_KNOT_REF,
                                 "executed_flop_per_knot": NCU_MIX["executed_flop_per_knot"],
                                 "achieved_executed": fp32_executed,
                                 "frac_executed": fp32_executed / fp32_peak,
                                 "peak_source": fp32["source"],
                                 "peak_probe": {k: v for k, v in fp32.items() if k.endswith("tflops")}},
            "clocks": dict(clk, window="warm-up (>= 1.5 s of launches) + timed steps"),
            "wall_s_timed_region": wall,
            "gpu_launches": args.steps,
        }
    if not args.no_cpu_baseline and rank == 0:
        line["cpu_baseline"] = cpu_baseline(q, qd, u)
    for s in sets:
        s[4].close()
    ctx.close()
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_frg(args)


if __name__ == "__main__":
    sys.exit(main())
