"""Serving measurements over the C++ load generator (frg/libfrg_loadgen.so).

bench_latency():   closed-loop saturation, then Poisson arrivals at 50 % of
                   the saturated session rate: sessions of horizon
                   {16, 32, 64, 128}, 5 calls each, inputs perturbed by
                   N(0, 1e-2) per call; p50/p99 latency overall and for
                   64-knot calls, throughput.  Once with host inputs and
                   results (frg_server_submit), once device-resident
                   (iterates already on the GPU, results kept there:
                   frg_server_submit_device).
bench_admission(): 20,000 sessions queued at once, horizons U{8..512}, 10
                   calls each, device pool capped at 2 GiB so admission
                   throttles; throughput, p50/p99, admission stalls, and 1 %
                   of calls verified by the FP64 GPU build (frg_verify_f64).
"""
import ctypes
import os

import numpy as np

from .native import DQDD_FLOATS, MINV_FLOATS, NUM_JOINTS, FrgError, Server, lib

_HERE = os.path.dirname(os.path.abspath(__file__))
LOADGEN_PATH = os.path.join(_HERE, "libfrg_loadgen.so")


class LoadgenCfg(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("rate", ctypes.c_double), ("concurrency", ctypes.c_int),
                ("total_sessions", ctypes.c_int), ("duration_s", ctypes.c_double), ("calls", ctypes.c_int),
                ("horizons", ctypes.POINTER(ctypes.c_int)), ("n_horizons", ctypes.c_int),
                ("horizon_lo", ctypes.c_int), ("horizon_hi", ctypes.c_int), ("sigma", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("sample_frac", ctypes.c_double), ("sample_cap", ctypes.c_int),
                ("sample_q", ctypes.c_void_p), ("sample_qd", ctypes.c_void_p), ("sample_u", ctypes.c_void_p),
                ("sample_dqdd", ctypes.c_void_p), ("sample_qdd", ctypes.c_void_p), ("sample_minv", ctypes.c_void_p),
                ("sample_h", ctypes.c_void_p), ("threads", ctypes.c_int), ("source", ctypes.c_int)]


class LoadgenResult(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("calls", "knots", "sessions", "errors", "samples", "sample_knots")] + \
               [(f, ctypes.c_double) for f in ("elapsed_s", "calls_per_s", "knots_per_s", "p50_us", "p90_us",
                                               "p99_us", "max_us", "mean_us", "p50_h64_us", "p99_h64_us",
                                               "mean_batch_requests")]


_lg = None


def loadgen():
    global _lg
    if _lg is None:
        lib()  # libfrg.so first (the load generator links it)
        if not os.path.exists(LOADGEN_PATH):
            raise FrgError(9, f"{LOADGEN_PATH} is missing: build with __graft_entry__.build()")
        L = ctypes.CDLL(LOADGEN_PATH)
        L.frg_loadgen_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(LoadgenCfg), ctypes.POINTER(LoadgenResult)]
        L.frg_loadgen_run.restype = ctypes.c_int
        _lg = L
    return _lg


def run(server, mode, rate=0.0, concurrency=0, total_sessions=0, duration_s=1.0, calls=5, horizons=(16, 32, 64, 128),
        horizon_range=None, sigma=1e-2, seed=1, sample_frac=0.0, sample_cap=0, threads=None, source=0):
    """One load-generator run; source 0: host inputs and results, 1: inputs
    already on the GPU and results kept there."""
    cfg = LoadgenCfg()
    cfg.source = int(source)
    cfg.threads = threads or min(8, max(1, (os.cpu_count() or 2) // 2))
    cfg.mode, cfg.rate, cfg.concurrency, cfg.total_sessions = mode, rate, concurrency, total_sessions
    cfg.duration_s, cfg.calls, cfg.sigma, cfg.seed = duration_s, calls, sigma, seed
    hz = (ctypes.c_int * max(1, len(horizons)))(*horizons) if horizons else None
    if horizons:
        cfg.horizons, cfg.n_horizons = ctypes.cast(hz, ctypes.POINTER(ctypes.c_int)), len(horizons)
    else:
        cfg.n_horizons = 0
        cfg.horizon_lo, cfg.horizon_hi = horizon_range
    bufs = None
    if sample_frac > 0 and sample_cap > 0:
        bufs = {k: np.zeros((sample_cap, w), np.float32) for k, w in
                (("q", 7), ("qd", 7), ("u", 7), ("dqdd", DQDD_FLOATS), ("qdd", NUM_JOINTS), ("minv", MINV_FLOATS))}
        bufs["h"] = np.zeros(sample_cap, np.int64)
        cfg.sample_frac, cfg.sample_cap = sample_frac, sample_cap
        for k in ("q", "qd", "u", "dqdd", "qdd", "minv"):
            setattr(cfg, "sample_" + k, bufs[k].ctypes.data)
        cfg.sample_h = bufs["h"].ctypes.data
    res = LoadgenResult()
    rc = loadgen().frg_loadgen_run(server._h, ctypes.byref(cfg), ctypes.byref(res))
    out = {f: getattr(res, f) for f, _ in LoadgenResult._fields_}
    out["rc"] = rc
    if bufs is not None:
        n = int(res.sample_knots)
        out["sample"] = {k: v[:n] for k, v in bufs.items() if k != "h"}
        out["sample"]["h"] = bufs["h"][:int(res.samples)]
    return out


def _summ(r, keys):
    return {k: (round(r[k], 3) if isinstance(r[k], float) else r[k]) for k in keys}


def bench_latency(ctx, seconds=3.0, sat_seconds=1.5, concurrency=512):
    """Saturation (closed loop) then 50 % load (open loop), for host-submitted
    calls and for device-resident ones."""
    keys = ("calls", "knots", "sessions", "errors", "elapsed_s", "calls_per_s", "knots_per_s", "p50_us", "p90_us",
            "p99_us", "max_us", "mean_us", "p50_h64_us", "p99_h64_us", "mean_batch_requests")
    out = {"workload": "sessions of horizon {16,32,64,128}, 5 calls each, inputs perturbed by N(0,1e-2) per call"}
    for source, name in ((0, None), (1, "device_resident")):
        with Server(ctx, pool_bytes=1 << 30, max_inflight=3) as srv:
            run(srv, 1, concurrency=64, duration_s=0.3, seed=11, source=source)  # warm-up
            sat = run(srv, 1, concurrency=concurrency, duration_s=sat_seconds, seed=12, source=source)
            session_rate = 0.5 * sat["calls_per_s"] / 5.0
            half = run(srv, 0, rate=session_rate, duration_s=seconds, seed=13, source=source)
            stats = srv.stats()
        leg = {
            "saturation": dict(_summ(sat, keys), concurrency=concurrency),
            "half_load": dict(_summ(half, keys), session_rate_per_s=round(session_rate, 1)),
            "launches": stats["launches"],
        }
        if name is None:
            out.update(leg)
        else:
            out[name] = dict(leg, calls="frg_server_submit_device: iterates already on the GPU (staged before "
                                        "the run), results kept in the device slot; latency = submit -> results "
                                        "in device memory")
    return out


def bench_admission(ctx, sessions=20000, pool_bytes=2 << 30):
    """20k queued sessions, horizons U{8..512}, 10 calls each, 2 GiB pool."""
    cap = 200_000
    with Server(ctx, pool_bytes=pool_bytes, max_inflight=3) as srv:
        r = run(srv, 2, total_sessions=sessions, calls=10, horizons=(), horizon_range=(8, 512), seed=21,
                sample_frac=0.01, sample_cap=cap)
        stats = srv.stats()
    out = _summ(r, ("calls", "knots", "sessions", "errors", "elapsed_s", "calls_per_s", "knots_per_s", "p50_us",
                    "p99_us", "max_us", "mean_batch_requests"))
    out.update(admission_stalls=stats["admission_stalls"], pool_bytes_cap=stats["pool_bytes_cap"],
               pool_bytes_peak=stats["pool_bytes_peak"], launches=stats["launches"])
    if "sample" in r and len(r["sample"]["q"]):
        s = r["sample"]
        err, ms = verify_f64_gpu(ctx, s)
        chk = {
            "sampled_calls": int(len(s["h"])), "sampled_knots": int(len(s["q"])),
            "max_frob_rel_dqdd": float(err[:, 0].max()),
            "max_frob_rel_qdd": float(err[:, 1].max()),
            "max_frob_rel_minv": float(err[:, 2].max()),
            "gpu_verify_ms": round(ms, 3),
            "where": "FP64 GPU verification build (frg_verify_f64) on 1 % of calls, after the run",
        }
        out["fp64_check"] = chk
    return out


def verify_f64_gpu(ctx, s):
    """Per-knot FP64 errors [n, 3] of sampled FP32 results, on the GPU; and the
    device time of one verification call (ms), its scratch already sized."""
    import torch
    n = len(s["q"])
    t = {k: torch.from_numpy(np.ascontiguousarray(s[k], np.float32)).cuda()
         for k in ("q", "qd", "u", "dqdd", "qdd", "minv")}
    err = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    args = (n, t["q"], t["qd"], t["u"], t["dqdd"], t["qdd"], t["minv"], err)
    ctx.verify_f64(*args, stream=st)  # sizes the context's FP64 scratch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    ctx.verify_f64(*args, stream=st)
    e1.record(st)
    st.synchronize()
    return err.cpu().numpy(), e0.elapsed_time(e1)
