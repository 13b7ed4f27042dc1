"""ctypes access to the oracle (test infrastructure only).

ORACLE TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline / reference arm, as the checker or as the timed CPU
baseline, never by the product path.

  libfrg_oracle.so   C restatement of the reference's CPU path (frg_oracle.c),
                     FP64/FP32, and its threaded driver.
  _ref/libfrg_ref.so the reference's own helpers_CPU code, where it was built
                     (needs the reference tree; absent on machines without it).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libfrg_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfrg_ref.so")

_oracle = None
_ref = None


def build():
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile"), "oracle"], check=True)


def _load():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        vp, i = ctypes.c_void_p, ctypes.c_int
        for name in ("frg_oracle_gradient_f64", "frg_oracle_gradient_f32"):
            getattr(L, name).argtypes = [i, vp, vp, vp, vp, i, i, vp, vp, vp]
            getattr(L, name).restype = i
        L.frg_oracle_time_threaded_f32.argtypes = [i, vp, vp, vp, vp, vp, vp, i, i]
        L.frg_oracle_time_threaded_f32.restype = ctypes.c_double
        L.frg_oracle_time_threaded_mode_f32.argtypes = [i, vp, vp, vp, vp, vp, vp, i, i, i]
        L.frg_oracle_time_threaded_mode_f32.restype = ctypes.c_double
        L.frg_oracle_gradient_given_f32.argtypes = [i, vp, vp, vp, vp, vp]
        L.frg_oracle_gradient_given_f32.restype = i
        L.frg_oracle_model_f64.argtypes = [vp, vp, vp]
        L.frg_oracle_pool_shutdown.argtypes = []
        L.frg_oracle_dofs.argtypes = []
        L.frg_oracle_dofs.restype = i
        _oracle = L
    return _oracle


def ref_available():
    return os.path.exists(REF_SO)


def _load_ref():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_SO)
        vp, i = ctypes.c_void_p, ctypes.c_int
        for name in ("frg_ref_gradient_f64", "frg_ref_gradient_f32"):
            getattr(L, name).argtypes = [i, vp, vp, vp, i, i, vp, vp, vp]
            getattr(L, name).restype = i
        _ref = L
    return _ref


def _run(fn, dtype, q, qd, u, damping, mpc, fext=None, with_fext=True):
    q, qd, u = (np.ascontiguousarray(x, dtype=dtype) for x in (q, qd, u))
    n, nj = q.shape[0], q.shape[1]
    dqdd = np.zeros((n, 2 * nj * nj), dtype)
    qdd = np.zeros((n, nj), dtype)
    minv = np.zeros((n, nj * nj), dtype)
    args = [n, q.ctypes.data, qd.ctypes.data, u.ctypes.data]
    if with_fext:
        fx = None if fext is None else np.ascontiguousarray(fext, dtype=dtype)
        args.append(None if fx is None else fx.ctypes.data)
    args += [int(damping), int(mpc), dqdd.ctypes.data, qdd.ctypes.data, minv.ctypes.data]
    rc = fn(*args)
    if rc != 0:
        raise RuntimeError(f"oracle returned {rc}")
    return dqdd, qdd, minv


def gradient_f64(q, qd, u, damping=False, mpc=False, fext=None):
    """Oracle in FP64: (dqdd [n,98], qdd [n,7], minv [n,49]) float64."""
    return _run(_load().frg_oracle_gradient_f64, np.float64, q, qd, u, damping, mpc, fext)


def gradient_f32(q, qd, u, damping=False, mpc=False, fext=None):
    return _run(_load().frg_oracle_gradient_f32, np.float32, q, qd, u, damping, mpc, fext)


def ref_gradient_f64(q, qd, u, damping=False, mpc=False):
    """The reference's own helpers_CPU path (oracle/_ref) in FP64."""
    return _run(_load_ref().frg_ref_gradient_f64, np.float64, q, qd, u, damping, mpc, with_fext=False)


def ref_gradient_f32(q, qd, u, damping=False, mpc=False):
    return _run(_load_ref().frg_ref_gradient_f32, np.float32, q, qd, u, damping, mpc, with_fext=False)


def model_f64(q):
    """(X [7,36], I [7,36]) column-major joint transforms and inertias at q."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    X = np.zeros((7, 36))
    I = np.zeros((7, 36))
    _load().frg_oracle_model_f64(q.ctypes.data, X.ctypes.data, I.ctypes.data)
    return X, I


def time_threaded_f32(q, qd, u, threads, iters):
    """Wall seconds of `iters` rounds of the FP32 full path over all knots on
    `threads` persistent workers (damping off, gravity on)."""
    q, qd, u = (np.ascontiguousarray(x, dtype=np.float32) for x in (q, qd, u))
    n = q.shape[0]
    dqdd = np.zeros((n, 98), np.float32)
    qdd = np.zeros((n, 7), np.float32)
    minv = np.zeros((n, 49), np.float32)
    t = _load().frg_oracle_time_threaded_f32(n, q.ctypes.data, qd.ctypes.data, u.ctypes.data, dqdd.ctypes.data,
                                             qdd.ctypes.data, minv.ctypes.data, int(threads), int(iters))
    if t < 0:
        raise RuntimeError("oracle thread pool failed")
    return t, (dqdd, qdd, minv)


def time_threaded_given_f32(q, qd, u, threads, iters):
    """Wall seconds of `iters` rounds of the reference's time_CPU mode: q̈ and
    Minv precomputed (untimed) and passed in, the gradient timed."""
    q, qd, u = (np.ascontiguousarray(x, dtype=np.float32) for x in (q, qd, u))
    n = q.shape[0]
    dqdd, qdd, minv = gradient_f32(q, qd, u)
    L = _load()
    t = L.frg_oracle_time_threaded_mode_f32(n, q.ctypes.data, qd.ctypes.data, u.ctypes.data, dqdd.ctypes.data,
                                            qdd.ctypes.data, minv.ctypes.data, int(threads), int(iters), 1)
    if t < 0:
        raise RuntimeError("oracle thread pool failed")
    return t, (dqdd, qdd, minv)


def gradient_given_f32(q, qd, qdd, minv):
    """dqdd [n,98] from q, qd and the given q̈ [n,7], Minv [n,49] (time_CPU mode)."""
    q, qd, qdd, minv = (np.ascontiguousarray(x, dtype=np.float32) for x in (q, qd, qdd, minv))
    n = q.shape[0]
    dqdd = np.zeros((n, 98), np.float32)
    _load().frg_oracle_gradient_given_f32(n, q.ctypes.data, qd.ctypes.data, qdd.ctypes.data, minv.ctypes.data,
                                          dqdd.ctypes.data)
    return dqdd


def shutdown_pool():
    if _oracle is not None:
        _oracle.frg_oracle_pool_shutdown()


def frob_rel(a, b, axis=-1):
    """Per-knot Frobenius-relative error ||a - b|| / ||b|| (b the reference)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b, axis=axis)
    num = np.linalg.norm(a - b, axis=axis)
    return num / np.maximum(den, 1e-300)
