"""URDF-generated robots on the GPU: the library built for a synthetic arm of
model_helpers (general frames, tilted joint axes, welded links, a live column
0 of d tau / dq) against the oracle built from the same tables, in every
mode, and its two thread mappings against each other -- for arms of 7, 6 and
3 joints (the joint count is a compile-time model parameter, as the
reference's NUM_POS is)."""
import ctypes

import numpy as np
import pytest

from conftest import ROOT, TOL, max_err
from model_helpers import build_oracle, oracle_gradient_f64, synthetic_urdf, write_tables

pytestmark = pytest.mark.gpu


class Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("vel_damping", ctypes.c_int), ("mpc_mode", ctypes.c_int),
                ("warps_per_cta", ctypes.c_int), ("ctas_per_sm", ctypes.c_int), ("lanes_per_knot", ctypes.c_int)]


@pytest.fixture(scope="module", params=[7, 6, 3])
def synthetic(tmp_path_factory, request):
    from frg import build
    d = tmp_path_factory.mktemp(f"synthetic_model{request.param}")
    header = write_tables(synthetic_urdf(joints=request.param), str(d / "synthetic_tables.h"))
    lib = ctypes.CDLL(build.build_model(header, str(d / "lib")))
    vp, i = ctypes.c_void_p, ctypes.c_int
    lib.frg_model_name.restype = ctypes.c_char_p
    lib.frg_model_dofs.restype = i
    assert lib.frg_model_dofs() == request.param
    lib.frg_options_default.argtypes = [ctypes.POINTER(Options)]
    lib.frg_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Options)]
    lib.frg_destroy.argtypes = [vp]
    lib.frg_set_lanes_per_knot.argtypes = [vp, i]
    lib.frg_gradient_host.argtypes = [vp, i, vp, vp, vp, vp, vp, vp]
    lib.frg_last_error.argtypes = [vp]
    lib.frg_last_error.restype = ctypes.c_char_p
    oracle = build_oracle(header, str(d / "liboracle_synthetic.so"), ROOT)
    return lib, oracle


def _gradient(lib, q, qd, u, damping, mpc, lanes):
    opt = Options()
    lib.frg_options_default(ctypes.byref(opt))
    opt.vel_damping, opt.mpc_mode = damping, mpc
    ctx = ctypes.c_void_p()
    assert lib.frg_create(ctypes.byref(ctx), ctypes.byref(opt)) == 0
    try:
        assert lib.frg_set_lanes_per_knot(ctx, lanes) == 0
        n, nj = q.shape
        out = [np.full((n, w), np.nan, np.float32) for w in (2 * nj * nj, nj, nj * nj)]
        st = lib.frg_gradient_host(ctx, n, *(x.ctypes.data for x in (q, qd, u)), *(o.ctypes.data for o in out))
        assert st == 0, lib.frg_last_error(ctx)
        return out
    finally:
        lib.frg_destroy(ctx)


def _knots(n, nj, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-2.5, 2.5, (n, nj)).astype(np.float32), rng.uniform(-2, 2, (n, nj)).astype(np.float32),
            rng.uniform(-20, 20, (n, nj)).astype(np.float32))


@pytest.mark.parametrize("damping,mpc", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_generated_model_matches_its_oracle(synthetic, damping, mpc):
    lib, oracle = synthetic
    assert lib.frg_model_name().decode() == "synthetic_arm"
    nj = lib.frg_model_dofs()
    q, qd, u = _knots(1500, nj, 40 + 2 * damping + mpc)
    got = _gradient(lib, q, qd, u, damping, mpc, lanes=1)
    ref = oracle_gradient_f64(oracle, q, qd, u, damping, mpc)
    for name, g, r in zip(("dqdd", "qdd", "minv"), got, ref):
        assert max_err(g, r) <= TOL, name
    if not mpc:  # the tilted base joint gives d qdd / dq a live column 0
        assert np.abs(got[0][:, :nj]).max() > 1e-2


def test_generated_model_thread_mappings_agree(synthetic):
    """The latency mapping computes d tau / dq column 0 on lane N for this
    robot; both mappings still give the same bits."""
    lib, _ = synthetic
    q, qd, u = _knots(3000, lib.frg_model_dofs(), 9)
    a = _gradient(lib, q, qd, u, 0, 0, lanes=1)
    b = _gradient(lib, q, qd, u, 0, 0, lanes=8)
    for x, y in zip(a, b):
        assert np.count_nonzero(x != y) == 0
