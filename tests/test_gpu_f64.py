"""FP64 verification build (GPU): frg_gradient_f64 against the reference's own
FP64 outputs (golden fixtures) and the FP64 oracle, and frg_verify_f64's
per-knot errors against the same errors computed on the host."""
import numpy as np
import pytest

import frg
import frg_oracle
from conftest import TOL

pytestmark = pytest.mark.gpu

# Both sides are double; only the operation order differs.
TOL64 = 1e-10


def f64_gradient(torch, ctx, q, qd, u):
    n = q.shape[0]
    tq, tqd, tu = (torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda() for a in (q, qd, u))
    out = [torch.full((n, w), float("nan"), device="cuda", dtype=torch.float64) for w in (98, 7, 49)]
    ctx.gradient_f64(n, tq, tqd, tu, *out)
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in out]


@pytest.mark.parametrize("damping,mpc", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_f64_matches_reference_fp64_golden(golden, damping, mpc):
    import torch
    q, qd, u = golden["q"], golden["qd"], golden["u"]
    with frg.Context(vel_damping=damping, mpc_mode=mpc) as ctx:
        got = f64_gradient(torch, ctx, q, qd, u)
    for name, g in zip(("dqdd", "qdd", "minv"), got):
        ref = golden[f"{name}_f64_d{damping}_m{mpc}"]
        assert float(frg_oracle.frob_rel(g, ref).max()) <= TOL64, name


@pytest.mark.parametrize("n", [1, 31, 33, 1001])
def test_f64_matches_oracle_sizes(n):
    """Odd counts put the scratch arrays of the verify path off 16-byte
    alignment; here they exercise the tail tile and idle lanes."""
    import torch
    q, qd, u = frg.sample_knots(n, seed=900 + n)
    with frg.Context() as ctx:
        got = f64_gradient(torch, ctx, q.astype(np.float64), qd.astype(np.float64), u.astype(np.float64))
    ref = frg_oracle.gradient_f64(q, qd, u)
    for g, r in zip(got, ref):
        assert float(frg_oracle.frob_rel(g, r).max()) <= TOL64


def test_f64_angles_outside_pi():
    """Angles beyond [-pi, pi] (the FP32 build switches sincos routines there)."""
    import torch
    n = 64
    q, qd, u = frg.sample_knots(n, seed=5)
    q = q.astype(np.float64) + np.where(np.arange(n)[:, None] % 2 == 0, 7.0, -9.5)
    with frg.Context() as ctx:
        got = f64_gradient(torch, ctx, q, qd.astype(np.float64), u.astype(np.float64))
    ref = frg_oracle.gradient_f64(q, qd, u)
    for g, r in zip(got, ref):
        assert float(frg_oracle.frob_rel(g, r).max()) <= TOL64


@pytest.mark.parametrize("n", [1, 97, 4099])
def test_verify_f64_errors(n):
    """frg_verify_f64 reports the FP32 engine's per-knot errors: they agree
    with the errors the host computes against the FP64 oracle, and lie inside
    the parity bar."""
    import torch
    q, qd, u = frg.sample_knots(n, seed=77 + n)
    tq, tqd, tu = (torch.from_numpy(a).cuda() for a in (q, qd, u))
    out = [torch.empty((n, w), device="cuda") for w in (98, 7, 49)]
    err = torch.full((n, 3), float("nan"), device="cuda", dtype=torch.float64)
    with frg.Context() as ctx:
        ctx.gradient(n, tq, tqd, tu, *out)
        ctx.verify_f64(n, tq, tqd, tu, *out, err)
        torch.cuda.synchronize()
    got = err.cpu().numpy()
    ref = frg_oracle.gradient_f64(q, qd, u)
    host = np.stack([frg_oracle.frob_rel(o.cpu().numpy(), r) for o, r in zip(out, ref)], axis=1)
    assert np.all(np.isfinite(got))
    assert float(got.max()) <= TOL
    np.testing.assert_allclose(got, host, rtol=1e-6, atol=1e-12)


def test_verify_f64_flags_a_bad_result_and_nan():
    """A corrupted FP32 result shows up in its knot's error only; a NaN input
    gives NaN errors for that knot and leaves the others finite."""
    import torch
    n = 70
    q, qd, u = frg.sample_knots(n, seed=3)
    q[41, 2] = np.nan
    tq, tqd, tu = (torch.from_numpy(a).cuda() for a in (q, qd, u))
    out = [torch.empty((n, w), device="cuda") for w in (98, 7, 49)]
    err = torch.empty((n, 3), device="cuda", dtype=torch.float64)
    with frg.Context() as ctx:
        ctx.gradient(n, tq, tqd, tu, *out)
        out[0][12, 5] += 1.0  # plant a wrong entry in knot 12's dqdd
        ctx.verify_f64(n, tq, tqd, tu, *out, err)
        torch.cuda.synchronize()
    e = err.cpu().numpy()
    assert np.all(np.isnan(e[41]))
    ok = np.delete(np.arange(n), [12, 41])
    assert float(e[ok].max()) <= TOL
    assert e[12, 0] > 1e-3 and e[12, 1] <= TOL and e[12, 2] <= TOL


def test_f64_argument_errors():
    import torch
    with frg.Context() as ctx:
        ctx.gradient_f64(0, None, None, None, None, None, None)  # empty batch: no-op
        ctx.verify_f64(0, None, None, None, None, None, None, None)
        x = torch.zeros((4, 7), device="cuda", dtype=torch.float64)
        with pytest.raises(frg.FrgError) as ei:
            ctx.gradient_f64(4, x, x, None, x, x, x)
        assert ei.value.status == 1
        with pytest.raises(frg.FrgError) as ei:
            ctx.verify_f64(-1, x, x, x, x, x, x, x)
        assert ei.value.status == 1


def test_verify_f64_scratch_survives_host_calls():
    """The FP64 scratch and the host-call staging are separate context buffers:
    growing one leaves the other valid (verify, host call, verify smaller and
    larger)."""
    import torch
    with frg.Context() as ctx:
        for n in (500, 3000, 200, 5000):
            q, qd, u = frg.sample_knots(n, seed=n)
            tq, tqd, tu = (torch.from_numpy(a).cuda() for a in (q, qd, u))
            out = [torch.empty((n, w), device="cuda") for w in (98, 7, 49)]
            err = torch.empty((n, 3), device="cuda", dtype=torch.float64)
            ctx.gradient(n, tq, tqd, tu, *out)
            ctx.verify_f64(n, tq, tqd, tu, *out, err)
            torch.cuda.synchronize()
            assert float(err.max()) <= TOL
            hd, hq, hm = ctx.gradient_host(q, qd, u)  # grows the staging buffer
            assert np.array_equal(hq, out[1].cpu().numpy())
