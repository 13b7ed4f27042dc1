"""CUDA path vs the oracle and the reference's golden outputs (GPU).

Bar: max Frobenius-relative error per output matrix (dqdd 7x14, qdd, Minv)
and knot <= 1e-4 against FP64 (the reference's own FP64 outputs in
tests/golden, and the FP64 oracle), and the same against the reference's
FP32 outputs."""
import numpy as np
import pytest

import frg
import frg_oracle
from conftest import TOL, max_err

pytestmark = pytest.mark.gpu
MODES = [(d, m) for d in (0, 1) for m in (0, 1)]


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


@pytest.mark.parametrize("damping,mpc", MODES)
def test_golden_all_modes(golden, damping, mpc):
    with frg.Context(vel_damping=damping, mpc_mode=mpc) as ctx:
        d, q, m = ctx.gradient_host(golden["q"], golden["qd"], golden["u"])
    tag = f"f64_d{damping}_m{mpc}"
    assert max_err(d, golden[f"dqdd_{tag}"]) <= TOL
    assert max_err(q, golden[f"qdd_{tag}"]) <= TOL
    assert max_err(m, golden[f"minv_{tag}"]) <= TOL


def test_golden_against_reference_fp32(golden):
    with frg.Context() as ctx:
        d, q, m = ctx.gradient_host(golden["q"], golden["qd"], golden["u"])
    assert max_err(d, golden["dqdd_f32_d0_m0"]) <= TOL
    assert max_err(q, golden["qdd_f32_d0_m0"]) <= TOL
    assert max_err(m, golden["minv_f32_d0_m0"]) <= TOL


@pytest.mark.parametrize("n", [1, 7, 31, 32, 33, 95, 1000, 4097])
def test_oracle_parity_sizes(n):
    q, qd, u = frg.sample_knots(n, seed=1000 + n)
    with frg.Context() as ctx:
        d, qq, m = ctx.gradient_host(q, qd, u)
    rd, rq, rm = frg_oracle.gradient_f64(q, qd, u)
    assert max_err(d, rd) <= TOL and max_err(qq, rq) <= TOL and max_err(m, rm) <= TOL


def test_device_path_equals_host_path(torch_cuda):
    torch = torch_cuda
    q, qd, u = frg.sample_knots(777, seed=11)
    with frg.Context() as ctx:
        hd, hq, hm = ctx.gradient_host(q, qd, u)
        tq, tqd, tu = (torch.from_numpy(x).cuda() for x in (q, qd, u))
        dd, dq, dm = frg.forward_dynamics_gradient(tq, tqd, tu, ctx=ctx)
        torch.cuda.synchronize()
    assert np.array_equal(dd.cpu().numpy(), hd)
    assert np.array_equal(dq.cpu().numpy(), hq)
    assert np.array_equal(dm.cpu().numpy(), hm)


def test_zero_knots_is_noop():
    with frg.Context() as ctx:
        ctx.gradient(0, 0, 0, 0, 0, 0, 0)
        ctx.gradient_host_into(0, None, None, None, None, None, None)


def test_negative_knots_rejected():
    with frg.Context() as ctx:
        with pytest.raises(frg.FrgError) as ei:
            ctx.gradient(-1, 0, 0, 0, 0, 0, 0)
        assert ei.value.status == 1


@pytest.mark.parametrize("shape", [(1, 1), (2, 4), (3, 3), (4, 2), (8, 1)])
def test_launch_shapes_bitwise_identical(shape):
    q, qd, u = frg.sample_knots(1500, seed=21)
    with frg.Context() as ctx:
        base = ctx.gradient_host(q, qd, u)
        ctx.set_launch_shape(*shape)
        other = ctx.gradient_host(q, qd, u)
    for a, b in zip(base, other):
        assert np.array_equal(a, b)


def test_full_size_properties(torch_cuda):
    """N = 65536 (largest plain config): outputs finite, Minv exactly
    symmetric and positive definite, and a strided sample within TOL of the
    FP64 oracle."""
    torch = torch_cuda
    n = 65536
    q, qd, u = frg.sample_knots(n, seed=65536)
    with frg.Context() as ctx:
        tq, tqd, tu = (torch.from_numpy(x).cuda() for x in (q, qd, u))
        d, qq, m = frg.forward_dynamics_gradient(tq, tqd, tu, ctx=ctx)
        torch.cuda.synchronize()
    d, qq, m = d.cpu().numpy(), qq.cpu().numpy(), m.cpu().numpy()
    assert np.isfinite(d).all() and np.isfinite(qq).all() and np.isfinite(m).all()
    M = m.reshape(-1, 7, 7)
    assert np.array_equal(M, M.transpose(0, 2, 1))
    idx = np.arange(0, n, 97)
    assert (np.linalg.eigvalsh(M[idx].astype(np.float64)) > 0).all()
    rd, rq, rm = frg_oracle.gradient_f64(q[idx], qd[idx], u[idx])
    assert max_err(d[idx], rd) <= TOL and max_err(qq[idx], rq) <= TOL and max_err(m[idx], rm) <= TOL


def test_nonfinite_input_stays_in_its_knot():
    q, qd, u = frg.sample_knots(64, seed=4)
    q = q.copy()
    q[5, 3] = np.nan
    with frg.Context() as ctx:
        d, qq, m = ctx.gradient_host(q, qd, u)
    bad = ~np.isfinite(d).all(axis=1)
    assert bad[5] and bad.sum() == 1
    keep = np.arange(64) != 5
    rd, _, _ = frg_oracle.gradient_f64(q[keep], qd[keep], u[keep])
    assert max_err(d[keep], rd) <= TOL


@pytest.mark.parametrize("damping,mpc", MODES)
@pytest.mark.parametrize("n", [1, 5, 37, 1000])
def test_latency_mapping_parity(golden, damping, mpc, n):
    """8 lanes per knot (latency mapping): same results as the throughput
    mapping and within TOL of the FP64 oracle."""
    q, qd, u = frg.sample_knots(n, seed=70 + n)
    with frg.Context(vel_damping=damping, mpc_mode=mpc) as ctx:
        a = ctx.gradient_host(q, qd, u)
        ctx.set_lanes_per_knot(8)
        assert ctx.lanes_per_knot() == 8
        b = ctx.gradient_host(q, qd, u)
        g = ctx.gradient_host(golden["q"], golden["qd"], golden["u"])
    rd, rq, rm = frg_oracle.gradient_f64(q, qd, u, damping, mpc)
    assert max_err(b[0], rd) <= TOL and max_err(b[1], rq) <= TOL and max_err(b[2], rm) <= TOL
    for x, y in zip(a, b):
        assert max_err(x, y) <= 1e-5
    tag = f"f64_d{damping}_m{mpc}"
    assert max_err(g[0], golden[f"dqdd_{tag}"]) <= TOL and max_err(g[2], golden[f"minv_{tag}"]) <= TOL


@pytest.mark.parametrize("n,lanes,offset", [(1, 1, 0), (31, 1, 0), (3000, 1, 0), (70001, 1, 0), (3000, 1, 1),
                                             (3000, 8, 0), (45, 8, 1)])
def test_host_call_pinned_zero_copy_equals_staged(n, lanes, offset):
    """frg_gradient_host on pinned buffers (the kernel reads inputs from host
    memory and writes results there, dqdd relayed through device memory as
    whole tiles) gives the same bits as on pageable buffers (staged copies):
    whole and partial tiles, both thread mappings, and host arrays that start
    one float off 16-byte alignment (the relay's element-wise branch)."""
    import ctypes
    q, qd, u = frg.sample_knots(n, seed=31 + n)
    L = frg.lib()
    bufs = {}
    for name, w in (("q", 7), ("qd", 7), ("u", 7), ("dqdd", 98), ("qdd", 7), ("minv", 49)):
        ptr = L.frg_host_alloc(4 * (w * n + offset))
        assert ptr
        addr = ptr + 4 * offset
        arr = np.ctypeslib.as_array((ctypes.c_float * (w * n)).from_address(addr)).reshape(n, w)
        bufs[name] = (ptr, addr, arr)
    try:
        bufs["q"][2][:], bufs["qd"][2][:], bufs["u"][2][:] = q, qd, u
        for k in ("dqdd", "qdd", "minv"):
            bufs[k][2][:] = np.nan
        with frg.Context() as ctx:
            ctx.set_lanes_per_knot(lanes)
            staged = ctx.gradient_host(q, qd, u)
            ctx.gradient_host_into(n, *(bufs[k][1] for k in ("q", "qd", "u", "dqdd", "qdd", "minv")))
        for name, ref in zip(("dqdd", "qdd", "minv"), staged):
            assert np.array_equal(bufs[name][2], ref), name
    finally:
        for ptr, _, _ in bufs.values():
            L.frg_host_free(ptr)


@pytest.mark.parametrize("damping,mpc", MODES)
def test_thread_mappings_give_identical_bits(damping, mpc):
    """Both thread mappings perform the same operations in the same order for
    every knot (the latency mapping only spreads the columns over lanes), so
    their results agree bit for bit, here on 20,000 knots."""
    n = 20000
    q, qd, u = frg.sample_knots(n, seed=500 + 2 * damping + mpc)
    with frg.Context(vel_damping=damping, mpc_mode=mpc) as ctx:
        ctx.set_lanes_per_knot(1)
        a = ctx.gradient_host(q, qd, u)
        ctx.set_lanes_per_knot(8)
        b = ctx.gradient_host(q, qd, u)
    for name, x, y in zip(("dqdd", "qdd", "minv"), a, b):
        diff = np.count_nonzero(x != y)
        assert diff == 0, f"{name}: {diff} values differ, max {max_err(x, y):.2e}"


@pytest.mark.parametrize("lanes", [1, 8])
@pytest.mark.parametrize("offsets", [(-60.0, -7.0, -3.5, 3.5, 7.0, 60.0), (-1000.0, -200.0, 200.0, 1000.0)])
def test_angles_beyond_pi_and_large_inputs(lanes, offsets):
    """Joint angles outside [-pi, pi] (up to +-1000 rad, a continuous joint
    after many turns: the range-reduced sincos path of the FP32 kernels), and
    velocities and torques ten times the experiment ranges, against the FP64
    oracle on the same FP32 inputs."""
    n = 2048
    q, qd, u = frg.sample_knots(n, seed=314)
    rng = np.random.default_rng(15)
    q = (q + rng.choice(offsets, size=q.shape)).astype(np.float32)
    qd = (qd * 10).astype(np.float32)
    u = (u * 10).astype(np.float32)
    with frg.Context() as ctx:
        ctx.set_lanes_per_knot(lanes)
        d, qq, m = ctx.gradient_host(q, qd, u)
    rd, rq, rm = frg_oracle.gradient_f64(q, qd, u)
    assert max_err(d, rd) <= TOL and max_err(qq, rq) <= TOL and max_err(m, rm) <= TOL
    assert np.isfinite(d).all()
