"""The allocation-free batched entry point (frg_gradient_ragged_noalloc).

Some callers cannot allocate device memory once they run: a real-time MPC
loop, where cudaFree synchronizes the whole device and cudaMalloc can block
for an unbounded time inside a control period, or a plug-in inside a host
application that owns every byte of device memory and only lends it input and
output buffers.  This entry point keeps its launch descriptors and work
counter in a fixed array compiled into the library instead of allocating them.

Checked through the C ABI:
- two calls in a row, a large batch and then a small one on the same stream
  with no host synchronisation between them, give exactly the bits of the
  regular batched call (frg_gradient_ragged), and are within the parity bar of
  the FP64 oracle, in all four damping / gravity modes;
- the same after the autotuner has chosen the context's launch shapes, and
  with the latency mapping (8 lanes per knot);
- batches beyond the fixed limits are refused with a clear error.

This file is collected last, and passes alone in a fresh process as well as
after the other tests.
"""
import ctypes

import numpy as np
import pytest

import frg
from conftest import TOL, max_err
from frg import native

pytestmark = pytest.mark.gpu

MODES = [(0, 0), (1, 0), (0, 1), (1, 1)]


def _call(ctx, off, arrays, stream=None):
    off = np.ascontiguousarray(off, dtype=np.int64)
    return native.lib().frg_gradient_ragged_noalloc(
        ctx.handle, len(off) - 1, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
        *[a.data_ptr() for a in arrays], stream)


def _case(torch, n_traj, seed):
    h, off = frg.ragged_horizons(n_traj, 1, 256, seed=seed)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(n, seed=seed + 1)
    ins = [torch.from_numpy(x).cuda() for x in (q, qd, u)]
    return off, n, (q, qd, u), ins


def _outs(torch, n):
    return [torch.full((n, w), float("nan"), device="cuda") for w in (98, 7, 49)]


def _check_two_calls(torch, ctx, damping, mpc, seeds=(71, 72), sizes=(300, 41)):
    """A large then a small call back to back on one stream (no host sync):
    each bitwise equal to frg_gradient_ragged and within TOL of the oracle."""
    import frg_oracle
    cases = [_case(torch, n_traj, seed) for n_traj, seed in zip(sizes, seeds)]
    got = [_outs(torch, c[1]) for c in cases]
    for (off, n, _, ins), outs in zip(cases, got):
        assert _call(ctx, off, ins + outs) == 0, ctx.last_error()
    torch.cuda.synchronize()
    for call, ((off, n, host_in, ins), outs) in enumerate(zip(cases, got)):
        want = _outs(torch, n)
        ctx.ragged(off, *ins, *want)
        torch.cuda.synchronize()
        a = [x.cpu().numpy() for x in outs]
        b = [x.cpu().numpy() for x in want]
        for name, x, y in zip(("dqdd", "qdd", "minv"), a, b):
            assert np.isfinite(x).all(), f"call {call}: {name} not written"
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), f"call {call}: {name} bits differ"
        ref = frg_oracle.gradient_f64(*host_in, damping=bool(damping), mpc=bool(mpc))
        for name, x, r in zip(("dqdd", "qdd", "minv"), a, ref):
            assert max_err(x, r) <= TOL, f"call {call}: {name} vs FP64 oracle"


@pytest.mark.parametrize("damping,mpc", MODES)
def test_noalloc_matches_regular_batched_call_twice(damping, mpc):
    import torch
    with frg.Context(vel_damping=bool(damping), mpc_mode=bool(mpc)) as ctx:
        _check_two_calls(torch, ctx, damping, mpc)


def test_noalloc_after_autotune_and_in_the_latency_mapping():
    import torch
    with frg.Context() as ctx:
        ctx.autotune(1 << 14)
        _check_two_calls(torch, ctx, 0, 0, seeds=(81, 82))
        ctx.set_lanes_per_knot(8)
        _check_two_calls(torch, ctx, 0, 0, seeds=(83, 84), sizes=(64, 3))


def test_noalloc_refuses_batches_beyond_its_limits():
    import torch
    with frg.Context() as ctx:
        x = torch.zeros(8, device="cuda")
        too_many = np.arange(4098, dtype=np.int64)  # 4097 trajectories of 1 knot each
        st = _call(ctx, too_many, [x] * 6)
        assert st == 1 and "FRG_NOALLOC_MAX_TRAJ" in ctx.last_error()
        too_big = np.array([0, 65536 * 32 + 1], dtype=np.int64)
        st = _call(ctx, too_big, [x] * 6)
        assert st == 1 and "FRG_NOALLOC_MAX_KNOTS" in ctx.last_error()
