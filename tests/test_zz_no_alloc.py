"""The allocation-free batched entry point (frg_gradient_ragged_noalloc).

It serves callers that cannot allocate device memory once they run: a
real-time MPC loop (cudaFree synchronizes the device, cudaMalloc may block) or
a plug-in inside an application that owns all device memory.  Its scratch is a
fixed array compiled into the library, so the test checks, through the C ABI,
that two calls in a row give the results of the regular batched call
(frg_gradient_ragged) within the parity tolerance, and that batches beyond the
fixed limits are refused with a clear error.  This file is collected last, and
passes alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

import frg
from conftest import TOL, max_err
from frg import native

pytestmark = pytest.mark.gpu


def _call(ctx, off, arrays):
    off = np.ascontiguousarray(off, dtype=np.int64)
    return native.lib().frg_gradient_ragged_noalloc(
        ctx.handle, len(off) - 1, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
        *[a.data_ptr() for a in arrays], None)


def _case(torch, n_traj, seed):
    h, off = frg.ragged_horizons(n_traj, 1, 256, seed=seed)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(n, seed=seed + 1)
    ins = [torch.from_numpy(x).cuda() for x in (q, qd, u)]
    return off, n, ins


def _outs(torch, n):
    return [torch.full((n, w), float("nan"), device="cuda") for w in (98, 7, 49)]


def test_noalloc_matches_regular_batched_call_twice():
    import torch
    with frg.Context() as ctx:
        for call, (n_traj, seed) in enumerate(((300, 71), (41, 72))):
            off, n, ins = _case(torch, n_traj, seed)
            got = _outs(torch, n)
            assert _call(ctx, off, ins + got) == 0, ctx.last_error()
            want = _outs(torch, n)
            ctx.ragged(off, *ins, *want)
            torch.cuda.synchronize()
            for a, b in zip(got, want):
                a, b = a.cpu().numpy(), b.cpu().numpy()
                assert np.isfinite(a).all(), f"call {call}: unwritten output"
                assert max_err(a, b) <= TOL


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
