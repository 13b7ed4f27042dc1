"""Host-buffer batches in one call (frg_gradient_host_batches, GPU): with two
launches in flight on two streams, every batch's results are exactly those of
frg_gradient_host on the same knots, for pinned and for pageable arrays."""
import ctypes

import numpy as np
import pytest

import frg
from frg import native

pytestmark = pytest.mark.gpu


def _pinned(shape):
    n = int(np.prod(shape))
    ptr = native.lib().frg_host_alloc(4 * n)
    assert ptr
    return ptr, np.ctypeslib.as_array((ctypes.c_float * n).from_address(ptr)).reshape(shape)


@pytest.mark.parametrize("pinned", [True, False])
def test_batches_match_single_calls_bitwise(pinned):
    sizes = [700, 33, 4097, 1, 2500, 64]
    data = [frg.sample_knots(n, seed=60 + i) for i, n in enumerate(sizes)]
    owned = []
    batches, outs = [], []
    for (q, qd, u), n in zip(data, sizes):
        arrs = []
        for x in (q, qd, u):
            if pinned:
                p, a = _pinned(x.shape)
                owned.append(p)
                a[:] = x
                arrs.append(a)
            else:
                arrs.append(x)
        o = []
        for w in (98, 7, 49):
            if pinned:
                p, a = _pinned((n, w))
                owned.append(p)
                a[:] = np.nan
                o.append(a)
            else:
                o.append(np.full((n, w), np.nan, np.float32))
        batches.append((n, *arrs, *o))
        outs.append(o)
    try:
        with frg.Context() as ctx:
            ctx.gradient_host_batches(batches)
            for (q, qd, u), o in zip(data, outs):
                want = ctx.gradient_host(q, qd, u)
                for a, b in zip(o, want):
                    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    finally:
        for p in owned:
            native.lib().frg_host_free(p)


def test_batches_reject_null_arrays():
    with frg.Context() as ctx:
        with pytest.raises(frg.FrgError):
            ctx.gradient_host_batches([(10, None, None, None, None, None, None)])
        ctx.gradient_host_batches([])  # nothing to do


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("lanes", [1, 8])
def test_results_not_asked_for_are_not_returned(pinned, lanes):
    """qdd and/or minv NULL: dqdd (and the other result asked for) carry the
    bits of the full call, in single calls and in batches."""
    sizes = [900, 31, 2049, 5]
    keep = [(True, False), (False, True), (False, False), (True, True)]  # (qdd, minv)
    data = [frg.sample_knots(n, seed=80 + i) for i, n in enumerate(sizes)]
    owned = []

    def arr(shape, fill=None):
        if pinned:
            p, a = _pinned(shape)
            owned.append(p)
        else:
            a = np.empty(shape, np.float32)
        if fill is not None:
            a[:] = fill
        return a

    try:
        with frg.Context() as ctx:
            ctx.set_lanes_per_knot(lanes)
            want = [ctx.gradient_host(q, qd, u) for q, qd, u in data]
            batches, outs = [], []
            for (q, qd, u), n, (kq, km) in zip(data, sizes, keep):
                ins = [arr(x.shape, x) for x in (q, qd, u)]
                o = [arr((n, 98), np.nan), arr((n, 7), np.nan) if kq else None, arr((n, 49), np.nan) if km else None]
                batches.append((n, *ins, *o))
                outs.append(o)
            ctx.gradient_host_batches(batches)
            for o, w in zip(outs, want):
                for a, b in zip(o, w):
                    if a is not None:
                        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
            for (n, *ins, _, _, _), (kq, km), w in zip(batches, keep, want):
                o = [arr((n, 98), np.nan), arr((n, 7), np.nan) if kq else None, arr((n, 49), np.nan) if km else None]
                ctx.gradient_host_into(n, *ins, *o)
                for a, b in zip(o, w):
                    if a is not None:
                        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
            d, qdd, minv = ctx.gradient_host(*data[0], want_qdd=False, want_minv=False)
            assert qdd is None and minv is None
            assert np.array_equal(d.view(np.uint32), want[0][0].view(np.uint32))
            with pytest.raises(frg.FrgError):  # dqdd is always returned
                ctx.gradient_host_into(5, *data[3], None, None, None)
    finally:
        for p in owned:
            native.lib().frg_host_free(p)


@pytest.mark.parametrize("lanes", [1, 8])
def test_packed_minv_batches_match_single_calls_bitwise(lanes):
    """Every batch returns Minv: with one lane per knot the call sends Minv's
    upper triangle and expands it on the host (some batches without q̈, so
    q̈ also goes to the relay's tail); the dense results carry the single
    call's bits, Minv exactly symmetric."""
    sizes = [3000, 64, 1, 4097, 777]
    data = [frg.sample_knots(n, seed=120 + i) for i, n in enumerate(sizes)]
    owned = []
    try:
        with frg.Context() as ctx:
            ctx.set_lanes_per_knot(lanes)
            want = [ctx.gradient_host(q, qd, u) for q, qd, u in data]
            batches, outs = [], []
            for i, ((q, qd, u), n) in enumerate(zip(data, sizes)):
                ins = []
                for x in (q, qd, u):
                    p, a = _pinned(x.shape)
                    owned.append(p)
                    a[:] = x
                    ins.append(a)
                o = []
                for w, keep in ((98, True), (7, i % 2 == 0), (49, True)):
                    if keep:
                        p, a = _pinned((n, w))
                        owned.append(p)
                        a[:] = np.nan
                        o.append(a)
                    else:
                        o.append(None)
                batches.append((n, *ins, *o))
                outs.append(o)
            for _ in range(2):  # the second call reuses the staging buffers and expansion threads
                ctx.gradient_host_batches(batches)
                for o, w in zip(outs, want):
                    for a, b in zip(o, w):
                        if a is not None:
                            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
                    m = o[2].reshape(-1, 7, 7)
                    assert np.array_equal(m, m.transpose(0, 2, 1))
    finally:
        for p in owned:
            native.lib().frg_host_free(p)


@pytest.mark.parametrize("want_qdd", [True, False])
def test_large_single_call_matches_device_launch_bitwise(want_qdd):
    """A single frg_gradient_host of 70,000 knots on pinned arrays (results
    streamed from the kernel as tiles finish) equals a device-array launch
    bitwise."""
    import torch
    n = 70000
    q, qd, u = frg.sample_knots(n, seed=321)
    owned = []
    try:
        ins = []
        for x in (q, qd, u):
            p, a = _pinned(x.shape)
            owned.append(p)
            a[:] = x
            ins.append(a)
        outs = []
        for w, keep in ((98, True), (7, want_qdd), (49, True)):
            if keep:
                p, a = _pinned((n, w))
                owned.append(p)
                a[:] = np.nan
                outs.append(a)
            else:
                outs.append(None)
        with frg.Context() as ctx:
            ctx.gradient_host_into(n, *ins, *outs)
            tq, tqd, tu = (torch.from_numpy(x).cuda() for x in (q, qd, u))
            dev = [torch.empty((n, w), device="cuda") for w in (98, 7, 49)]
            ctx.gradient(n, tq, tqd, tu, *dev)
            torch.cuda.synchronize()
        for a, b in zip(outs, dev):
            if a is not None:
                assert np.array_equal(a.view(np.uint32), b.cpu().numpy().view(np.uint32))
    finally:
        for p in owned:
            native.lib().frg_host_free(p)
