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
