"""Seeded synthetic inputs (CPU)."""
import numpy as np

import frg


def test_sample_knots_deterministic_and_in_range():
    a = frg.sample_knots(1000, seed=1)
    b = frg.sample_knots(1000, seed=1)
    for x, y in zip(a, b):
        assert x.dtype == np.float32 and x.shape == (1000, 7) and x.flags.c_contiguous
        assert np.array_equal(x, y)
    q, qd, u = a
    assert (np.abs(q) <= frg.JOINT_LIMITS.astype(np.float32)).all()
    assert np.abs(qd).max() <= 2 and np.abs(u).max() <= 20
    assert np.abs(q).max(axis=0).min() > 1.5  # covers the range


def test_ragged_horizons():
    h, off = frg.ragged_horizons(512, 8, 256, seed=2021)
    assert h.min() >= 8 and h.max() <= 256 and len(off) == 513
    assert off[0] == 0 and (np.diff(off) == h).all()
