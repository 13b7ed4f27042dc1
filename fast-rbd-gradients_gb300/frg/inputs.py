"""Seeded synthetic knot points with the benchmark distributions.

q_i ~ U(-lim_i, +lim_i) with the joint limits of utils/iiwa_14.urdf
(iiwa_joint_1..7 <limit>, lines 28, 44, 60, 76, 92, 108, 126), qd ~ U(-2, 2)
rad/s, u ~ U(-20, 20) N*m, all stored as float32.  numpy's PCG64 stream is the
generator, so every machine draws the same knots for the same seed.
"""
import numpy as np

NUM_JOINTS = 7

JOINT_LIMITS = np.array(
    [2.96705972839, 2.09439510239, 2.96705972839, 2.09439510239, 2.96705972839, 2.09439510239, 3.05432619099],
    dtype=np.float64,
)


def sample_knots(n, seed):
    """n knots (q, qd, u), each float32 [n, 7], C-contiguous."""
    rng = np.random.Generator(np.random.PCG64(seed))
    q = rng.uniform(-1.0, 1.0, (n, NUM_JOINTS)) * JOINT_LIMITS
    qd = rng.uniform(-2.0, 2.0, (n, NUM_JOINTS))
    u = rng.uniform(-20.0, 20.0, (n, NUM_JOINTS))
    return tuple(np.ascontiguousarray(x, dtype=np.float32) for x in (q, qd, u))


def ragged_horizons(n_traj, lo, hi, seed):
    """Trajectory horizons ~ U{lo..hi} (inclusive) and their prefix offsets
    (int64 [n_traj + 1], offsets[0] = 0)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = rng.integers(lo, hi + 1, size=n_traj).astype(np.int64)
    off = np.zeros(n_traj + 1, np.int64)
    np.cumsum(h, out=off[1:])
    return h, off


def perturb(x, sigma, seed):
    """x + N(0, sigma) noise (float32), for iLQR / line-search style re-calls."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.ascontiguousarray(x + rng.normal(0.0, sigma, x.shape), dtype=np.float32)
