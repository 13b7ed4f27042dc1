"""Sharding across GPUs: the path has no exchange step (knots and trajectories
are independent), so every rank computes its own ragged mix and the only
collectives are the timing barrier and the aggregation of the result."""
import numpy as np

from .inputs import ragged_horizons, sample_knots


def rank_mix(rank, n_traj, lo, hi, seed):
    """The ragged mix of one rank (weak scaling): horizons, offsets, q, qd, u.
    Ranks draw from disjoint seeds, so no two ranks compute the same knots."""
    h, off = ragged_horizons(n_traj, lo, hi, seed=seed + rank)
    n = int(off[-1])
    q, qd, u = sample_knots(n, seed=seed * 7 + rank)
    return h, off, n, q, qd, u


def aggregate(local_ms, local_knots, steps, device=None):
    """Whole-job throughput: (sum of knots over ranks) * steps / (max time over
    ranks).  Uses torch.distributed when initialised, else the local values."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return local_knots * steps / (local_ms * 1e-3), local_ms, local_knots
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    k = torch.tensor([float(local_knots)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(k, op=dist.ReduceOp.SUM)
    return float(k.item()) * steps / (float(t.item()) * 1e-3), float(t.item()), int(k.item())


def knot_checksum(q):
    """Order-independent fingerprint of a rank's knots (to show shards differ)."""
    return float(np.float64(q.astype(np.float64).sum()))
