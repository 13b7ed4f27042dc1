"""Multi-rank bench logic on CPU (gloo, world size 2): disjoint shards, max-time
and summed-knots aggregation.  No GPU and no data-path collective."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "fast-rbd-gradients_gb300"))
    import torch.distributed as dist
    from frg import dist as fdist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    h, off, n, q, qd, u = fdist.rank_mix(rank, 64, 8, 256, seed=2021)
    local_ms = 10.0 * (rank + 1)  # rank 1 is the slow one
    value, tmax, ktot = fdist.aggregate(local_ms, n, steps=3)
    out[rank] = (n, fdist.knot_checksum(q), value, tmax, ktot)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_and_aggregate():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    (n0, c0, v0, t0, k0), (n1, c1, v1, t1, k1) = res[0], res[1]
    assert c0 != c1  # different knots on each rank
    assert t0 == t1 == 20.0  # max over ranks
    assert k0 == k1 == n0 + n1  # knots of all ranks
    assert v0 == pytest.approx((n0 + n1) * 3 / 0.020)
