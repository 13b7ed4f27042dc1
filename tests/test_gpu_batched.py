"""Batched (persistent, ragged) and per-trajectory forms, plans / CUDA graphs
(GPU).  Every knot's result must not depend on what it is batched with."""
import numpy as np
import pytest

import frg
import frg_oracle
from conftest import TOL, max_err

pytestmark = pytest.mark.gpu


def alloc(torch, n):
    return (torch.empty((n, 98), device="cuda"), torch.empty((n, 7), device="cuda"), torch.empty((n, 49), device="cuda"))


def test_ragged_mix_matches_plain_bitwise():
    import torch
    h, off = frg.ragged_horizons(512, 8, 256, seed=2021)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(n, seed=17)
    tq, tqd, tu = (torch.from_numpy(x).cuda() for x in (q, qd, u))
    with frg.Context() as ctx:
        plain = alloc(torch, n)
        ctx.gradient(n, tq, tqd, tu, *plain)
        rag = alloc(torch, n)
        ctx.ragged(off, tq, tqd, tu, *rag)
        per = alloc(torch, n)
        trajs = [(int(off[t + 1] - off[t]), tq[off[t]:], tqd[off[t]:], tu[off[t]:], per[0][off[t]:], per[1][off[t]:],
                  per[2][off[t]:]) for t in range(512)]
        ctx.per_trajectory(trajs)
        torch.cuda.synchronize()
    for a, b, c in zip(plain, rag, per):
        assert torch.equal(a, b) and torch.equal(a, c)
    idx = np.arange(0, n, 53)
    rd, rq, rm = frg_oracle.gradient_f64(q[idx], qd[idx], u[idx])
    assert max_err(rag[0].cpu().numpy()[idx], rd) <= TOL
    assert max_err(rag[1].cpu().numpy()[idx], rq) <= TOL
    assert max_err(rag[2].cpu().numpy()[idx], rm) <= TOL


@pytest.mark.parametrize("horizons", [[1], [7], [8], [255], [256], [0, 5, 0, 33, 0], [1] * 70, [31, 1, 32, 33, 64, 2]])
def test_edge_horizons(horizons):
    import torch
    off = np.concatenate([[0], np.cumsum(horizons)]).astype(np.int64)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(max(n, 1), seed=len(horizons) + n)
    tq, tqd, tu = (torch.from_numpy(x).cuda() for x in (q, qd, u))
    with frg.Context() as ctx:
        out = alloc(torch, max(n, 1))
        ctx.ragged(off, tq, tqd, tu, *out)
        torch.cuda.synchronize()
    if n:
        rd, rq, rm = frg_oracle.gradient_f64(q[:n], qd[:n], u[:n])
        assert max_err(out[0].cpu().numpy()[:n], rd) <= TOL
        assert max_err(out[1].cpu().numpy()[:n], rq) <= TOL
        assert max_err(out[2].cpu().numpy()[:n], rm) <= TOL


@pytest.mark.parametrize("damping,mpc", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_full_mix_every_knot_vs_oracle(damping, mpc):
    """The benchmark's workload, every knot: the 512-trajectory mix (seed 2021,
    66,809 knots) stored in shuffled order, so a plan runs the persistent
    kernel over scattered trajectories; all of dqdd, q̈ and Minv of every knot
    against the FP64 CPU oracle."""
    import torch
    h, off = frg.ragged_horizons(512, 8, 256, seed=2021)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(n, seed=2022)
    perm = np.random.Generator(np.random.PCG64(2021)).permutation(512)
    mem_off = np.zeros(512, np.int64)
    pos = 0
    for t in perm:
        mem_off[t] = pos
        pos += int(h[t])
    # knot k of trajectory t sits at memory row mem_off[t] + k
    rows = np.concatenate([mem_off[t] + np.arange(h[t]) for t in range(512)])
    tq, tqd, tu = (torch.from_numpy(np.ascontiguousarray(x[np.argsort(rows)])).cuda() for x in (q, qd, u))
    out = [torch.full((n, w), float("nan"), device="cuda") for w in (98, 7, 49)]
    with frg.Context(vel_damping=bool(damping), mpc_mode=bool(mpc)) as ctx:
        o = [int(x) for x in mem_off]
        trajs = [(int(h[t]), tq[o[t]:], tqd[o[t]:], tu[o[t]:], out[0][o[t]:], out[1][o[t]:], out[2][o[t]:])
                 for t in range(512)]
        plan = ctx.plan(trajs)
        try:
            plan.launch()
            torch.cuda.synchronize()
        finally:
            plan.close()
    got = [x.cpu().numpy()[rows] for x in out]  # back to trajectory order
    ref = frg_oracle.gradient_f64(q, qd, u, damping=bool(damping), mpc=bool(mpc))
    for name, a, r in zip(("dqdd", "qdd", "minv"), got, ref):
        assert np.isfinite(a).all(), f"{name}: unwritten knots"
        assert max_err(a, r) <= TOL, name


def test_scattered_trajectories_alone_and_in_mix():
    """Trajectories in separate buffers: each one's result alone equals its
    result inside a 40-trajectory batch, bit for bit."""
    import torch
    rng = np.random.default_rng(8)
    hs = rng.integers(1, 200, size=40)
    bufs = []
    for i, hh in enumerate(hs):
        q, qd, u = frg.sample_knots(int(hh), seed=300 + i)
        bufs.append([int(hh)] + [torch.from_numpy(x).cuda() for x in (q, qd, u)] + list(alloc(torch, int(hh))))
    with frg.Context() as ctx:
        ctx.batched([tuple(b) for b in bufs])
        torch.cuda.synchronize()
        mixed = [[t.clone() for t in b[4:]] for b in bufs]
        for b in bufs:
            for t in b[4:]:
                t.zero_()
            ctx.batched([tuple(b)])
        torch.cuda.synchronize()
    for b, m in zip(bufs, mixed):
        for alone, mix in zip(b[4:], m):
            assert torch.equal(alone, mix)


def test_gaps_between_trajectories_stay_untouched():
    """Trajectories packed into shared buffers with gaps of 0..40 knots between
    them (tiles that mix up to many trajectories, and ones with idle lanes):
    the batched and plan results equal the plain kernel's bit for bit, and no
    value in a gap changes."""
    import torch
    rng = np.random.default_rng(31)
    hs = np.concatenate([rng.integers(1, 12, 60), rng.integers(1, 90, 90)])
    gaps = rng.integers(0, 41, hs.size)
    starts = np.concatenate([[0], np.cumsum(hs + gaps)[:-1]])
    total = int(starts[-1] + hs[-1] + gaps[-1])
    n = int(hs.sum())
    q, qd, u = frg.sample_knots(n, seed=77)
    packed = [np.full((total, 7), 3.0, np.float32) for _ in range(3)]
    for t, (s, hh) in enumerate(zip(starts, hs)):
        a = int(hs[:t].sum())
        for dst, src in zip(packed, (q, qd, u)):
            dst[s:s + hh] = src[a:a + hh]
    tq, tqd, tu = (torch.from_numpy(x).cuda() for x in packed)
    sentinel = -7.25
    with frg.Context() as ctx:
        ref = alloc(torch, n)
        ctx.gradient(n, *(torch.from_numpy(x).cuda() for x in (q, qd, u)), *ref)
        for form in ("batched", "plan"):
            out = [torch.full((total, w), sentinel, device="cuda") for w in (98, 7, 49)]
            trajs = [(int(hh), tq[s:], tqd[s:], tu[s:], out[0][s:], out[1][s:], out[2][s:])
                     for s, hh in zip(starts, hs)]
            if form == "batched":
                ctx.batched(trajs)
            else:
                plan = ctx.plan(trajs)
                try:
                    plan.launch()
                    torch.cuda.synchronize()
                finally:
                    plan.close()
            torch.cuda.synchronize()
            live = torch.zeros(total, dtype=torch.bool, device="cuda")
            for s, hh in zip(starts, hs):
                live[s:s + hh] = True
            for o, r in zip(out, ref):
                assert torch.equal(o[live], r), form
                assert bool((o[~live] == sentinel).all()), form


def test_plan_graph_replay_tracks_input_changes():
    import torch
    h, off = frg.ragged_horizons(64, 8, 256, seed=5)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(n, seed=6)
    tq, tqd, tu = (torch.from_numpy(x).cuda() for x in (q, qd, u))
    with frg.Context() as ctx:
        out = alloc(torch, n)
        plan = ctx.plan_ragged(off, tq, tqd, tu, *out)
        assert plan.knots == n
        for rep in range(3):
            plan.launch()
        torch.cuda.synchronize()
        first = [t.clone() for t in out]
        q2 = frg.perturb(q, 1e-2, seed=9)
        tq.copy_(torch.from_numpy(q2))
        plan.launch()
        torch.cuda.synchronize()
        rd, rq, rm = frg_oracle.gradient_f64(q2, qd, u)
        assert max_err(out[0].cpu().numpy(), rd) <= TOL
        tq.copy_(torch.from_numpy(q))
        plan.launch()
        torch.cuda.synchronize()
        for a, b in zip(first, out):
            assert torch.equal(a, b)
        plan.close()


def test_autotune_picks_a_valid_shape():
    with frg.Context() as ctx:
        kps = ctx.autotune(32768)
        w, c = ctx.launch_shape()
    assert kps > 0 and 1 <= w <= 8 and c >= 1


def test_latency_mapping_ragged_and_plan():
    import torch
    h, off = frg.ragged_horizons(100, 1, 64, seed=12)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(n, seed=13)
    tq, tqd, tu = (torch.from_numpy(x).cuda() for x in (q, qd, u))
    with frg.Context(lanes_per_knot=8) as ctx:
        out = alloc(torch, n)
        ctx.ragged(off, tq, tqd, tu, *out)
        out2 = alloc(torch, n)
        plan = ctx.plan_ragged(off, tq, tqd, tu, *out2)
        plan.launch()
        plan.launch()
        torch.cuda.synchronize()
        plan.close()
    rd, rq, rm = frg_oracle.gradient_f64(q, qd, u)
    for o in (out, out2):
        assert max_err(o[0].cpu().numpy(), rd) <= TOL
        assert max_err(o[1].cpu().numpy(), rq) <= TOL
        assert max_err(o[2].cpu().numpy(), rm) <= TOL


def test_back_to_back_launches_keep_stream_order():
    """Launches start early (programmatic dependent launch) but wait for the
    work before them: a launch whose joint angles are the previous launch's q̈
    output, issued with no synchronisation between them, reads the finished
    values.  Checked over a chain of plain, ragged and plan launches against
    the same chain with a device synchronisation after every launch."""
    import torch
    h, off = frg.ragged_horizons(96, 8, 256, seed=40)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(n, seed=41)
    tqd, tu = (torch.from_numpy(x).cuda() for x in (qd, u))

    def chain(sync):
        bufs = [torch.from_numpy(q).cuda()] + [torch.zeros((n, 7), device="cuda") for _ in range(6)]
        outs = []
        with frg.Context() as ctx:
            plan = None
            for i in range(6):
                d = torch.zeros((n, 98), device="cuda")
                m = torch.zeros((n, 49), device="cuda")
                # this launch's joint angles are the previous launch's q̈ (q enters through
                # sin and cos, so the chain stays finite)
                if i % 3 == 0:
                    ctx.gradient(n, bufs[i], tqd, tu, d, bufs[i + 1], m, torch.cuda.current_stream())
                elif i % 3 == 1:
                    ctx.ragged(off, bufs[i], tqd, tu, d, bufs[i + 1], m, torch.cuda.current_stream())
                else:
                    plan = ctx.plan_ragged(off, bufs[i], tqd, tu, d, bufs[i + 1], m)
                    plan.launch(torch.cuda.current_stream())
                if sync:
                    torch.cuda.synchronize()
                outs.append(d)
            torch.cuda.synchronize()
            if plan is not None:
                plan.close()
        return [o.cpu() for o in outs] + [b.cpu() for b in bufs]

    unsynced, synced = chain(False), chain(True)
    assert all(bool(torch.isfinite(t).all()) for t in synced)
    for a, b in zip(unsynced, synced):
        assert torch.equal(a, b)


def test_plans_prepared_ahead_chain_without_synchronisation():
    """Plans prepared before the chain launch back to back, each reading the
    previous launch's q̈ output as its joint angles: the kernels bring their
    first tile's inputs into L2 before they wait for the launch ahead of them,
    and still read the finished values.  Checked against the same chain with a
    device synchronisation after every launch: plans alone, plans between
    plain gradient and forward-dynamics launches (which prefetch too), and both
    again in the latency mapping (8 lanes per knot)."""
    import torch
    h, off = frg.ragged_horizons(128, 8, 256, seed=60)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(n, seed=61)
    tqd, tu = (torch.from_numpy(x).cuda() for x in (qd, u))

    def chain(sync, kinds, lanes):
        steps = len(kinds)
        bufs = [torch.from_numpy(q).cuda()] + [torch.zeros((n, 7), device="cuda") for _ in range(steps)]
        outs = [(torch.zeros((n, 98), device="cuda"), torch.zeros((n, 49), device="cuda")) for _ in range(steps)]
        with frg.Context() as ctx:
            ctx.set_lanes_per_knot(lanes)
            plans = {i: ctx.plan_ragged(off, bufs[i], tqd, tu, outs[i][0], bufs[i + 1], outs[i][1])
                     for i, k in enumerate(kinds) if k == "plan"}
            torch.cuda.synchronize()
            st = torch.cuda.current_stream()
            for i, k in enumerate(kinds):
                if k == "plan":
                    plans[i].launch(st)
                elif k == "plain":
                    ctx.gradient(n, bufs[i], tqd, tu, outs[i][0], bufs[i + 1], outs[i][1], st)
                else:
                    ctx.forward_dynamics(n, bufs[i], tqd, tu, bufs[i + 1], outs[i][1], stream=st)
                if sync:
                    torch.cuda.synchronize()
            torch.cuda.synchronize()
            for p in plans.values():
                p.close()
        return [t.cpu() for o in outs for t in o] + [b.cpu() for b in bufs]

    for lanes in (1, 8):
        for kinds in (["plan"] * 6, ["plan", "plain", "plan", "fd", "plan", "plain"]):
            unsynced, synced = chain(False, kinds, lanes), chain(True, kinds, lanes)
            assert all(bool(torch.isfinite(t).all()) for t in synced)
            for a, b in zip(unsynced, synced):
                assert torch.equal(a, b)


def test_plan_launch_many_matches_single_launches():
    """Independent plans several in flight (frg_plan_launch_many: plan i on
    stream i mod in_flight) give the bits of launching each plan alone, for
    1 to 4 in flight; work queued on the stream after the call sees every
    result without a host synchronisation; a plan at two residues, an
    in_flight outside 1..4, or a plan of another context is refused."""
    import torch
    with frg.Context() as ctx, frg.Context() as other:
        sets = []
        for i in range(4):
            h, off = frg.ragged_horizons(48, 8, 256, seed=90 + i)
            n = int(off[-1])
            q, qd, u = frg.sample_knots(n, seed=190 + i)
            ins = [torch.from_numpy(x).cuda() for x in (q, qd, u)]
            alone, many = alloc(torch, n), alloc(torch, n)
            sets.append((ctx.plan_ragged(off, *ins, *alone), ctx.plan_ragged(off, *ins, *many), alone, many, off, ins))
        for p_alone, _, _, _, _, _ in sets:
            p_alone.launch()
        torch.cuda.synchronize()
        st = torch.cuda.current_stream()
        for in_flight in (1, 2, 3, 4):
            k = 3 if in_flight == 3 else 4  # plans per period: each plan keeps one residue
            for _, _, _, many, _, _ in sets:
                for t in many:
                    t.fill_(float("nan"))
            ctx.plan_launch_many([s[1] for s in sets[:k]] * 3, st, in_flight)
            sums = [torch.stack([t.sum() for t in s[3]]) for s in sets[:k]]  # queued after the call, no host sync
            torch.cuda.synchronize()
            for (_, _, alone, many, _, _), sm in zip(sets[:k], sums):
                for a, b in zip(alone, many):
                    assert torch.equal(a, b), in_flight
                assert torch.equal(sm, torch.stack([t.sum() for t in alone])), in_flight
        ctx.plan_launch_many([], st)
        with pytest.raises(frg.FrgError, match="another residue"):
            ctx.plan_launch_many([sets[0][1], sets[1][1], sets[1][1]], st, 2)  # plan 1 at positions 1 and 2
        with pytest.raises(frg.FrgError, match="another residue"):
            ctx.plan_launch_many([sets[0][1], sets[1][1]] * 2, st, 3)  # plan 0 at positions 0 and 2
        for bad in (0, 5):
            with pytest.raises(frg.FrgError, match="in_flight"):
                ctx.plan_launch_many([sets[0][1]], st, bad)
        foreign = other.plan_ragged(sets[0][4], *sets[0][5], *alloc(torch, int(sets[0][4][-1])))
        with pytest.raises(frg.FrgError, match="another context"):
            ctx.plan_launch_many([sets[0][1], foreign], st)
        foreign.close()
        for s in sets:
            s[0].close()
            s[1].close()


def test_plan_launches_capture_into_a_cuda_graph():
    """Plan launches captured into a CUDA graph (torch.cuda.graph) replay with
    the bits of direct launches."""
    import torch
    h, off = frg.ragged_horizons(64, 8, 256, seed=50)
    n = int(off[-1])
    q, qd, u = frg.sample_knots(n, seed=51)
    tq, tqd, tu = (torch.from_numpy(x).cuda() for x in (q, qd, u))
    with frg.Context() as ctx:
        direct = alloc(torch, n)
        p1 = ctx.plan_ragged(off, tq, tqd, tu, *direct)
        p1.launch(torch.cuda.current_stream())
        torch.cuda.synchronize()
        graphed = alloc(torch, n)
        p2 = ctx.plan_ragged(off, tq, tqd, tu, *graphed)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            p2.launch(s)  # warm-up outside the capture
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        for t in graphed:
            t.zero_()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            p2.launch(torch.cuda.current_stream())
            p2.launch(torch.cuda.current_stream())
        g.replay()
        torch.cuda.synchronize()
        for a, b in zip(direct, graphed):
            assert torch.equal(a, b)
        p1.close()
        p2.close()
