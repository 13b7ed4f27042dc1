"""Continuous-batching server (GPU): results alone vs in a mix, resident
device state, admission by pool bytes, errors."""
import threading

import numpy as np
import pytest

import frg
import frg_oracle
from conftest import TOL, max_err

pytestmark = pytest.mark.gpu


def knots(h, seed):
    return frg.sample_knots(h, seed=seed)


def test_single_call_matches_plain_path_bitwise():
    q, qd, u = knots(64, 1)
    with frg.Context() as ctx:
        plain = ctx.gradient_host(q, qd, u)
        with frg.Server(ctx) as srv:
            st, rid = srv.submit(7, q, qd, u)
            assert st == 0
            st, info = srv.wait(rid, timeout_us=10_000_000)
            assert st == 0 and info.status == 0 and info.horizon == 64
            got = frg.Server.results(info)
            assert info.latency_us > 0 and info.batch_requests >= 1
    for a, b in zip(got, plain):
        assert np.array_equal(a, b)


def test_results_same_alone_and_in_mix():
    """Each trajectory's result alone equals its result when submitted together
    with 200 others from 4 client threads (continuous batching), bit for bit."""
    rng = np.random.default_rng(3)
    hs = rng.choice([16, 32, 64, 128], size=200)
    data = [knots(int(h), 100 + i) for i, h in enumerate(hs)]
    with frg.Context() as ctx:
        alone = []
        with frg.Server(ctx) as srv:
            for i, (q, qd, u) in enumerate(data[:20]):
                st, rid = srv.submit(i, q, qd, u)
                st, info = srv.wait(rid)
                alone.append(frg.Server.results(info))
        mixed = [None] * len(data)
        batches = set()
        with frg.Server(ctx, max_inflight=3) as srv:
            ids = {}
            lock = threading.Lock()

            def client2(lo, hi):
                for i in range(lo, hi):
                    q, qd, u = data[i]
                    st, rid = srv.submit(1000 + i, q, qd, u)
                    assert st == 0
                    with lock:
                        ids[rid] = i
            ths = [threading.Thread(target=client2, args=(k * 50, (k + 1) * 50)) for k in range(4)]
            for t in ths:
                t.start()
            for t in ths:
                t.join()
            for _ in range(len(data)):
                st, info = srv.wait_any(timeout_us=20_000_000)
                assert st == 0 and info.status == 0
                mixed[ids[info.request_id]] = frg.Server.results(info)
                batches.add((info.batch_id, info.batch_requests))
            stats = srv.stats()
        assert stats["completed"] == 200 and stats["launches"] >= 1
        assert any(n > 1 for _, n in batches), "no call was batched with another"
    for i in range(20):
        for a, b in zip(alone[i], mixed[i]):
            assert np.array_equal(a, b)
    for i in range(0, 200, 17):
        rd, rq, rm = frg_oracle.gradient_f64(*data[i])
        assert max_err(mixed[i][0], rd) <= TOL and max_err(mixed[i][2], rm) <= TOL


def dev_to_host(ptr, shape):
    """Copy a device array (raw pointer) to numpy through the CUDA runtime the
    engine already loaded."""
    import ctypes
    rt = ctypes.CDLL("libcudart.so.13")
    out = np.empty(shape, np.float32)
    rc = rt.cudaMemcpy(ctypes.c_void_p(out.ctypes.data), ctypes.c_void_p(ptr), ctypes.c_size_t(out.nbytes), 2)
    assert rc == 0
    return out


def test_resident_device_state_and_repeated_calls():
    """Five iLQR-style calls of one trajectory (perturbed inputs): every result
    matches the oracle, and the trajectory's resident device copy holds the
    latest inputs and the same results as the host slot."""
    q, qd, u = knots(40, 9)
    with frg.Context() as ctx, frg.Server(ctx) as srv:
        for call in range(5):
            qq = frg.perturb(q, 1e-2, seed=call)
            st, rid = srv.submit(5, qq, qd, u)
            assert st == 0
            st, info = srv.wait(rid)
            assert st == 0 and info.status == 0
            host = frg.Server.results(info)
            assert np.array_equal(dev_to_host(info.dev_q, (40, 7)), qq)
            assert np.array_equal(dev_to_host(info.dev_dqdd, (40, 98)), host[0])
            assert np.array_equal(dev_to_host(info.dev_minv, (40, 49)), host[2])
            rd, _, _ = frg_oracle.gradient_f64(qq, qd, u)
            assert max_err(host[0], rd) <= TOL
        assert srv.release(5) == 0
        assert srv.release(5) == 8  # FRG_ERR_NOT_FOUND


def test_admission_waits_for_pool_space():
    """Pool fits exactly two 256-knot trajectories: the third waits (admission
    stall) and runs once one is released."""
    h = 256
    slot = 175 * 4 * h
    with frg.Context() as ctx, frg.Server(ctx, pool_bytes=2 * slot) as srv:
        ids = []
        for t in range(3):
            q, qd, u = knots(h, 50 + t)
            st, rid = srv.submit(t, q, qd, u)
            assert st == 0
            ids.append(rid)
        st, info = srv.wait(ids[0], timeout_us=10_000_000)
        assert st == 0
        st, _ = srv.wait(ids[1], timeout_us=10_000_000)
        assert st == 0
        st, _ = srv.wait(ids[2], timeout_us=200_000)
        assert st == 6  # FRG_ERR_TIMEOUT: still waiting for admission
        s = srv.stats()
        assert s["admission_stalls"] == 1 and s["queued_admission"] == 1
        assert srv.release(0) == 0
        st, info = srv.wait(ids[2], timeout_us=10_000_000)
        assert st == 0 and info.status == 0
        q, qd, u = knots(h, 52)
        rd, _, _ = frg_oracle.gradient_f64(q, qd, u)
        assert max_err(frg.Server.results(info)[0], rd) <= TOL


def test_server_argument_errors():
    q, qd, u = knots(8, 1)
    with frg.Context() as ctx, frg.Server(ctx, pool_bytes=1 << 20) as srv:
        big = knots(4096, 2)
        st, _ = srv.submit(1, *big)  # 4096 knots * 700 B > 1 MiB pool
        assert st == 5  # FRG_ERR_ADMISSION
        st, rid = srv.submit(2, q, qd, u)
        assert st == 0
        st2, _ = srv.submit(2, q, qd, u)  # same trajectory while in flight (or just done)
        assert st2 in (0, 4)
        srv.wait(rid)
        assert srv.poll(123456)[0] == 8
        assert srv.stats()["rejected"] == 1


def test_thread_mapping_threshold_keeps_bits():
    """A small call is served with 8 lanes per knot by default and with one
    lane per knot when latency_mapping_max_knots = 0; both give the plain
    path's bits, so a call's result does not depend on the size of the batch
    it lands in."""
    q, qd, u = knots(48, 5)
    with frg.Context() as ctx:
        ctx.set_lanes_per_knot(1)
        plain = ctx.gradient_host(q, qd, u)
        results = []
        for threshold in (0, None):
            with frg.Server(ctx, latency_mapping_max_knots=threshold) as srv:
                st, rid = srv.submit(3, q, qd, u)
                st, info = srv.wait(rid, timeout_us=10_000_000)
                assert st == 0 and info.status == 0
                results.append(frg.Server.results(info))
    for res in results:
        for a, b in zip(res, plain):
            assert np.array_equal(a, b)


def test_cancel_a_call_waiting_for_admission():
    """A call still waiting for pool space is withdrawn: it completes at once
    with FRG_ERR_CANCELLED and no results, the calls around it are unaffected,
    the trajectory can be submitted again, and a call already taken cannot be
    cancelled."""
    h = 256
    q, qd, u = knots(h, 31)
    with frg.Context() as ctx:
        plain = ctx.gradient_host(q, qd, u)
        # room for one 256-knot trajectory (700 B per knot), not two
        with frg.Server(ctx, pool_bytes=int(700 * h * 1.5)) as srv:
            st, a = srv.submit(1, q, qd, u)
            assert st == 0
            st, b = srv.submit(2, q, qd, u)  # waits until trajectory 1 releases its slot
            assert st == 0
            assert srv.cancel(b) == 0
            st, info = srv.wait(b, timeout_us=5_000_000)
            assert st == 0 and info.status == 10 and not info.dqdd
            st, info = srv.wait(a, timeout_us=5_000_000)
            assert st == 0 and info.status == 0
            for x, y in zip(frg.Server.results(info), plain):
                assert np.array_equal(x, y)
            assert srv.cancel(a) == 8   # taken: not found
            assert srv.cancel(12345) == 8
            assert srv.stats()["cancelled"] == 1
            assert srv.release(1) == 0
            st, b2 = srv.submit(2, q, qd, u)  # the cancelled trajectory runs normally now
            assert st == 0
            st, info = srv.wait(b2, timeout_us=5_000_000)
            assert st == 0 and info.status == 0
            for x, y in zip(frg.Server.results(info), plain):
                assert np.array_equal(x, y)
