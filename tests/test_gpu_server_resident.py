"""Device-resident serving (GPU): calls whose inputs are already on the GPU
(frg_server_submit_device), calls on the inputs resident in a trajectory's
device slot (frg_server_submit_resident), in-place updates of that slot
(frg_server_slot), and results kept on the device.  Every result must be bit
for bit the host-submitted call's on the same inputs, alone and in a mix."""
import ctypes

import numpy as np
import pytest

import frg
import frg_oracle
from conftest import TOL, max_err
from frg import native

pytestmark = pytest.mark.gpu

OK, NOT_FOUND = 0, 8
H2D, D2H = 1, 2


def _cudart():
    """The CUDA runtime libfrg.so loaded (for raw-pointer copies)."""
    native.lib()
    for line in open("/proc/self/maps"):
        path = line.split()[-1]
        if "libcudart.so" in path:
            L = ctypes.CDLL(path)
            L.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
            L.cudaMemcpy.restype = ctypes.c_int
            return L
    raise RuntimeError("libcudart not loaded")


def _dev_results(info):
    """Host copies of (dqdd, qdd, minv) from a call's device-slot pointers."""
    rt = _cudart()
    out = []
    for ptr, w in ((info.dev_dqdd, 98), (info.dev_qdd, 7), (info.dev_minv, 49)):
        a = np.empty((info.horizon, w), np.float32)
        assert rt.cudaMemcpy(a.ctypes.data, ptr, a.nbytes, D2H) == 0
        out.append(a)
    return out


def _same(a, b):
    return all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a, b))


def _host_call(srv, tid, q, qd, u):
    st, rid = srv.submit(tid, q, qd, u)
    assert st == OK
    st, info = srv.wait(rid, timeout_us=20_000_000)
    assert st == OK and info.status == OK
    return frg.Server.results(info)


@pytest.mark.parametrize("latency_max", [4096, 0])
def test_device_resident_and_in_place_calls_match_host_calls(latency_max):
    """Both thread mappings (small batches take the 8-lane mapping unless
    latency_mapping_max_knots is 0)."""
    import torch
    rt = _cudart()
    with frg.Context() as ctx, frg.Server(ctx, latency_mapping_max_knots=latency_max) as srv:
        for k, h in enumerate((16, 64, 200)):
            q, qd, u = frg.sample_knots(h, seed=700 + k)
            base = _host_call(srv, 10 + k, q, qd, u)
            # resident: the host call left its inputs in the device slot
            st, rid = srv.submit_resident(10 + k)
            assert st == OK
            st, info = srv.wait(rid, timeout_us=20_000_000)
            assert st == OK and info.status == OK
            assert not info.dqdd  # results stayed on the device
            assert _same(_dev_results(info), base)
            # a new iterate already on the GPU, results to both slots
            q2, qd2, u2 = (frg.perturb(x, 1e-2, seed=50 + k + i) for i, x in enumerate((q, qd, u)))
            dq2, dqd2, du2 = (torch.from_numpy(x).cuda() for x in (q2, qd2, u2))
            torch.cuda.synchronize()
            st, rid = srv.submit_device(10 + k, dq2, dqd2, du2, host_results=True)
            assert st == OK
            st, info = srv.wait(rid, timeout_us=20_000_000)
            assert st == OK and info.status == OK
            want = _host_call(srv, 100 + k, q2, qd2, u2)
            assert _same(frg.Server.results(info), want)
            assert _same(_dev_results(info), want)
            # in-place update of the slot's inputs, then a resident call
            q3, qd3, u3 = (frg.perturb(x, 1e-2, seed=80 + k + i) for i, x in enumerate((q, qd, u)))
            st, slot = srv.slot(10 + k)
            assert st == OK and slot.horizon == h
            for ptr, x in ((slot.q, q3), (slot.qd, qd3), (slot.u, u3)):
                assert rt.cudaMemcpy(ptr, x.ctypes.data, x.nbytes, H2D) == 0
            st, rid = srv.submit_resident(10 + k, host_results=True)
            assert st == OK
            st, info = srv.wait(rid, timeout_us=20_000_000)
            assert st == OK
            got = frg.Server.results(info)
            assert _same(got, _host_call(srv, 200 + k, q3, qd3, u3))
            ref = frg_oracle.gradient_f64(q3, qd3, u3)
            for a, r in zip(got, ref):
                assert max_err(a, r) <= TOL


def test_mixed_sources_in_one_batch_match_alone():
    """Host, device and resident calls submitted together (so the dispatcher
    folds them into shared launches) each give their alone bits."""
    import torch
    rng = np.random.default_rng(5)
    hs = [int(h) for h in rng.choice([16, 32, 64, 128], size=60)]
    data = [frg.sample_knots(h, seed=900 + i) for i, h in enumerate(hs)]
    with frg.Context() as ctx, frg.Server(ctx, max_inflight=2) as srv:
        alone = [_host_call(srv, 5000 + i, *d) for i, d in enumerate(data)]
        # give every trajectory resident inputs first (a host call each)
        for i, d in enumerate(data):
            _host_call(srv, i, *d)
        dev = [tuple(torch.from_numpy(x).cuda() for x in d) for d in data]
        torch.cuda.synchronize()
        rids = {}
        for i in range(len(data)):
            if i % 3 == 0:
                st, rid = srv.submit(i, *data[i])
            elif i % 3 == 1:
                st, rid = srv.submit_device(i, *dev[i], host_results=True)
            else:
                st, rid = srv.submit_resident(i, host_results=True)
            assert st == OK
            rids[rid] = i
        shared = 0
        for rid, i in rids.items():
            st, info = srv.wait(rid, timeout_us=20_000_000)
            assert st == OK and info.status == OK
            assert _same(frg.Server.results(info), alone[i]), f"call {i}"
            assert _same(_dev_results(info), alone[i]), f"call {i} (device slot)"
            shared += info.batch_requests > 1
        assert shared > 0  # some calls really shared a launch


def test_resident_calls_need_a_completed_call():
    with frg.Context() as ctx, frg.Server(ctx) as srv:
        st, _ = srv.submit_resident(12345)
        assert st == NOT_FOUND
        st, _ = srv.slot(12345)
        assert st == NOT_FOUND
