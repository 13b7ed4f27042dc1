"""Per-knot status flags (frg_knot_status) and the tuning get/set round trip (GPU)."""
import numpy as np
import pytest

import frg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 33, 5000])
def test_knot_status_flags_nonfinite_knots_only(n):
    import torch
    q, qd, u = frg.sample_knots(n, seed=60 + n)
    bad_in = sorted({0, n // 2, n - 1})
    q[bad_in[0], 3] = np.nan
    if len(bad_in) > 1:
        qd[bad_in[1], 0] = np.inf
        u[bad_in[-1], 6] = -np.inf
    tq, tqd, tu = (torch.from_numpy(a).cuda() for a in (q, qd, u))
    out = [torch.empty((n, w), device="cuda") for w in (98, 7, 49)]
    status = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    with frg.Context() as ctx:
        ctx.gradient(n, tq, tqd, tu, *out)
        ctx.knot_status(n, tq, tqd, tu, None, None, None, status)  # inputs only
        torch.cuda.synchronize()
        s_in = status.cpu().numpy().copy()
        ctx.knot_status(n, tq, tqd, tu, *out, status)
        torch.cuda.synchronize()
        s_all = status.cpu().numpy()
    expect_in = np.zeros(n, np.int32)
    expect_in[bad_in] = frg.KNOT_NONFINITE_INPUT
    assert np.array_equal(s_in, expect_in)
    # a non-finite input makes its own knot's results non-finite, nobody else's
    expect_all = expect_in.copy()
    expect_all[bad_in] |= frg.KNOT_NONFINITE_OUTPUT
    assert np.array_equal(s_all, expect_all)


def test_knot_status_flags_an_output_alone():
    import torch
    n = 100
    q, qd, u = frg.sample_knots(n, seed=2)
    tq, tqd, tu = (torch.from_numpy(a).cuda() for a in (q, qd, u))
    out = [torch.empty((n, w), device="cuda") for w in (98, 7, 49)]
    status = torch.empty((n,), dtype=torch.int32, device="cuda")
    with frg.Context() as ctx:
        ctx.gradient(n, tq, tqd, tu, *out)
        out[2][77, 48] = float("nan")
        ctx.knot_status(n, tq, tqd, tu, *out, status)
        torch.cuda.synchronize()
    s = status.cpu().numpy()
    assert s[77] == frg.KNOT_NONFINITE_OUTPUT and np.count_nonzero(s) == 1


def test_tuning_round_trip_and_validation():
    import torch
    n = 3000
    q, qd, u = frg.sample_knots(n, seed=4)
    with frg.Context() as ctx:
        ctx.autotune(4096)
        tuned = ctx.tuning()
        with frg.Context() as other:
            other.set_tuning(tuned)
            assert other.tuning() == tuned
            a = ctx.gradient_host(q, qd, u)
            b = other.gradient_host(q, qd, u)
            for x, y in zip(a, b):
                assert np.array_equal(x, y)
            for bad in ({"warps_per_cta": 0}, {"lanes_per_knot": 4}, {"ragged_ctas_per_sm": 0},
                        {"ragged_ctas_per_sm": 10000}, {"ragged_warps_per_cta": 9}):
                with pytest.raises(frg.FrgError) as ei:
                    other.set_tuning({**tuned, **bad})
                assert ei.value.status == 1
            assert other.tuning() == tuned  # a rejected set changes nothing
