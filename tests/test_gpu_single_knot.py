"""Single-knot latency entry point (frg_single_knot_latency), the counterpart
of the reference's kern_single_full (time_GPU.cu:23-51): one warp repeats the
whole path over one knot.  Its results must be exactly those of a one-knot
frg_gradient call, in both thread mappings, whatever the repetition count."""
import numpy as np
import pytest

import frg
import frg_oracle
from conftest import TOL, max_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("damping,mpc", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("lanes", [1, 8])
def test_single_knot_repeats_give_the_plain_bits(lanes, damping, mpc):
    import torch
    q, qd, u = frg.sample_knots(1, seed=400 + 10 * lanes + 2 * damping + mpc)
    tq, tqd, tu = (torch.from_numpy(x).cuda() for x in (q, qd, u))
    with frg.Context(vel_damping=bool(damping), mpc_mode=bool(mpc)) as ctx:
        want = [torch.empty((1, w), device="cuda") for w in (98, 7, 49)]
        ctx.gradient(1, tq, tqd, tu, *want)
        for iters in (1, 37):
            got = [torch.full((1, w), float("nan"), device="cuda") for w in (98, 7, 49)]
            us = ctx.single_knot_latency(lanes, iters, tq, tqd, tu, *got, timed=True)
            assert us > 0.0
            for a, b in zip(got, want):
                assert torch.equal(a, b), f"iters={iters}"
    ref = frg_oracle.gradient_f64(q, qd, u, damping=bool(damping), mpc=bool(mpc))
    for a, r in zip(want, ref):
        assert max_err(a.cpu().numpy(), r) <= TOL


def test_single_knot_rejects_bad_arguments():
    import torch
    x = torch.zeros(98, device="cuda")
    with frg.Context() as ctx:
        for lanes, iters in ((2, 10), (1, 0)):
            with pytest.raises(frg.FrgError):
                ctx.single_knot_latency(lanes, iters, x, x, x, x, x, x)
