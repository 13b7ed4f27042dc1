"""The oracle (C restatement of the reference CPU path) against the reference's
own outputs (tests/golden, generated from oracle/_ref) and against finite
differences of itself.  CPU only."""
import numpy as np
import pytest

import frg
import frg_oracle
from conftest import max_err

MODES = [(d, m) for d in (0, 1) for m in (0, 1)]


@pytest.mark.parametrize("damping,mpc", MODES)
def test_oracle_f64_matches_reference_golden(golden, damping, mpc):
    d, q, m = frg_oracle.gradient_f64(golden["q"], golden["qd"], golden["u"], damping, mpc)
    tag = f"f64_d{damping}_m{mpc}"
    assert max_err(d, golden[f"dqdd_{tag}"]) < 1e-11
    assert max_err(q, golden[f"qdd_{tag}"]) < 1e-11
    assert max_err(m, golden[f"minv_{tag}"]) < 1e-11


def test_oracle_f32_matches_reference_f32_golden(golden):
    d, q, m = frg_oracle.gradient_f32(golden["q"], golden["qd"], golden["u"])
    assert max_err(d, golden["dqdd_f32_d0_m0"]) < 2e-5
    assert max_err(q, golden["qdd_f32_d0_m0"]) < 2e-5
    assert max_err(m, golden["minv_f32_d0_m0"]) < 2e-5


def test_reference_fp32_meets_the_bar(golden):
    # the reference's own FP32 path is within the 1e-4 bar of its FP64 path
    for out in ("dqdd", "qdd", "minv"):
        assert max_err(golden[f"{out}_f32_d0_m0"], golden[f"{out}_f64_d0_m0"]) < 1e-4


def test_equivalence_point_is_present(golden):
    # the reference's TEST_FOR_EQUIVALENCE knot q = qd = u = 0.1
    assert golden["names"][0] == "equivalence_0.1"
    assert np.all(golden["q"][0] == np.float32(0.1))
    assert np.all(np.isfinite(golden["dqdd_f64_d0_m0"][0]))


def test_minv_symmetric_positive_definite(golden):
    _, _, m = frg_oracle.gradient_f64(golden["q"], golden["qd"], golden["u"])
    M = m.reshape(-1, 7, 7)
    assert np.abs(M - M.transpose(0, 2, 1)).max() == 0.0
    assert (np.linalg.eigvalsh(M) > 0).all()


@pytest.mark.parametrize("damping", [0, 1])
def test_oracle_against_finite_differences(damping):
    q, qd, u = frg.sample_knots(12, seed=99)
    q, qd, u = (x.astype(np.float64) for x in (q, qd, u))
    d, _, minv = frg_oracle.gradient_f64(q, qd, u, damping)
    h = 1e-6
    n = q.shape[0]
    fd = np.zeros((n, 7, 14))
    fdu = np.zeros((n, 7, 7))
    for j in range(7):
        e = np.zeros(7)
        e[j] = h
        for col, (dq, dqd, du) in enumerate(((e, 0, 0), (0, e, 0), (0, 0, e))):
            _, qp, _ = frg_oracle.gradient_f64(q + dq, qd + dqd, u + du, damping)
            _, qm, _ = frg_oracle.gradient_f64(q - dq, qd - dqd, u - du, damping)
            g = (qp - qm) / (2 * h)
            if col < 2:
                fd[:, :, 7 * col + j] = g
            else:
                fdu[:, :, j] = g
    grad = d.reshape(n, 14, 7).transpose(0, 2, 1)  # column-major 7x14
    assert max_err(grad.reshape(n, -1), fd.reshape(n, -1)) < 1e-6
    # d qdd / d u = Minv
    assert max_err(minv.reshape(n, 7, 7).reshape(n, -1), fdu.transpose(0, 2, 1).reshape(n, -1)) < 1e-6


@pytest.mark.skipif(not frg_oracle.ref_available(), reason="oracle/_ref not built (reference tree absent)")
@pytest.mark.parametrize("damping,mpc", MODES)
def test_oracle_matches_live_reference(damping, mpc):
    q, qd, u = frg.sample_knots(300, seed=5 + 2 * damping + mpc)
    a = frg_oracle.gradient_f64(q, qd, u, damping, mpc)
    b = frg_oracle.ref_gradient_f64(q, qd, u, damping, mpc)
    for x, y in zip(a, b):
        assert max_err(x, y) < 1e-11


def test_threaded_driver_matches_serial():
    q, qd, u = frg.sample_knots(257, seed=3)
    t, (d, qq, m) = frg_oracle.time_threaded_f32(q, qd, u, threads=3, iters=2)
    d2, q2, m2 = frg_oracle.gradient_f32(q, qd, u)
    assert t > 0
    assert np.array_equal(d, d2) and np.array_equal(qq, q2) and np.array_equal(m, m2)


def test_time_cpu_mode_matches_full_path():
    """The reference's time_CPU mode (q̈ and Minv passed in) gives the full
    path's dqdd bit for bit when fed the full path's own q̈ and Minv; the
    threaded driver in that mode agrees with the serial call."""
    q, qd, u = frg.sample_knots(130, seed=8)
    d, qq, m = frg_oracle.gradient_f32(q, qd, u)
    assert np.array_equal(frg_oracle.gradient_given_f32(q, qd, qq, m), d)
    t, (d3, q3, m3) = frg_oracle.time_threaded_given_f32(q, qd, u, threads=3, iters=2)
    assert t > 0 and np.array_equal(d3, d) and np.array_equal(q3, qq) and np.array_equal(m3, m)
