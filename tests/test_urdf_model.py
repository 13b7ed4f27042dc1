"""URDF-driven models (CPU): the tables generator (frg/urdf.py), and the oracle
built for a generated robot checked against an independent world-frame
Newton-Euler model of the same URDF."""
import os

import numpy as np
import pytest

from conftest import REFERENCE_DIR, ROOT
from frg import urdf
from model_helpers import NewtonEuler, build_oracle, oracle_gradient_f64, synthetic_urdf, write_tables

IIWA_URDF = os.path.join(REFERENCE_DIR, "utils", "iiwa_14.urdf")
IIWA_HEADER = os.path.join(ROOT, "fast-rbd-gradients_gb300", "csrc", "frg_model_iiwa14.h")


@pytest.mark.skipif(not os.path.exists(IIWA_URDF), reason="reference URDF not present")
def test_iiwa_tables_regenerate_from_the_urdf():
    """The committed iiwa tables are exactly what the generator writes from the
    reference's utils/iiwa_14.urdf."""
    with open(IIWA_URDF) as f:
        t = urdf.tables(urdf.parse(f.read()))
    t["name"] = "iiwa_14"
    with open(IIWA_HEADER) as f:
        assert f.read() == urdf.emit_header(t, "utils/iiwa_14.urdf")
    assert t["dq_column0_zero"]


def _chain(joints, extra=""):
    parts = ['<robot name="r"><link name="b"/>']
    parent = "b"
    for k, kind in enumerate(joints):
        parts.append(f'<joint name="j{k}" type="{kind}"><parent link="{parent}"/><child link="l{k}"/>'
                     '<origin xyz="0 0 0.1"/><axis xyz="0 0 1"/></joint>'
                     f'<link name="l{k}"><inertial><mass value="1"/>'
                     '<inertia ixx="0.1" ixy="0" ixz="0" iyy="0.1" iyz="0" izz="0.1"/></inertial></link>')
        parent = f"l{k}"
    return "".join(parts) + extra + "</robot>"


def test_generator_rejects_what_the_kernels_cannot_take():
    with pytest.raises(ValueError, match="1 to 8 moving joints"):
        urdf.parse(_chain(["revolute"] * 9))
    with pytest.raises(ValueError, match="1 to 8 moving joints"):
        urdf.parse(_chain(["fixed"] * 2))
    with pytest.raises(ValueError, match="not supported"):
        urdf.parse(_chain(["revolute"] * 3 + ["prismatic"] + ["revolute"] * 3))
    branch = ('<joint name="extra" type="revolute"><parent link="l2"/><child link="x"/><axis xyz="0 0 1"/></joint>'
              '<link name="x"/>')
    with pytest.raises(ValueError, match="serial chain"):
        urdf.parse(_chain(["revolute"] * 7, branch))


def test_generator_reorients_axes_and_merges_fixed_links():
    t = urdf.tables(urdf.parse(synthetic_urdf()))
    assert not t["dq_column0_zero"]
    for F in t["F"]:  # each F a rotation
        R = np.array(F).reshape(3, 3, order="F")
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and np.isclose(np.linalg.det(R), 1.0)
    m = urdf.parse(synthetic_urdf())
    # link 4 carries the welded sensor, link 7 the tool
    assert m["inertials"][3].m > 0.4 and m["inertials"][6].m > 0.7
    m6 = urdf.parse(synthetic_urdf(joints=6))
    assert len(m6["joints"]) == 6 and m6["inertials"][5].m > 0.7


@pytest.fixture(scope="module", params=[7, 6, 3, 8])
def synthetic_oracle(tmp_path_factory, request):
    joints = request.param
    d = tmp_path_factory.mktemp(f"model{joints}")
    text = synthetic_urdf(joints=joints)
    header = write_tables(text, str(d / "synthetic_tables.h"))
    return text, header, build_oracle(header, str(d / "liboracle_synthetic.so"), ROOT)


def test_tables_carry_the_joint_count(synthetic_oracle):
    text, header, _ = synthetic_oracle
    nj = len(urdf.parse(text)["joints"])
    assert f"#define FRG_MODEL_NUM_JOINTS {nj}" in open(header).read()


@pytest.mark.parametrize("mpc", [0, 1])
def test_oracle_for_generated_model_matches_newton_euler(synthetic_oracle, mpc):
    """q̈ and Minv of the oracle built for the generated tables equal those of
    the world-frame Newton-Euler model of the URDF (FP64, <= 1e-10), and its
    gradient equals central differences of that model (<= 1e-6), for arms of
    7, 6, 3 and 8 joints."""
    text, _, so = synthetic_oracle
    ne = NewtonEuler(text)
    nj = ne.dofs
    rng = np.random.default_rng(5 + mpc)
    n = 6
    q, qd, u = rng.uniform(-2.5, 2.5, (n, nj)), rng.uniform(-2, 2, (n, nj)), rng.uniform(-20, 20, (n, nj))
    dqdd, qdd, minv = oracle_gradient_f64(so, q, qd, u, mpc=mpc)
    for k in range(n):
        r_qdd, r_minv = ne.forward(q[k], qd[k], u[k], gravity=not mpc)
        assert np.linalg.norm(qdd[k] - r_qdd) <= 1e-10 * np.linalg.norm(r_qdd)
        assert np.linalg.norm(minv[k] - r_minv.T.reshape(-1)) <= 1e-10 * np.linalg.norm(r_minv)
        G = ne.gradient(q[k], qd[k], u[k], gravity=not mpc)
        got = dqdd[k].reshape(2 * nj, nj).T  # column-major N x 2N
        assert np.linalg.norm(got - G) <= 1e-6 * np.linalg.norm(G)
        if not mpc:  # the tilted base joint: column 0 of d qdd / dq lives
            assert np.linalg.norm(got[:, 0]) > 1e-3 * np.linalg.norm(G)
