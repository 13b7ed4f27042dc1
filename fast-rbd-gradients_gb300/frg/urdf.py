"""Model tables for the gradient kernels from a URDF of a serial revolute arm.

The kernels take the robot at compile time: one header of tables (joint frame
rotations, joint origins, link inertials) that frg_model.cuh turns into
per-joint constants, so that structural zeros and signed-permutation frames
cost nothing at run time.  This module writes that header from a URDF:

    python -m frg.urdf robot.urdf -o robot_tables.h [--name NAME]
    FRG_MODEL_TABLES=$PWD/robot_tables.h python -c "import __graft_entry__ as g; g.build()"

Accepted robots: a fixed base followed by a serial chain of 1 to 8 revolute
(or continuous) joints; the header records the joint count N, and the
library built from it has the per-knot sizes of an N-joint arm (N x 2N
gradient, N x N Minv; frg_model_dofs() reports N).  Fixed joints are merged:
links rigidly attached before the first joint are part of the fixed base,
links rigidly attached to a moving link add their inertia to it.  Any joint
axis is accepted: each moving frame is re-oriented so that its joint turns
about z, the form the kernels use.

Conventions (URDF): a joint's <origin xyz rpy> places the joint frame in the
parent link frame, rpy = fixed-axis roll, pitch, yaw (R = Rz Ry Rx); a link's
<inertial><origin> places the centre of mass and the inertia tensor's frame.
The tables follow the reference's spatial model (helpers_CPU/
dynamicsGradient.h): joint transform iX(i-1) = [E 0; -E r^ E], E = Rz(q)^T F,
with F = R^T of the (re-oriented) joint frame and r its origin in the parent
frame; link inertia as (Ixx Ixy Ixz Iyy Iyz Izz at the COM, COM, mass) in the
link frame.  Gravity is -z of the base frame.
"""
import argparse
import math
import xml.etree.ElementTree as ET

import numpy as np

MAX_JOINTS = 8  # the latency mapping gives each joint a lane of its 8
_SNAP = 1e-12


def _floats(s, n, default=0.0):
    if s is None:
        return [default] * n
    v = [float(x) for x in s.split()]
    if len(v) != n:
        raise ValueError(f"expected {n} numbers, got {s!r}")
    return v


def rpy_matrix(r, p, y):
    """R = Rz(y) Ry(p) Rx(r) (URDF fixed-axis roll, pitch, yaw)."""
    cr, sr, cp, sp, cy, sy = math.cos(r), math.sin(r), math.cos(p), math.sin(p), math.cos(y), math.sin(y)
    rx = np.array([[1, 0, 0], [0, cr, -sr], [0, sr, cr]])
    ry = np.array([[cp, 0, sp], [0, 1, 0], [-sp, 0, cp]])
    rz = np.array([[cy, -sy, 0], [sy, cy, 0], [0, 0, 1]])
    return rz @ ry @ rx


def _snap(a):
    """Entries within 1e-12 of 0 or +-1 become exact (frames given in multiples
    of pi/2 then stay signed permutations, the kernels' fast form)."""
    a = np.array(a, dtype=np.float64)
    for t in (0.0, 1.0, -1.0):
        a[np.abs(a - t) < _SNAP] = t
    return a


def z_to_axis(axis):
    """A rotation Q with Q e_z = axis (unit)."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    z = np.array([0.0, 0.0, 1.0])
    c = float(z @ a)
    if c > 1 - 1e-15:
        return np.eye(3)
    if c < -1 + 1e-15:
        return np.diag([1.0, -1.0, -1.0])  # half turn about x
    k = np.cross(z, a)
    s = np.linalg.norm(k)
    k = k / s
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + s * K + (1 - c) * (K @ K)


class Inertial:
    """Mass, COM and inertia tensor at the COM, in some link frame."""

    def __init__(self, m=0.0, c=(0.0, 0.0, 0.0), icom=None):
        self.m = float(m)
        self.c = np.asarray(c, np.float64)
        self.icom = np.zeros((3, 3)) if icom is None else np.asarray(icom, np.float64)

    def moved(self, R, p):
        """The same body seen from a frame where this frame has rotation R and origin p."""
        return Inertial(self.m, R @ self.c + p, R @ self.icom @ R.T)

    def __add__(self, o):
        if o.m == 0:
            return Inertial(self.m, self.c, self.icom)
        if self.m == 0:  # exact: a massless start leaves the other body's numbers untouched
            return Inertial(o.m, o.c, o.icom)
        m = self.m + o.m
        c = (self.m * self.c + o.m * o.c) / m
        icom = np.zeros((3, 3))
        for b in (self, o):
            d = b.c - c
            icom += b.icom + b.m * (d @ d * np.eye(3) - np.outer(d, d))
        return Inertial(m, c, icom)


def _link_inertial(link):
    el = link.find("inertial")
    if el is None:
        return Inertial()
    org = el.find("origin")
    xyz = _floats(org.get("xyz") if org is not None else None, 3)
    rpy = _floats(org.get("rpy") if org is not None else None, 3)
    mass = float(el.find("mass").get("value"))
    it = el.find("inertia")
    ixx, ixy, ixz, iyy, iyz, izz = (float(it.get(k, "0")) for k in ("ixx", "ixy", "ixz", "iyy", "iyz", "izz"))
    I = np.array([[ixx, ixy, ixz], [ixy, iyy, iyz], [ixz, iyz, izz]])
    R = rpy_matrix(*rpy)
    return Inertial(mass, np.array(xyz), R @ I @ R.T)


def parse(text):
    """URDF text -> dict(name, joints=[{name, R0, xyz, axis}], inertials=[Inertial])
    for the 7 moving links, fixed joints merged (see the module docstring)."""
    root = ET.fromstring(text)
    links = {l.get("name"): l for l in root.findall("link")}
    children = {}
    child_names = set()
    for j in root.findall("joint"):
        children.setdefault(j.find("parent").get("link"), []).append(j)
        child_names.add(j.find("child").get("link"))
    roots = [n for n in links if n not in child_names]
    if len(roots) != 1:
        raise ValueError(f"expected one root link, found {roots}")

    def placement(j):
        org = j.find("origin")
        xyz = np.array(_floats(org.get("xyz") if org is not None else None, 3))
        rpy = _floats(org.get("rpy") if org is not None else None, 3)
        return rpy_matrix(*rpy), xyz

    def weld(link, R, p):
        """Links rigidly attached to `link` (itself included) with their
        placements, and the moving joints leaving any of them."""
        bodies, movers = [(link, R, p)], []
        for j in children.get(link, []):
            kind = j.get("type")
            Rj, pj = placement(j)
            Rc, pc = R @ Rj, R @ pj + p
            if kind == "fixed":
                b, m = weld(j.find("child").get("link"), Rc, pc)
                bodies += b
                movers += m
            elif kind in ("revolute", "continuous"):
                movers.append((j, Rc, pc))
            else:
                raise ValueError(f"joint {j.get('name')}: type {kind} is not supported "
                                 "(revolute, continuous and fixed only)")
        return bodies, movers

    out_joints, inertials = [], []
    link, moving = roots[0], None  # moving: index of the moving body `link` belongs to
    while True:
        bodies, movers = weld(link, np.eye(3), np.zeros(3))
        if moving is not None:  # before the first joint the bodies are the fixed base
            for name, R, p in bodies:
                inertials[moving] = inertials[moving] + _link_inertial(links[name]).moved(R, p)
        if not movers:
            break
        if len(movers) > 1:
            raise ValueError(f"more than one moving joint after link {link}: a tree, not a serial chain")
        j, R0, xyz = movers[0]
        ax = j.find("axis")
        axis = np.array(_floats(ax.get("xyz") if ax is not None else "1 0 0", 3))
        out_joints.append({"name": j.get("name"), "R0": R0, "xyz": xyz, "axis": axis})
        inertials.append(Inertial())
        moving = len(out_joints) - 1
        link = j.find("child").get("link")
    if not 1 <= len(out_joints) <= MAX_JOINTS:
        raise ValueError(f"the kernels take 1 to {MAX_JOINTS} moving joints; this chain has {len(out_joints)}")
    return {"name": root.get("name", "robot"), "joints": out_joints, "inertials": inertials}


def tables(model):
    """Per-joint F (column-major 3x3), origin r, link inertial rows, and whether
    column 0 of d tau / d q vanishes (gravity along the first joint's axis)."""
    F, origin, inertial = [], [], []
    Q_prev = np.eye(3)
    for j, ine in zip(model["joints"], model["inertials"]):
        Q = z_to_axis(j["axis"])
        R0 = Q_prev.T @ j["R0"] @ Q          # parent (re-oriented) -> joint frame turning about z
        F.append(_snap(R0.T).T.reshape(-1))  # column-major F = R0^T
        origin.append(_snap(Q_prev.T @ j["xyz"]))
        c = Q.T @ ine.c
        I = _snap(Q.T @ ine.icom @ Q)
        inertial.append([I[0, 0], I[0, 1], I[0, 2], I[1, 1], I[1, 2], I[2, 2], *_snap(c), ine.m])
        Q_prev = Q
    F0 = np.array(F[0]).reshape(3, 3, order="F")
    col0_zero = bool(abs(F0[0, 2]) < _SNAP and abs(F0[1, 2]) < _SNAP)
    return {"name": model["name"], "F": np.array(F), "origin": np.array(origin), "inertial": np.array(inertial),
            "dq_column0_zero": col0_zero}


def _fmt(x):
    r = repr(float(x))
    return "0.0" if r in ("0.0", "-0.0") else r


def emit_header(t, source="a URDF"):
    """C/C++ header text of the tables (included by frg_model.cuh and the oracle)."""
    def rows(a):
        return " \\\n".join("    {" + ", ".join(_fmt(x) for x in row) + "}," for row in a)
    return f"""/* Model tables of {t['name']}: written by frg/urdf.py from {source}.
 * Per joint k: F = R^T of the joint frame in its parent's frame (column-major
 * 3x3, the joint turning about z), the joint origin r in the parent frame, and
 * the link inertial (Ixx Ixy Ixz Iyy Iyz Izz at the COM, COM x y z, mass) in
 * the link frame.  FRG_MODEL_DQ_COLUMN0_ZERO is 1 when gravity (-z of the
 * base) lies along the first joint's axis, which makes column 0 of d tau / dq
 * vanish identically. */
#pragma once
#define FRG_MODEL_NAME "{t['name']}"
#define FRG_MODEL_NUM_JOINTS {len(t['F'])}
#define FRG_MODEL_DQ_COLUMN0_ZERO {1 if t['dq_column0_zero'] else 0}
#define FRG_MODEL_JOINT_F {{ \\
{rows(t['F'])} }}
#define FRG_MODEL_JOINT_ORIGIN {{ \\
{rows(t['origin'])} }}
#define FRG_MODEL_LINK_INERTIAL {{ \\
{rows(t['inertial'])} }}
"""


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("urdf")
    ap.add_argument("-o", "--out", required=True)
    ap.add_argument("--name", default=None)
    args = ap.parse_args(argv)
    with open(args.urdf) as f:
        model = parse(f.read())
    if args.name:
        model["name"] = args.name
    t = tables(model)
    with open(args.out, "w") as f:
        f.write(emit_header(t, source=args.urdf.split("/")[-1]))
    print(f"{args.out}: {t['name']}, column 0 of d tau/dq {'zero' if t['dq_column0_zero'] else 'computed'}")


if __name__ == "__main__":
    main()
