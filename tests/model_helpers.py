"""Test helpers for URDF-generated models.

synthetic_urdf(): a seeded serial arm (7 joints by default, any count from 1
to 8) that exercises every general
form the kernels and the oracle take: frames at arbitrary roll/pitch/yaw,
joint origins off the axes, joint axes other than z (one reversed), inertial
frames with their own rotation, fixed links before the first joint and after
the last, and a welded leaf in the middle of the chain; its base joint is
tilted, so column 0 of d tau / dq does not vanish.

NewtonEuler: an independent check of the dynamics, written from the URDF
directly in the world frame (classical Newton-Euler about the centres of
mass, gravity -9.81 z): it shares nothing with the spatial-algebra code of
the kernels or the oracle, nor with the re-orientation done by frg/urdf.py.
"""
import ctypes
import subprocess

import numpy as np

from frg import urdf

GRAVITY = 9.81


def _rpy(rng, scale=np.pi):
    return rng.uniform(-scale, scale, 3)


def _fmt(v):
    return " ".join(f"{x:.17g}" for x in v)


def synthetic_urdf(seed=11, name="synthetic_arm", joints=7):
    rng = np.random.default_rng(seed)
    parts = [f'<robot name="{name}">', '<link name="world"/>',
             # a mount rigidly attached to the world: part of the fixed base
             '<joint name="mount" type="fixed"><parent link="world"/><child link="pedestal"/>'
             f'<origin xyz="{_fmt(rng.uniform(-0.2, 0.2, 3))}" rpy="{_fmt(_rpy(rng, 0.3))}"/></joint>',
             '<link name="pedestal"><inertial><origin xyz="0 0 0.1"/><mass value="9"/>'
             '<inertia ixx="1" ixy="0" ixz="0" iyy="1" iyz="0" izz="1"/></inertial></link>']
    parent = "pedestal"
    for k in range(joints):
        axis = rng.normal(size=3)
        if k == 3:
            axis = np.array([0.0, 0.0, -1.0])  # reversed z
        if k == 0:
            axis = np.array([0.3, 0.1, 1.0])   # tilted against gravity: column 0 lives
        axis /= np.linalg.norm(axis)
        parts.append(f'<joint name="j{k + 1}" type="{"continuous" if k == 5 else "revolute"}">'
                     f'<parent link="{parent}"/><child link="l{k + 1}"/>'
                     f'<origin xyz="{_fmt(rng.uniform(-0.15, 0.25, 3))}" rpy="{_fmt(_rpy(rng))}"/>'
                     f'<axis xyz="{_fmt(axis)}"/></joint>')
        A = rng.normal(size=(3, 3))
        I = A @ A.T * 0.02 + np.eye(3) * 0.01
        parts.append(f'<link name="l{k + 1}"><inertial><origin xyz="{_fmt(rng.uniform(-0.1, 0.1, 3))}" '
                     f'rpy="{_fmt(_rpy(rng))}"/><mass value="{rng.uniform(0.8, 5.0):.17g}"/>'
                     f'<inertia ixx="{I[0, 0]:.17g}" ixy="{I[0, 1]:.17g}" ixz="{I[0, 2]:.17g}" '
                     f'iyy="{I[1, 1]:.17g}" iyz="{I[1, 2]:.17g}" izz="{I[2, 2]:.17g}"/></inertial></link>')
        if k == min(3, joints - 1):  # a welded sensor on link 4 (or the last)
            parts.append(f'<joint name="sensor_mount" type="fixed"><parent link="l{k + 1}"/><child link="sensor"/>'
                         f'<origin xyz="{_fmt(rng.uniform(-0.1, 0.1, 3))}" rpy="{_fmt(_rpy(rng))}"/></joint>'
                         '<link name="sensor"><inertial><origin xyz="0.01 0.02 0.03" rpy="0.1 0.2 0.3"/>'
                         '<mass value="0.4"/><inertia ixx="0.001" ixy="0.0001" ixz="0" iyy="0.002" iyz="0" '
                         'izz="0.0015"/></inertial></link>')
        parent = f"l{k + 1}"
    # a tool rigidly attached to the last link, with a frame of its own
    parts.append(f'<joint name="tool_mount" type="fixed"><parent link="l{joints}"/><child link="tool"/>'
                 f'<origin xyz="{_fmt(rng.uniform(-0.1, 0.1, 3))}" rpy="{_fmt(_rpy(rng))}"/></joint>'
                 '<link name="tool"><inertial><origin xyz="0 0 0.05" rpy="0 0.5 0"/><mass value="0.7"/>'
                 '<inertia ixx="0.003" ixy="0" ixz="0" iyy="0.004" iyz="0" izz="0.002"/></inertial></link>')
    parts.append("</robot>")
    return "\n".join(parts)


def _axis_angle(a, q):
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(q) * K + (1 - np.cos(q)) * (K @ K)


class NewtonEuler:
    """tau(q, qd, qdd) of the parsed chain by world-frame Newton-Euler."""

    def __init__(self, urdf_text):
        self.m = urdf.parse(urdf_text)

    def tau(self, q, qd, qdd, gravity=True):
        R, p = np.eye(3), np.zeros(3)
        w, dw = np.zeros(3), np.zeros(3)
        a_p = np.array([0.0, 0.0, GRAVITY if gravity else 0.0])  # base accelerates up: gravity
        z, P, C, F, N = [], [], [], [], []
        for k, (j, ine) in enumerate(zip(self.m["joints"], self.m["inertials"])):
            pj = p + R @ j["xyz"]                       # joint origin, fixed in the parent body
            d = pj - p
            a_p = a_p + np.cross(dw, d) + np.cross(w, np.cross(w, d))
            Rj = R @ j["R0"]
            zk = Rj @ (j["axis"] / np.linalg.norm(j["axis"]))
            R = Rj @ _axis_angle(j["axis"], q[k])       # body frame of link k
            dw = dw + zk * qdd[k] + np.cross(w, zk * qd[k])
            w = w + zk * qd[k]
            c = pj + R @ ine.c
            rc = c - pj
            a_c = a_p + np.cross(dw, rc) + np.cross(w, np.cross(w, rc))
            Iw = R @ ine.icom @ R.T
            z.append(zk); P.append(pj); C.append(c)
            F.append(ine.m * a_c)
            N.append(Iw @ dw + np.cross(w, Iw @ w))
            p = pj
        nj = len(z)
        tau = np.zeros(nj)
        f, n = np.zeros(3), np.zeros(3)
        for k in range(nj - 1, -1, -1):
            if k < nj - 1:
                n = n + np.cross(P[k + 1] - P[k], f)
            n = N[k] + n + np.cross(C[k] - P[k], F[k])
            f = F[k] + f
            tau[k] = z[k] @ n
        return tau

    @property
    def dofs(self):
        return len(self.m["joints"])

    def mass_matrix(self, q):
        nj = self.dofs
        Z = np.zeros(nj)
        return np.stack([self.tau(q, Z, np.eye(nj)[j], gravity=False) for j in range(nj)], axis=1)

    def forward(self, q, qd, u, gravity=True):
        M = self.mass_matrix(q)
        qdd = np.linalg.solve(M, u - self.tau(q, qd, np.zeros(self.dofs), gravity))
        return qdd, np.linalg.inv(M)

    def gradient(self, q, qd, u, gravity=True, h=1e-6):
        """[dqdd/dq | dqdd/dqd] (N x 2N) by central differences."""
        nj = self.dofs
        G = np.zeros((nj, 2 * nj))
        for j in range(nj):
            e = np.zeros(nj)
            e[j] = h
            G[:, j] = (self.forward(q + e, qd, u, gravity)[0] - self.forward(q - e, qd, u, gravity)[0]) / (2 * h)
            G[:, nj + j] = (self.forward(q, qd + e, u, gravity)[0] - self.forward(q, qd - e, u, gravity)[0]) / (2 * h)
        return G


def write_tables(text, path, source="synthetic_urdf()"):
    with open(path, "w") as f:
        f.write(urdf.emit_header(urdf.tables(urdf.parse(text)), source))
    return path


def build_oracle(header, out_so, root):
    """The oracle compiled for the robot of a tables header."""
    subprocess.run(["make", "-s", "-f", f"{root}/oracle/Makefile", "oracle", f"MODEL_TABLES={header}",
                    f"ORACLE_SO={out_so}"], check=True)
    return out_so


def oracle_gradient_f64(so, q, qd, u, damping=0, mpc=0):
    """dqdd [n,2N^2], qdd [n,N], minv [n,N^2] from a model's oracle library."""
    L = ctypes.CDLL(so)
    vp, i = ctypes.c_void_p, ctypes.c_int
    L.frg_oracle_gradient_f64.argtypes = [i, vp, vp, vp, vp, i, i, vp, vp, vp]
    L.frg_oracle_dofs.restype = i
    q, qd, u = (np.ascontiguousarray(x, np.float64) for x in (q, qd, u))
    n, nj = q.shape
    assert nj == L.frg_oracle_dofs(), "inputs do not match the oracle's joint count"
    out = [np.zeros((n, w)) for w in (2 * nj * nj, nj, nj * nj)]
    L.frg_oracle_gradient_f64(n, q.ctypes.data, qd.ctypes.data, u.ctypes.data, None, damping, mpc,
                              *(o.ctypes.data for o in out))
    return out
