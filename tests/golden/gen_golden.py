"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own CPU path (helpers_CPU/*.h compiled unmodified behind
oracle/eigen_shim by oracle/Makefile into oracle/_ref/libfrg_ref.so) on seeded
iiwa_14 knots and stores inputs and outputs in iiwa_golden.npz.  The reference
tree is needed only here, when (re)generating; tests read the .npz.

Contents (all knots share one input set):
  q, qd, u                float32 [n, 7]  inputs (row k = knot k)
  names                   str [n]         what each knot is
  {out}_f64_d{D}_m{M}     float64         reference at T=double, VEL_DAMPING=D, MPC_MODE=M
  {out}_f32_d0_m0         float32         reference at T=float (experiment defaults)
  out in {dqdd [n,98], qdd [n,7], minv [n,49]}

Knots: the reference's TEST_FOR_EQUIVALENCE point q = qd = u = 0.1
(utils/experiment_helpers.h:11, time_CPU.cpp:68-71); the zero state; joint-limit
corners; and 48 knots from the benchmark distributions (q ~ U(joint limits of
utils/iiwa_14.urdf), qd ~ U(-2, 2), u ~ U(-20, 20)), seed 20211.

Usage:  python tests/golden/gen_golden.py   (from the repository root)
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "fast-rbd-gradients_gb300"))

from frg.inputs import JOINT_LIMITS, sample_knots  # noqa: E402


def build_inputs():
    names, qs, qds, us = [], [], [], []

    def add(name, q, qd, u):
        names.append(name)
        qs.append(np.asarray(q, np.float32))
        qds.append(np.asarray(qd, np.float32))
        us.append(np.asarray(u, np.float32))

    add("equivalence_0.1", [0.1] * 7, [0.1] * 7, [0.1] * 7)
    add("zero_state", [0.0] * 7, [0.0] * 7, [0.0] * 7)
    lim = JOINT_LIMITS.astype(np.float32)
    add("upper_limits", lim, [2.0] * 7, [20.0] * 7)
    add("lower_limits", -lim, [-2.0] * 7, [-20.0] * 7)
    add("alternating_limits", lim * np.array([1, -1] * 3 + [1]), [2, -2] * 3 + [2], [-20, 20] * 3 + [-20])
    q, qd, u = sample_knots(48, seed=20211)
    for k in range(48):
        add(f"seeded_{k}", q[k], qd[k], u[k])
    return np.array(names), np.stack(qs), np.stack(qds), np.stack(us)


def main():
    subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile"), "ref"], check=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libfrg_ref.so"))
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    names, q, qd, u = build_inputs()
    n = q.shape[0]
    out = {"names": names, "q": q, "qd": qd, "u": u}
    for dt, tag, fn in ((np.float64, "f64", lib.frg_ref_gradient_f64), (np.float32, "f32", lib.frg_ref_gradient_f32)):
        combos = [(d, m) for d in (0, 1) for m in (0, 1)] if tag == "f64" else [(0, 0)]
        for d, m in combos:
            Q, QD, U = (np.ascontiguousarray(x.astype(dt)) for x in (q, qd, u))
            dqdd = np.zeros((n, 98), dt)
            qdd = np.zeros((n, 7), dt)
            minv = np.zeros((n, 49), dt)
            rc = fn(n, ptr(Q), ptr(QD), ptr(U), d, m, ptr(dqdd), ptr(qdd), ptr(minv))
            assert rc == 0
            out[f"dqdd_{tag}_d{d}_m{m}"] = dqdd
            out[f"qdd_{tag}_d{d}_m{m}"] = qdd
            out[f"minv_{tag}_d{d}_m{m}"] = minv
    np.savez_compressed(os.path.join(HERE, "iiwa_golden.npz"), **out)
    print(f"wrote {n} knots to {os.path.join(HERE, 'iiwa_golden.npz')}")


if __name__ == "__main__":
    main()
