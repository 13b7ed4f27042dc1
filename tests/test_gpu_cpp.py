"""C++ callers of the C ABI (GPU): the C++ parity test in tests/cpp (against the
oracle), and the time_frg driver (the time_GPU.cu counterpart): its
TEST_FOR_EQUIVALENCE printout against the reference's own outputs for that
point, its ragged mode, and its batch-size rows."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, TOL, max_err

pytestmark = pytest.mark.gpu

FRG_DIR = os.path.join(ROOT, "fast-rbd-gradients_gb300", "frg")
ORACLE_DIR = os.path.join(ROOT, "oracle")
TIME_FRG = os.path.join(FRG_DIR, "bin", "time_frg")


def _nvcc():
    from frg import build
    return build._nvcc()


def test_cpp_parity_against_oracle(tmp_path, built_lib):
    assert os.path.exists(os.path.join(ORACLE_DIR, "libfrg_oracle.so")), "build the oracle first (build())"
    exe = str(tmp_path / "test_frg_parity")
    cmd = [_nvcc(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_frg_parity.cpp"), "-o", exe, "-cudart", "shared",
           "-L", FRG_DIR, "-lfrg", "-L", ORACLE_DIR, "-lfrg_oracle",
           "-Xlinker", f"-rpath,{FRG_DIR}:{ORACLE_DIR}:/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "PASSED: 0 failure(s)" in r.stdout
    assert len(re.findall(r"vs FP64 oracle", r.stdout)) == 4  # every (damping, mpc) mode


def _matrix_after(lines, title, rows):
    i = lines.index(title)
    return np.array([[float(x) for x in lines[i + 1 + r].split()] for r in range(rows)])


def test_time_frg_equivalence_point_matches_reference(golden, built_lib):
    r = subprocess.run([TIME_FRG, "--equivalence"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = [ln.strip() for ln in r.stdout.splitlines()]
    k = list(golden["names"]).index("equivalence_0.1")
    i = lines.index("q,qd,qdd,u")
    qdd = np.array([float(x) for x in lines[i + 3].split()])
    minv = _matrix_after(lines, "Minv", 7)
    ddq = _matrix_after(lines, "dqdd/dq", 7)
    ddqd = _matrix_after(lines, "dqdd/dqd", 7)
    # printMat prints rows of the column-major matrices
    dqdd = np.concatenate([ddq.T.reshape(-1), ddqd.T.reshape(-1)])
    assert max_err(qdd[None], golden["qdd_f64_d0_m0"][k][None]) <= TOL
    assert max_err(minv.T.reshape(1, -1), golden["minv_f64_d0_m0"][k][None]) <= TOL
    assert max_err(dqdd[None], golden["dqdd_f64_d0_m0"][k][None]) <= TOL


def test_time_frg_ragged_and_batch_rows(built_lib):
    r = subprocess.run([TIME_FRG, "--ragged", "64", "--iters", "5"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert len(re.findall(r"^\[N:\d+\] (Plain|Batched)", r.stdout, re.M)) == 4
    assert re.search(r"^\[N:\d+\] Batched - two independent plans in flight", r.stdout, re.M)
    r = subprocess.run([TIME_FRG, "--iters", "5", "16", "1000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert len(re.findall(r"^\[N:(16|1000)\] Completely Fused", r.stdout, re.M)) == 4
