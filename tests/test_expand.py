"""The host threads that expand packed Minv (csrc/frg_expand.h) for the
pipelined host-buffer call: a C++ check compiled with the host compiler (no
GPU), at the iiwa's 7 joints and at 6 and 8, whose packed rows carry padding."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "fast-rbd-gradients_gb300", "csrc")


@pytest.mark.parametrize("joints", [7, 6, 8])
def test_expander_jobs_write_exactly_their_matrices(tmp_path, joints):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "test_expand"
    tables = tmp_path / "tables.h"  # the one macro the expander's sizes come from
    tables.write_text(f"#pragma once\n#define FRG_MODEL_NUM_JOINTS {joints}\n")
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", f'-DFRG_MODEL_TABLES="{tables}"', "-I", CSRC,
                    os.path.join(HERE, "cpp", "test_expand.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith(f"OK: N={joints},"), r.stdout
