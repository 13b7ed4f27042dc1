"""bench.py's contract on CPU: the reference arm's JSON line (the reference
algorithm's CPU path on this host), its rank handling under torchrun, and the
helpers the GPU arm's line is built from (the recorded ncu figures of the
benched kernel, the measured peaks)."""
import json
import os
import subprocess
import sys

from conftest import ROOT

BENCH = os.path.join(ROOT, "bench.py")


def _run(args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, BENCH] + args, capture_output=True, text=True, env=env, cwd=ROOT,
                          timeout=600)


def test_reference_arm_prints_the_contract_line():
    r = _run(["--impl", "reference", "--steps", "2", "--warmup", "1"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["unit"] == "knot-gradients/s" and d["scaling"] == "weak"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("port", "reference") and isinstance(cb["sample"], str)
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert d["config"]["knots_per_step"] == 66809


def test_reference_arm_other_ranks_do_no_work():
    r = _run(["--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"],
             {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_recorded_ncu_figures_are_consistent():
    """The GPU arm's roofline `traffic` and executed FLOP come from one ncu
    capture of the benched kernel on the benched mix: DRAM reads cover at least
    the algorithmic inputs, the executed FP32 work lies below the reference's
    op count (the kernel drops structural zeros), and the recorded FP32 peak is
    near the nominal 152 SMs x 128 lanes x 2 x 2.07 GHz."""
    sys.path.insert(0, ROOT)
    import bench
    m = bench.NCU_MIX
    assert m["knots"] == 66809
    assert m["dram_read_bytes"] >= 84 * m["knots"]
    assert 0 < m["executed_flop_per_knot"] < bench.FLOP_PER_KNOT_REF
    nominal = 152 * 128 * 2 * 2.07e9 / 1e12
    assert 0.9 * nominal < bench.FP32_PEAK_TFLOPS_MEASURED <= 1.01 * nominal


def test_peaks_are_read_from_the_measured_file():
    sys.path.insert(0, ROOT)
    import bench
    peaks, src = bench.load_peaks()
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        assert src == "measured"
    assert float(peaks["hbm_gbs"]) > 0


def test_rotating_sets_keep_one_stream_each():
    """The timed steps go through frg_plan_launch_many with IN_FLIGHT streams,
    step i on stream i mod IN_FLIGHT over set i mod ROTATING_SETS: every set
    must land on one stream only (the call refuses a plan at two residues),
    and the sets must still exceed L2 together."""
    sys.path.insert(0, ROOT)
    import bench
    assert 1 <= bench.IN_FLIGHT <= 4
    assert bench.ROTATING_SETS % bench.IN_FLIGHT == 0
    residues = {}
    for i in range(100):
        residues.setdefault(i % bench.ROTATING_SETS, set()).add(i % bench.IN_FLIGHT)
    assert all(len(r) == 1 for r in residues.values())
    assert bench.ROTATING_SETS * 66809 * bench.BYTES_PER_KNOT > 129e6
