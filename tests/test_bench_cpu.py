"""The benchmark's CPU legs run here without a GPU: the reference arm prints
its one JSON line with the contract's keys, and the config-0 CPU timing
reports the same CG count as the device run (5 iterations)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [line for line in r.stdout.splitlines() if line.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    # every variant was timed: four cachings in plain loops, and each at 2/4/8 lanes
    sample = d["cpu_baseline"]["sample"]
    assert sum(sample.count(f"/simd{w} ") for w in (2, 4, 8)) == 12


def test_cpu_heat_step_leg():
    sys.path.insert(0, ROOT)
    import bench
    out = bench.cpu_heat_step()
    assert out["cg_its"] == 5
    assert out["vmult_dofs_per_s"] >= out["vmult_all_dofs_per_s"]["plain"] > 0
