"""bench.py's reference arm on the CPU (it needs no GPU): one JSON line with
the contract's keys, timed on a tiny sample of the benchmark workload."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--cpu-steps", "1", "--workload", "obstacles_65536"], cwd=ROOT, capture_output=True, text=True,
                         timeout=600, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert "obstacles_65536" in d["config"]["workload"]


def test_reference_arm_restarts_like_the_gpu_arm(monkeypatch, capsys):
    """A workload with a restart period (the collapsing 1M column's lines
    restart before it outgrows the reference's capacities) restarts the CPU
    scene the same way, outside the timed updates; exercised here on the
    65,536-particle scene with a short period."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench, "RESTART_AFTER", {"obstacles_65536": 4})
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--workload", "obstacles_65536",
                                      "--steps", "3", "--warmup", "3"])
    assert bench.main() == 0
    line = json.loads([ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")][-1])
    assert line["steps"] == 3 and line["value"] > 0
    assert "restarted from update 3 before update 4 (2 restarts)" in line["cpu_baseline"]["sample"]
