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


class _FakeEvent:
    def __init__(self, **kw):
        pass

    def record(self, stream=None):
        pass

    def synchronize(self):
        pass

    def elapsed_time(self, other):
        return 10.0


class _NoStream:
    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


class _CountingSim:
    """Stands in for the simulation in the GPU arm's bookkeeping: its state
    is the number of updates it has taken (written into every array), so a
    loaded state tells which update it was taken after."""
    n = 64

    def __init__(self, domain, device=0):
        self.updates = 0
        self.loaded = []

    def __getattr__(self, name):  # scene set-up calls (add_particles, bodies, ...)
        return lambda *a, **k: None

    def update(self, dt):
        self.updates += 1

    def stream(self):
        return 0

    def dump_state(self, out=None):
        import numpy as np
        st = {k: np.full((self.n, 2), self.updates, np.float32) for k in ("pos", "prev", "vel", "acc", "dens", "press")}
        st.update({k: np.full(self.n, self.updates, np.int32) for k in ("id", "cell", "cell_start", "cell_count")})
        st["canonical_count"], st["grid"] = self.n, (8, 8)
        if out is not None:
            for k in out:
                out[k][...] = st[k]
        return st

    def dump_springs(self, out=None):
        import numpy as np
        return (np.full(self.n, self.updates, np.int32), np.zeros((self.n, 4), np.int32),
                np.zeros((self.n, 4), np.float32))

    def load_state(self, st):
        self.updates = int(st["pos"][0, 0])
        self.loaded.append(self.updates)

    def autotune(self, dt):
        return (4, 100, 12, 100)

    def kernel_launches(self):
        return 10 * self.updates

    def get_stats(self):
        return type("Stats", (), {"__getattr__": lambda self, k: 1.0})()

    def last_sweep_shape(self):
        return (4, 100, 12, 100)

    def read_particles(self, keys):
        import numpy as np
        return {"dens": np.ones((self.n, 2), np.float32)}

    def spring_count(self):
        return 0


def test_gpu_arm_restarts_from_update_3_and_spreads_the_e2e_states(monkeypatch):
    """The GPU arm's bookkeeping on the headline workload's default window
    (20 warm-up and 100 timed updates, restart before update 90), with a
    stand-in simulation: restarts load the update-3 state, and the
    end-to-end leg loads four states taken across the timed window, an equal
    share of the steps each after two untimed steps."""
    import numpy as np
    import torch
    sys.path.insert(0, ROOT)
    import bench
    sims = []

    class Sim(_CountingSim):
        def __init__(self, *a, **k):
            super().__init__(*a, **k)
            sims.append(self)

    monkeypatch.setattr(torch.cuda, "Event", _FakeEvent)
    monkeypatch.setattr(torch.cuda, "ExternalStream", lambda ptr: None)
    monkeypatch.setattr(torch.cuda, "stream", lambda s: _NoStream())
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a: None)
    monkeypatch.setattr(bench, "pinned_like", lambda torch_, arrays: {k: np.array(a) for k, a in arrays.items()})
    pkg = type("Pkg", (), {"Simulation": Sim})
    out = bench.measure_scene(torch, pkg, bench.HEADLINE, 0, 100, 20, 1, torch.zeros(4), 25)
    sim = sims[0]
    assert out["restarts"]["count"] == 1 and out["restarts"]["after_updates"] == 90
    assert sim.loaded[0] == 3  # the restart
    e2e_loads = sim.loaded[1:]
    assert out["e2e"]["steps"] == 28  # 4 states x ceil(25 / 4) steps
    assert e2e_loads == [45] * 9 + [70] * 9 + [8] * 9 + [33] * 9
    assert "45, 70, 8, 33" in out["e2e"]["states"]
    assert out["ms_per_step"] == 10.0 and out["steps"] == 100
