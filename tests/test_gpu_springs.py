"""Viscoelastic springs on the GPU against the oracle, through the C ABI.

The reference has no springs: both sides restate Clavet et al. 2005 in the
same deterministic parallel form, and the oracle's form is pinned against an
independent NumPy restatement (tests/test_springs_oracle.py).  Each
comparison is one teacher-forced update: the GPU's state and spring tables
are loaded into the oracle, both advance one step, and positions, velocities
and every spring (partner and rest length, per particle, in slot order) must
match exactly.
"""
import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes
from oracle import state as ostate
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
SPRINGS = dict(yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
DT = float(scenes.DT)


def _springs_by_id(count, partner, rest, ids):
    out = {}
    for k in range(len(count)):
        out[int(ids[k])] = [(int(ids[partner[k, q]]), float(rest[k, q])) for q in range(count[k])]
    return out


def _teacher_step(sim, orc):
    before = sim.dump_state()
    cnt, part, rest = sim.dump_springs()
    orc.set_state(ostate.to_reference_state(before))
    orc.set_spring_state(cnt, np.where(part < 0, 0, part), rest, tag=before["id"])
    orc.update(DT)
    sim.update(DT)
    after = sim.dump_state()
    res = ostate.compare_step(before, after, orc.get_state(lists=False))
    g = _springs_by_id(*sim.dump_springs(), after["id"])
    o = _springs_by_id(*orc.get_spring_state(), before["id"])
    return res, g, o


def test_springs_match_oracle_teacher_forced():
    scene = scenes.scaled_block(32, seed=21)
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.set_springs(True, **SPRINGS)
    orc = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(orc)
    orc.set_springs(True, **SPRINGS)
    total = 0
    for step in range(25):
        res, g, o = _teacher_step(sim, orc)
        assert res["cells_equal"] == 1.0, (step, res)
        for k in ("pos", "vel", "dens", "press"):
            assert res[k + "_rel"] <= REL_TOL, (step, k, res)
        assert res["pos_ulp"] == 0 and res["vel_ulp"] == 0, (step, res)
        assert g == o, step
        total = sum(len(v) for v in g.values())
    assert total > 0
    assert sim.spring_count() * 2 == total


def test_springs_free_run_invariants():
    scene = scenes.scaled_block(64, seed=4)
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.set_springs(True, yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=12)
    for _ in range(40):
        sim.update(DT)
    st = sim.dump_state()
    cnt, part, rest = sim.dump_springs()
    h = np.float32(scene.params[0])
    assert cnt.max() <= 12 and cnt.sum() > 0
    assert sim.spring_count() * 2 == int(cnt.sum())
    for i in np.nonzero(cnt)[0][:2000]:
        for q in range(cnt[i]):
            j, L = part[i, q], rest[i, q]
            assert 0 < L <= h
            back = np.nonzero(part[j, :cnt[j]] == i)[0]
            assert len(back) == 1 and rest[j, back[0]] == L
    assert np.all(np.isfinite(st["pos"]))


def test_springs_graph_replay_equals_eager():
    scene = scenes.scaled_block(40, seed=8)
    out = []
    for graphs in (False, True):
        sim = pkg.Simulation(scene.domain())
        sim.use_graphs(graphs)
        scene.apply(sim)
        sim.set_springs(True, **SPRINGS)
        for _ in range(20):
            sim.update(DT)
        out.append((sim.dump_state(), sim.dump_springs()))
        sim.close()
    (a, sa), (b, sb) = out
    for k in ("pos", "vel", "id", "cell_start", "cell_count"):
        assert np.array_equal(a[k], b[k]), k
    for x, y in zip(sa, sb):
        assert np.array_equal(x, y)


def test_springs_off_leaves_the_plain_step_unchanged():
    scene = scenes.scaled_block(24, seed=2)
    out = []
    for toggle in (False, True):
        sim = pkg.Simulation(scene.domain())
        scene.apply(sim)
        if toggle:
            sim.set_springs(True, **SPRINGS)
            sim.set_springs(False, **SPRINGS)
        for _ in range(10):
            sim.update(DT)
        out.append(sim.dump_state())
        sim.close()
    for k in ("pos", "vel", "dens", "id"):
        assert np.array_equal(out[0][k], out[1][k]), k
