"""Reference order on the GPU: free runs against the reference's own
trajectory, through the C ABI.

In reference order (``sph_set_reference_order``) the library visits particles
in AddParticle order in both ordered passes and the grid update, as the
reference's Update does on its own numbering (demo4.cpp:223-255, 344-352).
A free run then reproduces the reference's trajectory bit for bit:

* the golden fixtures that the reference's own solver made (tests/golden:
  the 4,096-particle dam break after 1, 2 and 10 updates; a block falling
  onto every body type after 6 updates) are matched at 0 ulp in positions,
  previous positions, velocities, densities and pressures, with identical
  cell arrays and statistics;
* 100 free updates against the oracle running in its own order, compared
  after every update; the same with particles added mid-run, with springs,
  and in every sweep shape.

The default (fast) order renumbers particles every update; its free-run
difference from the reference's trajectory is measured and printed here.
"""
import os

import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes
from nbodysimulation_experiment_gb300.simulation import DELTA_WARPS, VISC_WARPS
from oracle import state as ostate
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu

DT = float(scenes.DT)
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = ("pos", "prev", "vel", "dens", "press")


def _check_against(sim, want, prefix=""):
    """The simulation (AddParticle order) equals a reference state given as
    arrays in the reference's index order, at 0 ulp, with identical cell
    arrays (as id sequences) and statistics."""
    got = sim.read_particles(FIELDS)
    for k in FIELDS:
        assert ostate.ulp_diff(got[k], want[prefix + k]) == 0, prefix + k
    cells = ostate.gpu_cells_by_id(sim.dump_state())
    flat = np.asarray(want[prefix + "cell_flat"]).astype(np.int64)
    off = 0
    for c, cnt in enumerate(np.asarray(want[prefix + "cell_count"]).astype(np.int64)):
        assert np.array_equal(cells[c], flat[off:off + cnt]), (prefix, c)
        off += cnt
    if prefix + "stats" in want:
        st = sim.get_stats()
        assert [st.min_particle_neighbor_count, st.max_particle_neighbor_count, st.min_cell_particle_count,
                st.max_cell_particle_count] == [int(v) for v in want[prefix + "stats"]]


def _oracle_arrays(orc):
    st = orc.get_state(lists=False)
    out = {k: np.asarray(st[k], np.float32) for k in FIELDS}
    out["cell_count"] = st["cell_count"]
    out["cell_flat"] = st["cell_flat"]
    counts, _ = orc.get_stats()
    out["stats"] = counts
    return out


def test_reference_order_reproduces_the_reference_trajectory():
    g = np.load(os.path.join(GOLDEN, "dam_break_4096.npz"))
    scene = scenes.dam_break_4096()
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.set_reference_order(True)
    assert sim.reference_order()
    for step in range(1, 11):
        sim.update(DT)
        if step in (1, 2, 10):
            _check_against(sim, g, "step%d_" % step)
    sim.close()


def test_reference_order_bodies_golden():
    g = np.load(os.path.join(GOLDEN, "bodies_400.npz"))
    sim = pkg.Simulation(pkg.reference_domain())
    sim.set_gravity((0.0, -10.0))
    sim.set_params(pkg.Params.from_array(scenes.scenario_params()))
    for nx, ny, d in scenes.box_planes(scenes.REF_WIDTH, scenes.REF_HEIGHT):
        sim.add_plane((nx, ny), d)
    sim.add_circle((0.6, -0.8), 0.5)
    sim.add_line_segment((-2.0, -1.5), (-0.5, -2.2))
    sim.add_polygon(g["polygon"])
    sim.add_external_forces((1.0, 0.0))
    sim.add_particles(g["initial_pos"])
    sim.set_reference_order(True)
    for _ in range(6):
        sim.update(DT)
    _check_against(sim, g, "step6_")
    sim.close()


@pytest.mark.parametrize("shape", ["wide", "lean"])
def test_reference_order_free_run_100_updates(shape):
    scene = scenes.dam_break_4096()
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.set_reference_order(True)
    orc = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(orc)
    for step in range(100):
        sim.update(DT)
        orc.update(DT)
        if step == 1 and shape == "lean":
            base = sim.sweep_shape()
            sim.set_sweep_shape((VISC_WARPS[1], base[1], DELTA_WARPS[1], base[3]))
        _check_against(sim, _oracle_arrays(orc))
    sim.close()
    orc.close()


def test_reference_order_with_particles_added_mid_run():
    scene = scenes.scaled_block(24, seed=6)
    scene.max_particles = scene.n + 200
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.set_reference_order(True)
    orc = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(orc)
    rng = np.random.default_rng(8)
    for step in range(30):
        if step in (5, 17):
            extra = (rng.uniform(-1.0, 1.0, (80, 2)) * 0.6).astype(np.float32)
            force = np.tile(np.float32([[0.5, 1.0]]), (80, 1))
            sim.add_particles(extra, force)
            orc.add_particles(extra, force)
        sim.update(DT)
        orc.update(DT)
        _check_against(sim, _oracle_arrays(orc))
    sim.close()
    orc.close()


def test_reference_order_obstacles_65536_free_run():
    scene = scenes.obstacles_65536()
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.set_reference_order(True)
    orc = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(orc)
    for step in range(6):
        sim.update(DT)
        orc.update(DT)
    _check_against(sim, _oracle_arrays(orc))
    sim.close()
    orc.close()


def test_reference_order_with_springs_free_run():
    springs = dict(yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    scene = scenes.scaled_block(32, seed=21)
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.set_springs(True, **springs)
    sim.set_reference_order(True)
    orc = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(orc)
    orc.set_springs(True, **springs)
    for step in range(25):
        sim.update(DT)
        orc.update(DT)
        _check_against(sim, _oracle_arrays(orc))
    assert sim.spring_count() == orc.spring_total() // 2 > 0
    sim.close()
    orc.close()


def test_default_order_free_run_difference_is_reported():
    """The default order equals the reference on update 1 (every particle is
    then visited in AddParticle order); from update 2 on it visits the
    particles in its cell-colour numbering, a different Gauss-Seidel order of
    the same passes, so its trajectory departs from the reference's own.  The
    size of that departure against the reference's updates 2 and 10 is
    printed; measured on GB300: after update 2 the median position differs
    by 0.031 h and the largest by 0.27 h, after update 10 by 0.28 h and 2.4 h
    (the dam break is chaotic)."""
    g = np.load(os.path.join(GOLDEN, "dam_break_4096.npz"))
    scene = scenes.dam_break_4096()
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    h = float(scene.params[0])
    report = {}
    for step in range(1, 11):
        sim.update(DT)
        if step in (1, 2, 10):
            got = sim.read_particles(FIELDS)
            d = np.abs(got["pos"].astype(np.float64) - g["step%d_pos" % step]).max(axis=1)
            v = np.abs(got["vel"].astype(np.float64) - g["step%d_vel" % step]).max(axis=1)
            report[step] = {"pos_max_over_h": float(d.max() / h), "pos_median_over_h": float(np.median(d) / h),
                            "vel_max": float(v.max()), "differing": int(np.count_nonzero(d)),
                            "pos_ulp": ostate.ulp_diff(got["pos"], g["step%d_pos" % step])}
    print("default order vs the reference's own trajectory:", report)
    assert report[1]["pos_ulp"] == 0
    assert 0.0 < report[2]["pos_median_over_h"] < 0.2 and report[2]["pos_max_over_h"] < 1.0
    sim.close()
