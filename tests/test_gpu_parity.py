"""GPU parity: the CUDA step against the oracle, through the C ABI.

Every comparison is one update from an identical state: the GPU's state is
dumped, converted into the reference's full solver state (cell arrays,
indices in cell, neighbour lists) and loaded into the oracle, both advance one
step, and the results are matched particle by particle through the
AddParticle index.  Gates: cell arrays identical as ordered id sequences
(hence neighbour lists identical), positions and velocities within 1e-5
relative (the step is expected to be bit-identical; the max ulp distance is
also checked).
"""
import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes
from oracle import state as ostate
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5   # single-step relative error gate for positions/velocities
ULP_TOL = 0      # the step reproduces the reference's FP32 operation order


def _pair(scene, fp64=False):
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    orc = OracleSim(scene.oracle_domain(OracleSim), fp64=fp64)
    scene.apply(orc)
    return sim, orc


def _teacher_step(sim, orc, dt=float(scenes.DT)):
    before = sim.dump_state()
    orc.set_state(ostate.to_reference_state(before))
    orc.update(dt)
    sim.update(dt)
    after = sim.dump_state()
    return ostate.compare_step(before, after, orc.get_state(lists=False)), before, after


def _assert_step(res, ulp=ULP_TOL):
    assert res["cell_sets_equal"] == 1.0, res
    assert res["cells_equal"] == 1.0, res
    for k in ("pos", "prev", "vel", "dens", "press"):
        assert res[k + "_rel"] <= REL_TOL or res[k + "_ulp"] <= 4, (k, res)
    assert res["pos_ulp"] <= ulp and res["vel_ulp"] <= ulp, res


def test_first_update_from_scene_matches_reference_order():
    """The first update after loading runs in AddParticle order, as the
    reference does (demo4.cpp:286-451 on a freshly built scene)."""
    scene = scenes.dam_break_4096()
    sim, orc = _pair(scene)
    sim.update(float(scenes.DT))
    orc.update(float(scenes.DT))
    mine = sim.read_particles(("pos", "vel", "dens", "press"))
    ref = orc.get_state(lists=False)
    for k in ("pos", "vel", "dens", "press"):
        assert ostate.ulp_diff(mine[k], ref[k]) <= ULP_TOL, k
    counts, _ = orc.get_stats()
    st = sim.get_stats()
    assert [st.min_particle_neighbor_count, st.max_particle_neighbor_count, st.min_cell_particle_count,
            st.max_cell_particle_count] == [int(c) for c in counts]


def test_dam_break_4096_teacher_forced_100_steps():
    scene = scenes.dam_break_4096()
    sim, orc = _pair(scene)
    worst = {}
    for step in range(100):
        res, _, _ = _teacher_step(sim, orc)
        _assert_step(res)
        for k, v in res.items():
            worst[k] = max(worst.get(k, 0.0), v)
        counts, _ = orc.get_stats()
        st = sim.get_stats()
        assert st.min_particle_neighbor_count == counts[0] and st.max_particle_neighbor_count == counts[1]
    print("worst over 100 steps:", worst)


def test_obstacles_65536_teacher_forced():
    """Full-size 65,536-particle scene with circles and segments."""
    scene = scenes.obstacles_65536()
    sim, orc = _pair(scene)
    for _ in range(20):
        sim.update(float(scenes.DT))
    for _ in range(2):
        res, _, _ = _teacher_step(sim, orc)
        _assert_step(res)


def test_error_against_fp64():
    """Report the FP32 step's error against an FP64 build of the same step."""
    scene = scenes.scaled_block(32, seed=3)
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    for _ in range(10):
        sim.update(float(scenes.DT))
    orc64 = OracleSim(scene.oracle_domain(OracleSim), fp64=True)
    scene.apply(orc64)  # bodies, gravity, parameters
    before = sim.dump_state()
    orc64.set_state(ostate.to_reference_state(before))
    orc64.update(float(scenes.DT))
    sim.update(float(scenes.DT))
    after = sim.dump_state()
    ref = orc64.get_state(lists=False)
    res = ostate.compare_step(before, after, ref)
    print("FP32 GPU vs FP64 step (max, normwise):", {k: v for k, v in res.items() if k.endswith("_rel")})
    # Per-particle error relative to the largest position.  The reference's
    # step is discontinuous where particles coincide (Vec2Normalize maps a
    # zero vector to zero, vecmath.h:272-280) -- e.g. particles projected onto
    # the same wall corner -- so a few particles may differ by more than FP32
    # rounding between any two precisions; the bulk agrees to rounding.
    ids = before["id"].astype(np.int64)
    ref_pos = np.empty_like(ref["pos"])
    ref_pos[ids] = ref["pos"]
    mine = ostate.by_id(after, "pos").astype(np.float64)
    err = np.abs(mine - ref_pos).max(axis=1) / np.abs(ref_pos).max()
    print("per-particle position error vs FP64: median %.3g, 99th pct %.3g, max %.3g" %
          (np.median(err), np.percentile(err, 99), err.max()))
    assert np.median(err) < 1e-6
    assert res["dens_rel"] < 1e-4


def test_determinism():
    scene = scenes.scaled_block(24, seed=5)
    outs = []
    for _ in range(2):
        sim = pkg.Simulation(scene.domain())
        scene.apply(sim)
        for _ in range(15):
            sim.update(float(scenes.DT))
        outs.append(sim.read_particles(("pos", "vel")))
        sim.close()
    assert np.array_equal(outs[0]["pos"], outs[1]["pos"])
    assert np.array_equal(outs[0]["vel"], outs[1]["vel"])


def test_particles_added_between_updates():
    """Particles added after updates join as an appendix with empty lists."""
    scene = scenes.scaled_block(20, seed=9)
    scene.max_particles = scene.n + 64
    sim, orc = _pair(scene)
    for _ in range(3):
        res, _, _ = _teacher_step(sim, orc)
        _assert_step(res)
    rng = np.random.default_rng(4)
    extra = (rng.uniform(-1, 1, (50, 2)) * 0.5).astype(np.float32)
    sim.add_particles(extra, np.tile(np.float32([[1.0, 2.0]]), (50, 1)))
    for _ in range(3):
        res, _, _ = _teacher_step(sim, orc)
        _assert_step(res)


def test_edge_cases_empty_single_and_outside_grid():
    d = pkg.reference_domain()
    sim = pkg.Simulation(d)
    sim.set_gravity((0.0, -10.0))
    sim.update(float(scenes.DT))  # no particles
    st = sim.get_stats()
    assert st.min_particle_neighbor_count == d.max_neighbors and st.max_particle_neighbor_count == 0
    # Particles outside the box are clamped into border cells (sph.h:456-463);
    # one exactly on a cell edge; two coincident.
    pts = np.array([[-7.0, 0.0], [6.0, 4.0], [0.0, 0.0], [0.3, 0.3], [0.3, 0.3], [-5.0, -2.8125]], np.float32)
    sim.add_particles(pts)
    orc = OracleSim()
    orc.set_gravity(0.0, -10.0)
    orc.add_particles(pts)
    for _ in range(4):
        res, _, _ = _teacher_step(sim, orc)
        _assert_step(res)


def test_dense_cluster_and_bodies():
    """Many particles per cell, every body type, external force."""
    rng = np.random.default_rng(11)
    pts = (rng.normal(0, 0.4, (600, 2))).astype(np.float32)
    d = pkg.reference_domain()
    sim = pkg.Simulation(d)
    orc = OracleSim()
    for s in (sim, orc):
        gpu = s is sim
        s.set_gravity((0.0, -10.0)) if gpu else s.set_gravity(0.0, -10.0)
        for nx, ny, dist in scenes.box_planes(scenes.REF_WIDTH, scenes.REF_HEIGHT):
            s.add_plane((nx, ny), dist) if gpu else s.add_plane(nx, ny, dist)
        s.add_circle((1.5, -1.0), 0.6) if gpu else s.add_circle(1.5, -1.0, 0.6)
        s.add_line_segment((-2.0, -1.5), (-0.5, -2.2)) if gpu else s.add_segment(-2.0, -1.5, -0.5, -2.2)
        box = np.array([[0.5, -2.0], [-0.5, -2.0], [-0.5, -2.4], [0.5, -2.4]], np.float32)
        s.add_polygon(box)
        s.add_external_forces((2.0, 0.0)) if gpu else s.add_external_force(2.0, 0.0)
        s.add_particles(pts)
    for _ in range(6):
        res, _, _ = _teacher_step(sim, orc)
        _assert_step(res)


@pytest.mark.parametrize("lean", [False, True])
def test_cluster_beyond_the_pair_buffers(lean):
    """700 particles within 0.1 of one point, without pressure so that they
    stay together: ~700 in-range pairs each, more than either viscosity
    shape buffers (the chain computes the geometry inline), and delta lists
    of 700 entries."""
    from nbodysimulation_experiment_gb300.simulation import DELTA_WARPS, VISC_WARPS, Params
    params = scenes.scenario_params()
    params[5] = 0.0  # stiffness
    params[6] = 0.0  # near stiffness
    rng = np.random.default_rng(5)
    ang = rng.uniform(0, 2 * np.pi, 700)
    rad = 0.1 * np.sqrt(rng.uniform(0, 1, 700))
    # Centred on a cell corner (cells of 0.3 from (-5, -2.8125)): ~175 per cell.
    pts = np.stack([rad * np.cos(ang) + 0.1, rad * np.sin(ang) - 1.0125], 1).astype(np.float32)
    d = pkg.reference_domain()
    sim = pkg.Simulation(d)
    orc = OracleSim()
    for s in (sim, orc):
        gpu = s is sim
        s.set_params(Params.from_array(params)) if gpu else s.set_params(params)
        s.set_gravity((0.0, -10.0)) if gpu else s.set_gravity(0.0, -10.0)
        for nx, ny, dist in scenes.box_planes(scenes.REF_WIDTH, scenes.REF_HEIGHT):
            s.add_plane((nx, ny), dist) if gpu else s.add_plane(nx, ny, dist)
        s.add_particles(pts)
    sim.update(float(scenes.DT))
    orc.update(float(scenes.DT))
    if lean:
        base = sim.sweep_shape()
        sim.set_sweep_shape((VISC_WARPS[1], base[1], DELTA_WARPS[1], base[3]))
    for _ in range(3):
        res, _, _ = _teacher_step(sim, orc)
        _assert_step(res)


def test_dump_into_given_arrays():
    """sph_dump_state into caller-given arrays (the end-to-end benchmark's
    pinned buffers) gives the same state as a fresh dump."""
    scene = scenes.dam_break_4096()
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    for _ in range(3):
        sim.update(float(scenes.DT))
    want = sim.dump_state()
    out = {k: np.full_like(v, 7) for k, v in want.items() if isinstance(v, np.ndarray)}
    got = sim.dump_state(out=out)
    assert got is out
    for k, v in want.items():
        if isinstance(v, np.ndarray):
            assert np.array_equal(got[k], v), k
    assert got["canonical_count"] == want["canonical_count"] and got["grid"] == want["grid"]
    sim.close()


def test_emitter_matches_reference():
    """Emitters add particles during the update (demo4.cpp:257-284); the
    jitter comes from the C library's rand() in both."""
    d = pkg.reference_domain()
    sim = pkg.Simulation(d)
    orc = OracleSim()
    p = scenes.scenario_params(spacing=np.float32(0.3) / np.float32(4.0))
    sim.set_params(pkg.Params.from_array(p))
    orc.set_params(p)
    for s in (sim, orc):
        gpu = s is sim
        s.set_gravity((0.0, -2.0)) if gpu else s.set_gravity(0.0, -2.0)
        for nx, ny, dist in scenes.box_planes(scenes.REF_WIDTH, scenes.REF_HEIGHT):
            s.add_plane((nx, ny), dist) if gpu else s.add_plane(nx, ny, dist)
        s.add_emitter((-3.5, 0.0), (1.0, 0.0), 0.9, 2.5, 15.0, 30.0) if gpu else \
            s.add_emitter(-3.5, 0.0, 1.0, 0.0, 0.9, 2.5, 15.0, 30.0)
    for step in range(12):
        orc.srand(1000 + step)
        before = sim.dump_state()
        orc.set_state(ostate.to_reference_state(before))
        orc.update(float(scenes.DT))
        orc.srand(1000 + step)
        sim.update(float(scenes.DT))
        after = sim.dump_state()
        assert len(after["pos"]) == orc.particle_count()
        res = ostate.compare_step(before, after, orc.get_state(lists=False))
        _assert_step(res)


def test_read_particles_in_add_order():
    scene = scenes.scaled_block(16, seed=2)
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    for _ in range(5):
        sim.update(float(scenes.DT))
    st = sim.dump_state()
    rd = sim.read_particles(("pos", "vel"))
    assert np.array_equal(rd["pos"], ostate.by_id(st, "pos"))
    assert np.array_equal(rd["vel"], ostate.by_id(st, "vel"))
    assert sim.kernel_launches() > 0


def test_first_update_matches_reference_golden():
    """Bit-identical to the reference solver's own first update (golden
    fixture made on another machine by the reference, tests/golden)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dam_break_4096.npz"))
    scene = scenes.dam_break_4096()
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.update(float(scenes.DT))
    rd = sim.read_particles(("pos", "prev", "vel", "dens", "press"))
    for k in ("pos", "prev", "vel", "dens", "press"):
        assert np.array_equal(rd[k], g["step1_" + k]), k
    cells = ostate.gpu_cells_by_id(sim.dump_state())
    flat = g["step1_cell_flat"]
    off = 0
    for c, cnt in enumerate(g["step1_cell_count"]):
        assert np.array_equal(cells[c], flat[off:off + cnt]), c
        off += cnt
    st = sim.get_stats()
    assert [st.min_particle_neighbor_count, st.max_particle_neighbor_count, st.min_cell_particle_count,
            st.max_cell_particle_count] == list(g["step1_stats"])
