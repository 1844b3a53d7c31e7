"""Batched scenes and per-step graphs, through the C ABI.

A batch advances independent scenes with one launch per stage.  Its
contract is that every scene evolves exactly as a single-scene simulation
holding the same scene does -- which the parity tests tie to the reference's
own update -- so each test compares a batch scene against its own
single-scene run, bit for bit, over many updates (the state is compared in
the internal numbering: positions, velocities, densities, ids, cells and the
cell tables).  Graph replay is checked the same way against eager launches.
"""
import ctypes

import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes, simulation
from nbodysimulation_experiment_gb300.simulation import DELTA_WARPS, VISC_WARPS

pytestmark = pytest.mark.gpu

STATE_KEYS = ("pos", "prev", "vel", "acc", "dens", "press", "id", "cell", "cell_start", "cell_count")


def _single_run(scene, steps, graphs=True):
    sim = pkg.Simulation(scene.domain())
    sim.use_graphs(graphs)
    scene.apply(sim)
    for _ in range(steps):
        sim.update(float(scenes.DT))
    st = sim.dump_state()
    stats = sim.get_stats()
    sim.close()
    return st, stats


def _assert_same_state(a, b, what):
    assert a["canonical_count"] == b["canonical_count"], what
    for k in STATE_KEYS:
        assert np.array_equal(a[k], b[k]), (what, k)


def test_batch_scenes_equal_single_scene_runs():
    mix = scenes.batch_scenes(count=5, seed=7, n_min=1024, n_max=6000) + [scenes.dam_break_4096()]
    steps = 40
    batch = pkg.BatchSimulation(mix)
    assert batch.scene_count == len(mix)
    assert batch.get_particle_count() == sum(s.n for s in mix)
    for _ in range(steps):
        batch.update(float(scenes.DT))
    for k, sc in enumerate(mix):
        want, want_stats = _single_run(sc, steps)
        got = batch.dump_state(k)
        _assert_same_state(got, want, sc.name)
        st = batch.get_stats(k)
        for f in ("min_particle_neighbor_count", "max_particle_neighbor_count", "min_cell_particle_count",
                  "max_cell_particle_count"):
            assert getattr(st, f) == getattr(want_stats, f), (sc.name, f)
        rd = batch.read_particles(k)
        pos = np.zeros_like(got["pos"])
        pos[got["id"]] = got["pos"]
        assert np.array_equal(rd["pos"], pos)
    batch.close()


def test_graph_replay_equals_eager_launches():
    scene = scenes.scaled_block(48)
    eager, _ = _single_run(scene, 25, graphs=False)
    graphed, _ = _single_run(scene, 25, graphs=True)
    _assert_same_state(graphed, eager, "graphs")


def test_graph_is_dropped_when_the_scene_changes():
    """Changing gravity, parameters or adding particles between replays must
    take effect in the next update (the captured graph holds none of it)."""
    scene = scenes.scaled_block(32)
    runs = []
    for graphs in (False, True):
        scene.max_particles = scene.n + 64
        sim = pkg.Simulation(scene.domain())
        sim.use_graphs(graphs)
        scene.apply(sim)
        for k in range(12):
            if k == 4:
                sim.set_gravity((1.0, -5.0))
            if k == 7:
                sim.add_particles(np.array([[0.0, 0.0], [0.1, 0.05]], np.float32))
            if k == 9:
                p = sim.get_params()
                p.stiffness = 0.5
                sim.set_params(p)
            sim.update(float(scenes.DT))
        runs.append(sim.dump_state())
        sim.close()
    scene.max_particles = None
    _assert_same_state(runs[1], runs[0], "graph invalidation")


def test_batch_rejects_single_scene_mutators():
    batch = pkg.BatchSimulation(scenes.batch_scenes(count=2, seed=3, n_min=1024, n_max=2048))
    lib = pkg.load_library()
    v = simulation.Vec2(0.0, 0.0)
    idx = ctypes.c_size_t()
    assert lib.sph_add_particle(batch._h, v, v, ctypes.byref(idx)) == simulation.SPH_ERR_NOT_SUPPORTED
    assert lib.sph_set_gravity(batch._h, v) == simulation.SPH_ERR_NOT_SUPPORTED
    assert lib.sph_add_circle(batch._h, v, ctypes.c_float(1.0)) == simulation.SPH_ERR_NOT_SUPPORTED
    st = simulation.Stats()
    assert lib.sph_batch_get_stats(batch._h, 2, ctypes.byref(st)) == simulation.SPH_ERR_INVALID_ARGUMENT
    batch.close()


def test_full_batch_of_512_scenes():
    """The 512-scene workload (log-uniform 1,024..65,536 particles, about 8.1M
    in all): a few updates stay finite and keep every scene's particles, and
    sampled scenes equal their single-scene runs."""
    mix = scenes.batch_scenes()
    steps = 4
    batch = pkg.BatchSimulation(mix)
    for _ in range(steps):
        batch.update(float(scenes.DT))
    batch.synchronize()
    rng = np.random.default_rng(0)
    for k in sorted(rng.choice(len(mix), 3, replace=False).tolist()) + [int(np.argmax([s.n for s in mix]))]:
        got = batch.dump_state(k)
        assert np.all(np.isfinite(got["pos"]))
        assert np.array_equal(np.sort(got["id"]), np.arange(mix[k].n))
        want, _ = _single_run(mix[k], steps)
        _assert_same_state(got, want, mix[k].name)
    batch.close()


def test_autotune_keeps_results_and_state():
    """The autotuner times candidate launch shapes from a snapshot and
    restores it: the trajectory is the same as without tuning."""
    mix = scenes.batch_scenes(count=4, seed=17, n_min=1024, n_max=4096)
    runs = []
    for tune in (False, True):
        batch = pkg.BatchSimulation(mix)
        batch.update(float(scenes.DT))
        if tune:
            shape = batch.autotune(float(scenes.DT))
            assert shape[0] in VISC_WARPS and shape[2] in DELTA_WARPS and shape[1] > 0 and shape[3] > 0
        for _ in range(10):
            batch.update(float(scenes.DT))
        runs.append([batch.dump_state(k) for k in range(len(mix))])
        batch.close()
    for a, b in zip(*runs):
        _assert_same_state(a, b, "autotune")


def _run_with_shape(scene, shape, steps):
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.update(float(scenes.DT))
    if shape is not None:
        sim.set_adaptive_shapes(False)  # run the shape given, dense or not
        base = sim.sweep_shape()
        sim.set_sweep_shape((shape[0], base[1] if shape[1] is None else shape[1],
                             shape[2], base[3] if shape[3] is None else shape[3]))
    for _ in range(steps):
        sim.update(float(scenes.DT))
    st = sim.dump_state()
    sim.close()
    return st


@pytest.mark.parametrize("shape", [(VISC_WARPS[1], None, DELTA_WARPS[1], None),
                                   (VISC_WARPS[1], 152, DELTA_WARPS[0], 152),
                                   (VISC_WARPS[0], 152 * 3, DELTA_WARPS[1], 152 * 5),
                                   (VISC_WARPS[0], 152, DELTA_WARPS[2], 304),
                                   (VISC_WARPS[1], 152 * 3, DELTA_WARPS[3], 152 * 5),
                                   (VISC_WARPS[0], 152, DELTA_WARPS[4], 152 * 4),
                                   (VISC_WARPS[0], 152, DELTA_WARPS[5], 152)])
def test_sweep_shapes_give_identical_results(shape):
    """Lean, mid, tri, quad, wide and dense sweeps, with any resident block
    count, compute the same update."""
    scene = scenes.scaled_block(64, seed=13)
    want = _run_with_shape(scene, None, 12)
    got = _run_with_shape(scene, shape, 12)
    _assert_same_state(got, want, str(shape))


def test_lean_viscosity_with_long_pair_lists():
    """Particles with more in-range pairs than the lean sweep's geometry
    buffer (spacing h/10: ~300 pairs) take the inline path, with the same
    result."""
    h = float(scenes.H)
    pos = scenes.jittered_lattice(28, 28, -1.4, -2.5, spacing=h / 10, jitter=h / 200, seed=3)
    scene = scenes.Scene("dense", scenes.REF_WIDTH, scenes.REF_HEIGHT, pos,
                         scenes.box_planes(scenes.REF_WIDTH, scenes.REF_HEIGHT))
    want = _run_with_shape(scene, None, 6)
    got = _run_with_shape(scene, (VISC_WARPS[1], None, DELTA_WARPS[1], None), 6)
    _assert_same_state(got, want, "dense")
    got = _run_with_shape(scene, (VISC_WARPS[0], None, DELTA_WARPS[5], None), 6)
    _assert_same_state(got, want, "dense, 16-warp delta")
