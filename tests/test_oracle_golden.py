"""The oracle (CPU restatement of the reference step) against the golden
fixtures made by the reference's own Demo4 solver (tests/golden/), and --
where the reference tree is present -- against that solver directly.

Bit-exact: FP32 single-worker results must be identical.
"""
import os

import numpy as np
import pytest

from nbodysimulation_experiment_gb300 import scenes
from oracle import oracle
from oracle.oracle import OracleSim

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    oracle.build(reference=True)


def _check(sim, g, prefix):
    st = sim.get_state(lists=False)
    for k in ("pos", "prev", "vel", "dens", "press"):
        assert np.array_equal(st[k].astype(np.float32), g[prefix + k]), (prefix, k)
    assert np.array_equal(st["cell_count"].astype(np.int32), g[prefix + "cell_count"])
    assert np.array_equal(st["cell_flat"].astype(np.int32), g[prefix + "cell_flat"])
    counts, _ = sim.get_stats()
    assert np.array_equal(counts.astype(np.int64), g[prefix + "stats"])


def test_dam_break_golden():
    g = np.load(os.path.join(GOLDEN, "dam_break_4096.npz"))
    scene = scenes.dam_break_4096()
    assert np.array_equal(scene.positions, g["initial_pos"])
    sim = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(sim)
    for step in range(1, 11):
        sim.update(float(scenes.DT))
        if step in (1, 2, 10):
            _check(sim, g, "step%d_" % step)


def test_bodies_golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = np.load(os.path.join(GOLDEN, "bodies_400.npz"))
    pos, box = mg.bodies_scene()
    assert np.array_equal(pos, g["initial_pos"])
    sim = OracleSim()
    mg.apply_bodies(sim, pos, box)
    for _ in range(6):
        sim.update(float(scenes.DT))
    _check(sim, g, "step6_")


def test_params_ctor8_quirk():
    """The 8-argument SPHParameters constructor ignores its kernelHeight and
    restDensity arguments (sph.h:113, 117); the scene helper reproduces it."""
    g = np.load(os.path.join(GOLDEN, "params_ctor8.npz"))
    for a, stored in zip(g["args"], g["stored"]):
        mine = scenes.scenario_params(kernel_height=a[0], cell_size=a[1], spacing=a[2], near_stiffness=a[5])
        assert np.array_equal(mine, stored)


@pytest.mark.skipif(not oracle.reference_tree_present(), reason="reference tree not present")
def test_restatement_matches_reference_build_step_by_step():
    from oracle.oracle import ReferenceSim
    assert oracle.reference_available()
    scene = scenes.dam_break_4096()
    ref = ReferenceSim(multithreading=False)
    orc = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(ref)
    scene.apply(orc)
    for step in range(12):
        ref.update(float(scenes.DT))
        orc.update(float(scenes.DT))
        a = ref.get_state(lists=(step % 6 == 0))
        b = orc.get_state(lists=(step % 6 == 0))
        for k in ("pos", "prev", "vel", "dens", "press"):
            assert np.array_equal(a[k], b[k].astype(np.float32)), (step, k)
        assert np.array_equal(a["cell_flat"], b["cell_flat"])
        if step % 6 == 0:
            assert np.array_equal(a["nb_flat"], b["nb_flat"])
        assert np.array_equal(ref.get_stats()[0], orc.get_stats()[0])


@pytest.mark.skipif(not oracle.reference_tree_present(), reason="reference tree not present")
def test_reference_multithreading_is_racy_but_single_worker_deterministic():
    """The reference's threaded scatter races (demo4.cpp:233-234, 250); only
    its single-worker order is a reproducible oracle."""
    from oracle.oracle import ReferenceSim
    scene = scenes.dam_break_4096()
    outs = []
    for _ in range(2):
        ref = ReferenceSim(multithreading=False)
        scene.apply(ref)
        for _ in range(3):
            ref.update(float(scenes.DT))
        outs.append(ref.get_state(lists=False)["pos"])
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.skipif(not oracle.reference_tree_present(), reason="reference tree not present")
def test_restatement_matches_raised_constant_reference_on_the_65536_scene():
    """The restatement's runtime domain against the reference's own solver
    compiled with raised constants (kSPHBoundaryWidth 51.2, so a 170 x 96
    grid, and room for 65,536 particles; oracle/Makefile): the full
    65,536-particle obstacle scene, first updates from the scene as loaded,
    bit for bit -- grid sizing, clamping, cell arrays and statistics on a box
    other than the reference's 10 x 5.625 one."""
    from oracle.oracle import ReferenceSimBox51
    assert ReferenceSimBox51.available()
    scene = scenes.obstacles_65536()
    ref = ReferenceSimBox51(multithreading=False)
    orc = OracleSim(ReferenceSimBox51.oracle_domain())
    assert (orc.gx, orc.gy) == (ReferenceSimBox51.limits()["gx"], ReferenceSimBox51.limits()["gy"])
    scene.apply(ref)
    scene.apply(orc)
    for step in range(3):
        ref.update(float(scenes.DT))
        orc.update(float(scenes.DT))
        a = ref.get_state(lists=(step == 1))
        b = orc.get_state(lists=(step == 1))
        for k in ("pos", "prev", "vel", "dens", "press"):
            assert np.array_equal(a[k], b[k].astype(np.float32)), (step, k)
        assert np.array_equal(a["cell_count"], b["cell_count"]) and np.array_equal(a["cell_flat"], b["cell_flat"])
        if step == 1:
            assert np.array_equal(a["nb_flat"], b["nb_flat"])
        assert np.array_equal(ref.get_stats()[0], orc.get_stats()[0])
    ref.close()
    orc.close()


@pytest.mark.skipif(not oracle.reference_tree_present(), reason="reference tree not present")
def test_restatement_matches_raised_constant_reference_on_the_1m_block():
    """The same on the 1,048,576-particle block (the reference built with a
    204.8-wide box and room for 1,048,576 particles): the first two updates
    from the block as loaded, bit for bit.  The reference has no springs, so
    this pins the plain step at that size."""
    from conftest import host_memory_gb
    from oracle.oracle import ReferenceSimBox205
    if host_memory_gb() < 40:
        pytest.skip("the reference at 1M particles needs ~10 GB of host memory")
    assert ReferenceSimBox205.available()
    scene = scenes.block_1m()
    ref = ReferenceSimBox205(multithreading=False)
    orc = OracleSim(ReferenceSimBox205.oracle_domain())
    scene.apply(ref)
    scene.apply(orc)
    for step in range(2):
        ref.update(float(scenes.DT))
        orc.update(float(scenes.DT))
    a = ref.get_state(lists=False)
    b = orc.get_state(lists=False)
    for k in ("pos", "prev", "vel", "dens", "press"):
        assert np.array_equal(a[k], b[k].astype(np.float32)), k
    assert np.array_equal(a["cell_count"], b["cell_count"]) and np.array_equal(a["cell_flat"], b["cell_flat"])
    assert np.array_equal(ref.get_stats()[0], orc.get_stats()[0])
    ref.close()
    orc.close()
