"""The built-in scenarios (SPHScenarios[], sph.h:315-437) as the library
restates them, against the reference's own table and loader steps
(app.cpp:477-534) compiled into the oracle harness: every call's arguments
must be identical, bit for bit.  No GPU needed."""
import ctypes
import numpy as np

import pytest

from nbodysimulation_experiment_gb300 import simulation
from oracle import oracle


@pytest.fixture(scope="module")
def reference():
    oracle.build(reference=True)
    if not oracle.reference_available():
        pytest.skip("the reference tree is not available to build the harness")
    lib = oracle.ReferenceSim.load()
    lib.sphref_scenario_describe.argtypes = [ctypes.c_int, ctypes.POINTER(simulation.ScenarioDesc)]
    lib.sphref_scenario_describe.restype = ctypes.c_int
    lib.sphref_scenario_count.restype = ctypes.c_int
    return lib


def test_same_scenarios_as_the_reference(reference):
    assert simulation.scenario_count() == reference.sphref_scenario_count() == 8
    for k in range(8):
        want = simulation.ScenarioDesc()
        assert reference.sphref_scenario_describe(k, ctypes.byref(want)) == 0
        got = simulation.scenario_describe(k)
        assert got.name == want.name, k
        assert bytes(got) == bytes(want), (k, got.name)


def test_scenario_contents():
    names = [simulation.scenario_describe(k).name.decode() for k in range(8)]
    assert names == ["Dambreak", "Dambreak x 2", "Blob", "Blob x 2", "Liquid", "Glass", "Fontain", "Fun"]
    dam = simulation.scenario_describe(0)
    # Four walls and the dam's wall (a box); the loader walks five volume
    # slots, of which only the first is filled.
    assert dam.body_count == 5 and dam.bodies[4].type == simulation.SPH_BODY_POLYGON
    assert dam.volume_count == 5
    assert (dam.volumes[0].count_x, dam.volumes[0].count_y) == (50, 106)
    assert all(dam.volumes[v].count_x == 0 for v in range(1, 5))
    # The 8-argument SPHParameters constructor keeps kSPHRestDensity.
    assert dam.params.rest_density == 20.0
    fun = simulation.scenario_describe(7)
    assert fun.emitter_count == 1 and fun.body_count == 7
    assert sum(fun.bodies[b].type == simulation.SPH_BODY_PLANE for b in range(7)) == 3  # no top wall


def test_describe_rejects_bad_indices():
    for k in (-1, 8):
        with pytest.raises(simulation.SphError):
            simulation.scenario_describe(k)


@pytest.mark.parametrize("index", range(8))
def test_restatement_runs_every_scenario_like_the_reference(reference, index):
    """Free runs of each built-in scenario, loaded by the same calls into the
    reference's own solver and into the restatement (FP32, one worker), with
    the C library's rand() seeded alike before loading and before every
    update (emitters, volume jitter): identical particles, cell arrays and
    statistics after every update, neighbour lists at the first and last."""
    from oracle.oracle import OracleSim, ReferenceSim
    from oracle.scenario_calls import load_description
    from nbodysimulation_experiment_gb300 import scenes
    d = simulation.scenario_describe(index)
    ref = ReferenceSim(multithreading=False)
    orc = OracleSim()
    for sim in (ref, orc):
        sim.srand(4242 + index)
        load_description(sim, d)
    assert ref.particle_count() == orc.particle_count()
    steps = 20
    for step in range(steps):
        for sim in (ref, orc):
            sim.srand(77 + step)
            sim.update(float(scenes.DT))
        lists = step in (0, steps - 1)
        a, b = ref.get_state(lists=lists), orc.get_state(lists=lists)
        assert len(a["pos"]) == len(b["pos"]), (d.name, step)
        for k in ("pos", "prev", "vel", "dens", "press"):
            assert np.array_equal(a[k], b[k]), (d.name, step, k)
        assert np.array_equal(a["cell_flat"], b["cell_flat"]), (d.name, step)
        if lists:
            assert np.array_equal(a["nb_flat"], b["nb_flat"]), (d.name, step)
        assert np.array_equal(ref.get_stats()[0], orc.get_stats()[0]), (d.name, step)
    assert ref.particle_count() > 0 or d.emitter_count == 0, d.name
