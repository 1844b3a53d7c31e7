"""The reference's built-in scenarios loaded through the C ABI
(sph_load_scenario, DemoApplication::LoadScenario, app.cpp:477-534) on the
GPU, against the same calls on the oracle: identical particles after
loading (volume and emitter jitter come from the C library's rand() in both)
and one-step parity for the first updates, emitters included: cell arrays
identical, positions and velocities bit for bit."""
import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes, simulation
from oracle import state as ostate
from oracle.oracle import OracleSim
from oracle.scenario_calls import load_description

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("index", range(8))
def test_scenario_loads_and_steps_like_the_reference(index):
    d = simulation.scenario_describe(index)
    sim = pkg.Simulation(pkg.reference_domain())
    orc = OracleSim()
    orc.srand(4242 + index)
    sim.load_scenario(index)
    n_gpu = sim.get_particle_count()
    orc.srand(4242 + index)
    load_description(orc, d)
    assert n_gpu == orc.particle_count()
    if n_gpu:
        rd = sim.read_particles(("pos", "vel"))
        want = orc.get_state(lists=False)
        assert np.array_equal(rd["pos"], want["pos"][:n_gpu]), d.name
    steps = 6 if d.emitter_count else 3
    for step in range(steps):
        before = sim.dump_state()
        orc.set_state(ostate.to_reference_state(before))
        orc.srand(77 + step)
        orc.update(float(scenes.DT))
        orc.srand(77 + step)
        sim.update(float(scenes.DT))
        after = sim.dump_state()
        assert len(after["pos"]) == orc.particle_count(), (d.name, step)
        if len(after["pos"]) == 0:
            continue
        res = ostate.compare_step(before, after, orc.get_state(lists=False))
        assert res["cells_equal"] == 1.0, (d.name, step, res)
        # Positions and velocities bit for bit, as in the other parity tests.
        assert res["pos_ulp"] == 0 and res["vel_ulp"] == 0, (d.name, step, res)
        for k in ("prev", "dens", "press"):
            assert res[k + "_rel"] <= 1e-5 or res[k + "_ulp"] <= 4, (d.name, step, k, res)
    sim.close()
