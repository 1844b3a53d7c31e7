"""The reference's built-in scenarios loaded through the C ABI
(sph_load_scenario, DemoApplication::LoadScenario, app.cpp:477-534) on the
GPU, against the same calls on the oracle: identical particles after
loading (volume and emitter jitter come from the C library's rand() in both)
and one-step parity for the first updates, emitters included."""
import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes, simulation
from oracle import state as ostate
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu


def _load_oracle(orc, d):
    """The calls of the scenario description, on the oracle."""
    orc.reset_stats()
    orc.clear_bodies()
    orc.clear_particles()
    orc.clear_emitters()
    orc.set_gravity(d.gravity.x, d.gravity.y)
    p = d.params
    orc.set_params([p.kernel_height, p.cell_size, p.particle_spacing, p.inv_kernel_height, p.rest_density,
                    p.stiffness, p.near_stiffness, p.linear_viscosity, p.quadratic_viscosity])
    for b in range(d.body_count):
        o = d.bodies[b]
        if o.type == simulation.SPH_BODY_PLANE:
            orc.add_plane(o.normal.x, o.normal.y, o.distance)
        elif o.type == simulation.SPH_BODY_CIRCLE:
            orc.add_circle(o.center.x, o.center.y, o.radius)
        elif o.type == simulation.SPH_BODY_LINE_SEGMENT:
            orc.add_segment(o.verts[0].x, o.verts[0].y, o.verts[1].x, o.verts[1].y)
        else:
            orc.add_polygon([(o.verts[k].x, o.verts[k].y) for k in range(o.vertex_count)])
    for v in range(d.volume_count):
        o = d.volumes[v]
        orc.add_volume(o.center.x, o.center.y, o.force.x, o.force.y, o.count_x, o.count_y, o.spacing)
    for e in range(d.emitter_count):
        o = d.emitters[e]
        orc.add_emitter(o.position.x, o.position.y, o.direction.x, o.direction.y, o.radius, o.speed, o.rate,
                        o.duration)


@pytest.mark.parametrize("index", range(8))
def test_scenario_loads_and_steps_like_the_reference(index):
    d = simulation.scenario_describe(index)
    sim = pkg.Simulation(pkg.reference_domain())
    orc = OracleSim()
    orc.srand(4242 + index)
    sim.load_scenario(index)
    n_gpu = sim.get_particle_count()
    orc.srand(4242 + index)
    _load_oracle(orc, d)
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
        assert res["pos_rel"] <= 1e-5 and res["vel_rel"] <= 1e-5, (d.name, step, res)
    sim.close()
