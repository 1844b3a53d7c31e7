"""Test infrastructure: the calls of a built-in scenario's description
(sph_scenario_describe), made on one of the CPU solvers of oracle.py -- the
reference's own LoadScenario sequence (app.cpp:477-534): ResetStats, the
Clear* calls, SetGravity, SetParams, then the bodies, volumes and emitters in
table order (sph.h:315-437).  Volume and emitter jitter come from the C
library's rand(), so callers seed it (srand) first."""
from nbodysimulation_experiment_gb300 import simulation


def load_description(sim, d) -> None:
    sim.reset_stats()
    sim.clear_bodies()
    sim.clear_particles()
    sim.clear_emitters()
    sim.set_gravity(d.gravity.x, d.gravity.y)
    p = d.params
    sim.set_params([p.kernel_height, p.cell_size, p.particle_spacing, p.inv_kernel_height, p.rest_density,
                    p.stiffness, p.near_stiffness, p.linear_viscosity, p.quadratic_viscosity])
    for b in range(d.body_count):
        o = d.bodies[b]
        if o.type == simulation.SPH_BODY_PLANE:
            sim.add_plane(o.normal.x, o.normal.y, o.distance)
        elif o.type == simulation.SPH_BODY_CIRCLE:
            sim.add_circle(o.center.x, o.center.y, o.radius)
        elif o.type == simulation.SPH_BODY_LINE_SEGMENT:
            sim.add_segment(o.verts[0].x, o.verts[0].y, o.verts[1].x, o.verts[1].y)
        else:
            sim.add_polygon([(o.verts[k].x, o.verts[k].y) for k in range(o.vertex_count)])
    for v in range(d.volume_count):
        o = d.volumes[v]
        sim.add_volume(o.center.x, o.center.y, o.force.x, o.force.y, o.count_x, o.count_y, o.spacing)
    for e in range(d.emitter_count):
        o = d.emitters[e]
        sim.add_emitter(o.position.x, o.position.y, o.direction.x, o.direction.y, o.radius, o.speed, o.rate,
                        o.duration)
