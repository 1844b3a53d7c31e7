"""Generate the golden fixtures from the reference's own Demo4 solver.

Run in a checkout where the reference tree is available (it builds
oracle/_ref/libsphref.so from it):  python tests/golden/make_golden.py

Fixtures (small .npz files, committed):

* dam_break_4096.npz -- the seeded 4,096-particle dam break
  (nbodysimulation_experiment_gb300.scenes.dam_break_4096) advanced by the
  reference for 1, 2 and 10 updates from the scene as loaded: positions,
  velocities, densities, pressures, cell arrays and statistics.
* bodies_400.npz -- a 20x20 block falling onto every body type (planes,
  circle, line segment, polygon) with an external force, 6 updates.
* params_ctor8.npz -- what the 8-argument SPHParameters constructor stores
  (sph.h:112-122) for the scenario table's argument lists.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from nbodysimulation_experiment_gb300 import scenes  # noqa: E402
from oracle import oracle  # noqa: E402


def snapshot(sim, prefix, out):
    st = sim.get_state(lists=False)
    for k in ("pos", "prev", "vel", "dens", "press"):
        out[prefix + k] = st[k].astype(np.float32)
    out[prefix + "cell_count"] = st["cell_count"].astype(np.int32)
    out[prefix + "cell_flat"] = st["cell_flat"].astype(np.int32)
    counts, _ = sim.get_stats()
    out[prefix + "stats"] = counts.astype(np.int64)


def bodies_scene():
    pos = scenes.jittered_lattice(20, 20, -1.0, 0.5, seed=77)
    box = np.array([[0.5, -2.0], [-0.5, -2.0], [-0.5, -2.4], [0.5, -2.4]], np.float32)
    return pos, box


def apply_bodies(sim, pos, box):
    sim.reset_stats()
    sim.clear_bodies()
    sim.clear_particles()
    sim.clear_emitters()
    sim.set_gravity(0.0, -10.0)
    sim.set_params(scenes.scenario_params())
    for nx, ny, d in scenes.box_planes(scenes.REF_WIDTH, scenes.REF_HEIGHT):
        sim.add_plane(nx, ny, d)
    sim.add_circle(0.6, -0.8, 0.5)
    sim.add_segment(-2.0, -1.5, -0.5, -2.2)
    sim.add_polygon(box)
    sim.add_external_force(1.0, 0.0)
    sim.add_particles(pos)


def main():
    oracle.build(reference=True)
    if not oracle.reference_available():
        raise SystemExit("the reference harness could not be built (reference tree missing)")
    dt = float(scenes.DT)

    scene = scenes.dam_break_4096()
    ref = oracle.ReferenceSim(multithreading=False)
    scene.apply(ref)
    out = {"initial_pos": scene.positions}
    for step in range(1, 11):
        ref.update(dt)
        if step in (1, 2, 10):
            snapshot(ref, "step%d_" % step, out)
    np.savez_compressed(os.path.join(HERE, "dam_break_4096.npz"), **out)

    pos, box = bodies_scene()
    ref = oracle.ReferenceSim(multithreading=False)
    apply_bodies(ref, pos, box)
    out = {"initial_pos": pos, "polygon": box}
    for step in range(1, 7):
        ref.update(dt)
    snapshot(ref, "step6_", out)
    np.savez_compressed(os.path.join(HERE, "bodies_400.npz"), **out)

    h = np.float32(6.0) * np.float32(0.05)
    args = []
    for spacing_div, near in ((6.0, 6.0), (3.0, 12.0), (4.0, 6.0), (4.0, 3.6), (4.0, 1.2)):
        args.append([h, h, h / np.float32(spacing_div), 20.0, 0.6, np.float32(near), 0.5, 0.3])
    args = np.array(args, np.float32)
    stored = np.stack([oracle.ReferenceSim.params_from_ctor8(a) for a in args])
    np.savez_compressed(os.path.join(HERE, "params_ctor8.npz"), args=args, stored=stored)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
