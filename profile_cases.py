"""Small, self-contained workloads for profiling single kernels with a
profiler such as Nsight Compute (each runs a few launches of its kernels on
inputs larger than L2 but a few hundred MB on the device at most).

    python profile_cases.py plain
    python profile_cases.py springs
    python profile_cases.py mpnn
    python profile_cases.py batched
    python profile_cases.py learned_frame
"""
from __future__ import annotations

import os
import sys

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from nbodysimulation_experiment_gb300 import learned, scenes  # noqa: E402
from nbodysimulation_experiment_gb300.simulation import (  # noqa: E402
    DELTA_WARPS, VISC_WARPS, BatchSimulation, Mpnn, Simulation)


def plain(updates: int = 3, warm: int = 20) -> None:
    """The 65,536-particle obstacle scene (the benchmark's workload) with the
    default (wide) sweep shapes: the scene's first update, `warm` updates,
    then `updates` more, so each sweep kernel's launches after the first
    1 + warm are steady-state ones."""
    scene = scenes.obstacles_65536()
    sim = Simulation(scene.domain())
    scene.apply(sim)
    for _ in range(1 + warm + updates):
        sim.update(float(scenes.DT))
    sim.synchronize()
    print("shape", sim.sweep_shape())
    sim.close()


def springs(updates: int = 3) -> None:
    """262,144-particle block with springs (gamma 0.1, alpha 0.3, k 0.3)."""
    scene = scenes.scaled_block(512, seed=3, obstacles=False)
    sim = Simulation(scene.domain())
    scene.apply(sim)
    sim.set_springs(True, yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    for _ in range(updates):
        sim.update(float(scenes.DT))
    sim.synchronize()
    print("springs", sim.spring_count())
    sim.close()


def mpnn(steps: int = 3) -> None:
    """Three training steps of the network on one 65,536-particle frame."""
    model = Mpnn(70000, seed=1)
    learned.collect(model, lambda s: scenes.obstacles_65536(seed=s), (1,), 1)
    for _ in range(steps):
        loss = model.train_step(0, 1e-3)
    print("loss", loss)
    model.close()


def batched(updates: int = 3) -> None:
    """64 scenes of the batched workload's distribution, lean sweep shapes
    (3 viscosity and 8 delta blocks per SM)."""
    mix = scenes.batch_scenes(count=64, seed=11)
    batch = BatchSimulation(mix)
    batch.update(float(scenes.DT))
    sms = batch.sweep_shape()[1] // 4  # the default viscosity shape runs 4 blocks per SM
    batch.set_sweep_shape((VISC_WARPS[1], 3 * sms, DELTA_WARPS[1], 8 * sms))
    for _ in range(updates):
        batch.update(float(scenes.DT))
    batch.synchronize()
    print("particles", batch.get_particle_count())
    batch.close()


def learned_frame(frames: int = 3) -> None:
    """Learned frames (untrained network, judge off) on the 65,536-particle
    obstacle scene."""
    scene = scenes.obstacles_65536()
    sim = Simulation(scene.domain())
    scene.apply(sim)
    sim.update(float(scenes.DT) / 4)
    model = Mpnn(70000, seed=2)
    for _ in range(frames):
        sim.learned_frame(model, float(scenes.DT), 4, bound=1e9)
    sim.synchronize()
    print("frames", frames)
    model.close()
    sim.close()


CASES = {"plain": plain, "springs": springs, "mpnn": mpnn, "batched": batched, "learned_frame": learned_frame}

if __name__ == "__main__":
    CASES[sys.argv[1]]()
