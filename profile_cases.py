"""Small, self-contained workloads for profiling single kernels with a
profiler such as Nsight Compute (each runs a few launches of its kernels on
inputs larger than L2 but a few hundred MB on the device at most).

    python profile_cases.py plain
    python profile_cases.py springs
    python profile_cases.py mpnn
    python profile_cases.py batched
    python profile_cases.py learned_frame
    python profile_cases.py learned_dam    # 262,144-particle dam break, learned frames
    python profile_cases.py block [side]   # side x side block, springs on, lean sweep shapes
    python profile_cases.py dense_shapes   # the shapes taken in dense states
    python profile_cases.py dense_tasks    # delta-sweep task timestamps at update 91 of the 1M collapse
    python profile_cases.py all            # every kernel of the library, small sizes
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


def learned_dam(frames: int = 3) -> None:
    """Learned frames (untrained network, judge on at a bound that accepts
    every frame) on the 262,144-particle dam break with obstacles, the
    benchmark's learned-frame scene, after 4 plain updates."""
    scene = scenes.dam_break_262144()
    sim = Simulation(scene.domain())
    scene.apply(sim)
    for _ in range(4):
        sim.update(float(scenes.DT) / 4)
    model = Mpnn(scene.n + 128, seed=2)
    for _ in range(frames):
        sim.learned_frame(model, float(scenes.DT), 4, bound=1e9)
    sim.synchronize()
    print("frames", frames)
    model.close()
    sim.close()


def block(side: int = 512, updates: int = 3) -> None:
    """A side x side jittered block with springs on (yield 0.1, plasticity
    0.3, stiffness 0.3, at most 16), in the sweep shapes the autotuner picks
    for the 1,048,576-particle block (lean 5-warp viscosity at 3 blocks per
    SM, pipelined 3-warp delta at 5 per SM): 3 + `updates` updates."""
    scene = scenes.block_1m() if side == 1024 else scenes.scaled_block(side, seed=3, obstacles=False)
    sim = Simulation(scene.domain())
    scene.apply(sim)
    sim.set_springs(True, yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    for _ in range(3):
        sim.update(float(scenes.DT))
    sms = sim.sweep_shape()[3]  # the default delta shape runs one block per SM
    sim.set_sweep_shape((VISC_WARPS[1], 3 * sms, DELTA_WARPS[3], 5 * sms))
    for _ in range(updates):
        sim.update(float(scenes.DT))
    sim.synchronize()
    print("particles", scene.n, "springs", sim.spring_count())
    sim.close()


def dense_shapes(side: int = 256, updates: int = 2) -> None:
    """A side x side block with springs on in the shapes the library takes
    for dense states (wide viscosity, 16-warp delta), after 3 updates."""
    scene = scenes.scaled_block(side, seed=5, obstacles=False)
    sim = Simulation(scene.domain())
    scene.apply(sim)
    sim.set_springs(True, yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    for _ in range(3):
        sim.update(float(scenes.DT))
    sms = sim.sweep_shape()[3]  # the default delta shape runs one block per SM
    sim.set_adaptive_shapes(False)
    sim.set_sweep_shape((VISC_WARPS[0], 4 * sms, DELTA_WARPS[5], sms))
    for _ in range(updates):
        sim.update(float(scenes.DT))
    sim.synchronize()
    sim.close()


def dense_tasks(update: int = 91) -> None:
    """Task timestamps (sph_profile_tasks) of the delta sweep on the
    1,048,576-particle block with springs at the given update of its collapse,
    in the shapes the library picks there, under the full grid and with a
    single block (the same tasks one after another): sweep time, total task
    time, time spent staging, and the slowest tasks."""
    import ctypes
    import json
    import numpy as np
    from nbodysimulation_experiment_gb300 import simulation as sm
    lib = sm.load_library()
    lib.sph_profile_tasks.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.sph_profile_read.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                     ctypes.POINTER(ctypes.c_size_t)]
    scene = scenes.block_1m()
    sim = Simulation(scene.domain())
    scene.apply(sim)
    sim.set_springs(True, yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    for k in range(update):
        if k == 5:
            sim.autotune(float(scenes.DT))
        sim.update(float(scenes.DT))
    shape = sim.last_sweep_shape()
    st0, sp0 = sim.dump_state(), sim.dump_springs()
    sim.set_adaptive_shapes(False)
    out = {"update": update, "shape": list(shape)}
    for label, blocks in (("full_grid", shape[3]), ("one_block", 1)):
        sim.load_state(st0)
        sim.load_springs(*sp0)
        sim.set_sweep_shape((shape[0], shape[1], shape[2], blocks))
        lib.sph_profile_tasks(sim._h, 1)
        sim.update(float(scenes.DT))
        sim.synchronize()
        stride = ctypes.c_size_t()
        lib.sph_profile_read(sim._h, None, 0, ctypes.byref(stride))
        buf = np.zeros(8 * stride.value, np.uint64)
        lib.sph_profile_read(sim._h, buf.ctypes.data, buf.size, ctypes.byref(stride))
        lib.sph_profile_tasks(sim._h, 0)
        a = buf[4 * stride.value:8 * stride.value].reshape(-1, 4).astype(np.float64)  # the delta sweep
        a = a[a[:, 3] > 0]
        ready = np.where(a[:, 1] > 0, a[:, 1], a[:, 0])
        run, stage = (a[:, 3] - ready) / 1e3, (a[:, 2] - ready) / 1e3
        span = (a[:, 3].max() - a[:, 0].min()) / 1e3
        out[label] = {"delta_ms": sim.get_stats().time_delta_positions, "tasks": int(len(a)),
                      "task_time_s": float(run.sum() / 1e6), "staging_s": float(stage.sum() / 1e6),
                      "tasks_in_flight": float(run.sum() / span),
                      "slowest_tasks_us": [round(float(x), 1) for x in np.sort(run)[-5:][::-1]]}
    print(json.dumps(out))
    sim.close()


def everything() -> None:
    """Every kernel the library launches, on small cases: the plain step
    (wide shapes), the springs block (lean shapes), training steps, learned
    frames, a small batch and the host-facing reads."""
    plain(updates=2, warm=4)
    block(side=512, updates=2)
    dense_shapes(side=256, updates=2)
    mpnn(steps=2)
    learned_frame(frames=2)
    batched(updates=2)
    scene = scenes.dam_break_4096()
    sim = Simulation(scene.domain())
    scene.apply(sim)
    sim.set_springs(True, yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    sim.update(float(scenes.DT))
    sim.read_particles(("pos", "vel"))
    sim.particle_colors()
    sim.render_points(320, 180)
    st, spr = sim.dump_state(), sim.dump_springs()  # snapshot: device-side checks on load
    sim.load_state(st)
    sim.load_springs(*spr)
    sim.set_reference_order(True)  # the reference-order sweeps
    for _ in range(2):
        sim.update(float(scenes.DT))
    sim.synchronize()
    sim.close()
    import ctypes
    import torch
    from nbodysimulation_experiment_gb300 import simulation as sm
    lib = sm.load_library()
    fn = lib.sph_density_pressure_noalloc
    fn.argtypes = [ctypes.POINTER(sm.Domain), ctypes.POINTER(sm.Params), ctypes.c_void_p, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    pos = torch.from_numpy(scene.positions).cuda()
    out = torch.empty((2, scene.n, 2), device="cuda")
    d, p = scene.domain(), sm.Params.from_array(scene.params)
    fn(ctypes.byref(d), ctypes.byref(p), pos.data_ptr(), scene.n, out[0].data_ptr(), out[1].data_ptr(), None)
    torch.cuda.synchronize()
    print("all cases ran")


CASES = {"plain": plain, "springs": springs, "mpnn": mpnn, "batched": batched, "learned_frame": learned_frame,
         "learned_dam": learned_dam, "block": block,
         "dense_shapes": dense_shapes, "dense_tasks": dense_tasks, "all": everything}

if __name__ == "__main__":
    CASES[sys.argv[1]](*[int(a) for a in sys.argv[2:]])
