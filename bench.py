"""Benchmark of the GB300 Demo4 SPH step (one JSON line on rank 0).

Headline workload (one "step" = one ``Update`` of the whole scene):
``block_1m_springs`` -- a 1024x1024 jittered lattice (1,048,576 particles,
spacing h/6, uniform jitter +-0.1h) in a 204.8 x 115.2 box with four walls,
gravity (0, -10), the reference's sph.h constants, FP32, with viscoelastic
springs on (yield ratio 0.1, plasticity 0.3, spring stiffness 0.3, at most 16
springs per particle in fixed-capacity int32/float tables).

* ``value``: particle-steps/s with the scene resident in HBM; each timed step
  is bracketed by CUDA events on the simulation's stream, and L2 is flushed
  (a 256 MiB write) between steps, outside the events.
* ``e2e``: the same metric through the C ABI with host buffers: every step
  loads the full state and the spring tables from pinned host memory
  (``sph_load_state``, ``sph_load_springs``), updates, and reads the state
  and the spring tables back into pinned host memory (``sph_dump_state``,
  ``sph_dump_springs``).
* ``roofline``: the dominant kernel of the step (the slower of the two ordered
  sweeps) against the measured HBM copy bandwidth; achieved = its algorithmic
  bytes (24 B per particle: read position and velocity or pressure, write
  velocity or position) / its event-timed duration.  ``roofline.step`` puts
  the whole step's algorithmic bytes (480 B per particle-step with springs)
  over the step time.
* ``cpu_baseline``: the CPU restatement of the reference step (oracle/),
  multithreaded like the reference's ThreadPool on all host cores, on a
  bounded sample of the same workload.

Further objects in the same line (other configurations and forms of the step):

* ``obstacles_65536``: the 65,536-particle scene (256x256 block, 51.2 x 28.8
  box, walls, 8 circles, 4 segments), plain step, with its own e2e and
  roofline.
* ``block_1m_plain``: the 1,048,576-particle block without springs.
* ``batched``: 512 independent scenes (log-uniform 1,024..65,536 particles,
  ~8.1M in all) advanced by one update per step from the per-step CUDA graph,
  sweep shapes chosen by the autotuner.
* ``long_runs``: a free run of 1,000 updates of ``obstacles_65536`` from
  the scene's start (config 2's length), timed in blocks of 100 updates.
  The 1,048,576-particle column exceeds the reference's own neighbour
  capacity after ~110 updates, so its lines reload the scene from its state
  after update 3 every 87 updates, outside the timed region (``restarts``).
* ``learned``: the message-passing network trained on the GPU on plain
  frames of seeded 65,536-particle scenes, then learned frames on a
  262,144-particle dam break with obstacles against plain frames (four
  updates of dt/4), under the density-deviation judge.

``--impl reference`` times that CPU implementation alone on the headline
workload (rank 0 only).  Multi-GPU runs are independent replicas (the step
does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (1 GB300) plain vs batched vs learned at stated density error"
UNIT = "particle-steps/s"
SWEEP_BYTES_PER_PARTICLE = 24  # viscosity: read pos + vel, write vel; delta: read pos + pressure, write pos
STEP_BYTES_PLAIN = 224         # whole plain step, compulsory HBM bytes per particle-step
STEP_BYTES_SPRINGS = 480       # with 16 spring slots (int32 partner + float rest length), read and written
SPRINGS = dict(yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)

WORKLOADS = {
    "block_1m_springs": ("block_1m", True,
                         "block_1m_springs: 1,048,576-particle 1024x1024 jittered lattice (spacing h/6) in a "
                         "204.8 x 115.2 box, 4 walls, viscoelastic springs on (yield 0.1, plasticity 0.3, "
                         "stiffness 0.3, <= 16 per particle), FP32"),
    "obstacles_65536": ("obstacles_65536", False,
                        "obstacles_65536: 65,536-particle jittered block (spacing h/6) in a 51.2 x 28.8 box, "
                        "4 walls + 8 circles + 4 segments, plain Demo4 step (viscosity on, springs off), FP32"),
    "block_1m_plain": ("block_1m", False,
                       "block_1m_plain: 1,048,576-particle 1024x1024 jittered lattice (spacing h/6) in a "
                       "204.8 x 115.2 box, 4 walls, plain Demo4 step (springs off), FP32"),
}
HEADLINE = "block_1m_springs"

# A 1024x1024 column collapsing under gravity compresses to ~2.9x the rest
# density at its foot: by update 100 a particle has 985 neighbours, and after
# ~110 updates the scene exceeds the reference's own capacity of 1,000
# neighbours per particle (kSPHMaxParticleNeighborCount, sph.h:69).  The
# benchmark therefore reloads such a scene from its state after update 3
# (outside the timed region) before it reaches this many updates.
RESTART_AFTER = {"block_1m_springs": 90, "block_1m_plain": 90}

STAGES = ("time_integration", "time_viscosity_forces", "time_predict", "time_update_grid",
          "time_neighbor_search", "time_density_and_pressure", "time_delta_positions", "time_collisions")
STAGE_KEYS = {"time_neighbor_search": "springs"}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def job_seconds(local_s, world, device):
    """Duration of a timed region for the whole job: the maximum over ranks
    (independent replicas, so the job ends with its slowest one)."""
    if world <= 1:
        return float(local_s)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(local_s)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(particles, steps, world, seconds):
    """Whole-job particle-steps/s: every rank advances its own replica of
    ``particles`` by ``steps`` updates within ``seconds``."""
    return particles * steps * world / seconds


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(kernel: str, n_particles: int):
    """DRAM bytes per launch of `kernel` from the committed ncu summaries
    (captured on a smaller case of the same kernel and shape, scaled by
    particle count), or None."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d[kernel]["dram_bytes_per_particle"]) * n_particles
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_memory_gb() -> float:
    """Memory this process may use, in GB (host availability, capped by the
    control group's limit where one is set)."""
    avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    for path in ("/sys/fs/cgroup/memory.max", "/sys/fs/cgroup/memory/memory.limit_in_bytes"):
        try:
            with open(path) as f:
                v = f.read().strip()
            if v.isdigit():
                avail = min(avail, int(v))
        except OSError:
            pass
    return avail / 1e9


# Host memory the CPU restatement needs per particle: the reference's layout
# (1,000 neighbour slots of 8 bytes per particle, 500 per cell).
ORACLE_BYTES_PER_PARTICLE = 9000


def make_scene(workload: str):
    from nbodysimulation_experiment_gb300 import scenes
    name, springs, desc = WORKLOADS[workload]
    return getattr(scenes, name)(), springs, desc


def cpu_port_rate(scene, springs: bool, workers: int, min_updates: int, budget_s: float, warm_updates: int = 1):
    """Time the CPU restatement of the reference step (multithreaded like the
    reference's ThreadPool) on the scene from its start: the first update
    (AddParticle order) and `warm_updates` more untimed, then updates until
    `min_updates` ran and `budget_s` passed.  Returns (particle-steps/s,
    updates timed, seconds)."""
    from nbodysimulation_experiment_gb300 import scenes
    from oracle.oracle import OracleSim
    orc = OracleSim(scene.oracle_domain(OracleSim), fp64=False, workers=workers)
    scene.apply(orc)
    if springs:
        orc.set_springs(True, **SPRINGS)
    dt = float(scenes.DT)
    for _ in range(1 + warm_updates):
        orc.update(dt)
    t0 = time.perf_counter()
    k = 0
    while k < min_updates or time.perf_counter() - t0 < budget_s:
        orc.update(dt)
        k += 1
    sec = time.perf_counter() - t0
    orc.close()
    return scene.n * k / sec, k, sec


def run_reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from nbodysimulation_experiment_gb300 import scenes
    from oracle.oracle import OracleSim, build as build_oracle
    build_oracle(reference=False)
    scene, springs, desc = make_scene(args.workload)
    need = 2.0 * ORACLE_BYTES_PER_PARTICLE * scene.n / 1e9
    if host_memory_gb() < need:
        print(json.dumps({"impl": "reference", "unavailable": "the CPU step at %d particles needs ~%.0f GB of host "
                          "memory; %.0f GB available" % (scene.n, need, host_memory_gb())}), flush=True)
        return 0
    workers = OracleSim.hardware_threads()
    dt = float(scenes.DT)
    restart_after = RESTART_AFTER.get(args.workload)

    def fresh():
        # The scene from its start: the first update in AddParticle order,
        # then two more (the GPU arm's snapshot point).
        o = OracleSim(scene.oracle_domain(OracleSim), fp64=False, workers=workers)
        scene.apply(o)
        if springs:
            o.set_springs(True, **SPRINGS)
        for _ in range(3):
            o.update(dt)
        return o

    orc = fresh()
    done, restarts = 3, 0
    per = max(1, args.cpu_steps // max(1, args.steps)) if args.workload not in RESTART_AFTER else 1

    def restart_if_due():
        # The same window as the GPU arm: the scene restarts (outside the
        # timed region) before it outgrows the reference's capacities.
        nonlocal orc, done, restarts
        if restart_after is not None and done >= restart_after:
            orc.close()
            orc = fresh()
            done = 3
            restarts += 1

    for _ in range(max(0, args.warmup - 3)):
        restart_if_due()
        orc.update(dt)
        done += 1
    times = []
    for _ in range(args.steps):
        restart_if_due()
        t0 = time.perf_counter()
        for _ in range(per):
            orc.update(dt)
        times.append(time.perf_counter() - t0)
        done += per
    orc.close()
    total = sum(times)
    value = scene.n * per * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / (per * args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": {"workload": desc, "particles": scene.n, "springs": springs},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                         "sample": "%d update(s) of the %d-particle scene per step, %d steps, after %d warm-up "
                                   "updates from the scene's start%s" % (
                                       per, scene.n, args.steps, max(3, args.warmup),
                                       "; restarted from update 3 before update %d (%d restarts), as the GPU arm"
                                       % (restart_after, restarts) if restart_after is not None else "")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def sweep_kernels(shape):
    """Kernel names of the two ordered sweeps for a launch shape
    (viscosity warps, blocks, delta warps, blocks)."""
    visc = "k_viscosity_multi<ViscLean>" if shape[0] == 5 else "k_viscosity<ViscWide>"
    delta = {12: "k_delta<DeltaWide>", 8: "k_delta<DeltaMid>", 2: "k_delta<DeltaLean>", 3: "k_delta<DeltaTri>",
             4: "k_delta<DeltaQuad>", 16: "k_delta<DeltaDense>"}.get(shape[2], "k_delta")
    return visc, delta


def pinned_like(torch, arrays):
    out = {}
    for k, a in arrays.items():
        t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32, pin_memory=True)
        out[k] = t.numpy()
        out[k][...] = a
    return out


STATE_KEYS = ("pos", "prev", "vel", "acc", "dens", "press", "id", "cell", "cell_start", "cell_count")


def measure_scene(torch, pkg, workload: str, device: int, steps: int, warmup: int, world: int, flush,
                  e2e_steps: int, clocks: bool = False):
    """One configuration of the plain (or springs) step: device-resident
    event-timed updates with L2 flushed between them, per-stage times, the
    dominant sweep's roofline, and the end-to-end rate through the C ABI with
    pinned host buffers."""
    from nbodysimulation_experiment_gb300 import scenes
    scene, springs, desc = make_scene(workload)
    sim = pkg.Simulation(scene.domain(), device=device)
    scene.apply(sim)
    if springs:
        sim.set_springs(True, **SPRINGS)
    dt = float(scenes.DT)
    stream = torch.cuda.ExternalStream(sim.stream())
    restart_after = RESTART_AFTER.get(workload)
    done = 0
    for _ in range(3):
        sim.update(dt)
        done += 1
    restart_state = sim.dump_state()
    restart_springs = sim.dump_springs() if springs else None
    restarts = 0

    def restart_if_due():
        nonlocal done, restarts
        if restart_after is not None and done >= restart_after:
            sim.load_state(restart_state)
            if springs:
                sim.load_springs(*restart_springs)
            done = 3
            restarts += 1

    for _ in range(max(0, warmup - 3)):
        restart_if_due()
        sim.update(dt)
        done += 1
    sim.synchronize()
    tuned = sim.autotune(dt)

    launches0 = sim.kernel_launches()
    sampler = ClockSampler(device) if clocks else None
    if sampler:
        sampler.start()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    step_ms = []
    stage_sum = dict.fromkeys(STAGES, 0.0)
    # States for the end-to-end part, spread over the timed window (taken
    # after the step's events, outside the timed region).
    n_e2e_states = min(4, steps)
    e2e_at = {(steps * (q + 1)) // n_e2e_states - 1 for q in range(n_e2e_states)}
    e2e_states = []
    for k in range(steps):
        restart_if_due()
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        sim.update(dt)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        done += 1
        step_ms.append(e0.elapsed_time(e1))
        stats = sim.get_stats()
        for key in STAGES:
            stage_sum[key] += getattr(stats, key)
        if k in e2e_at:
            st = sim.dump_state()
            host = pinned_like(torch, {key: st[key] for key in STATE_KEYS})
            host["canonical_count"] = st["canonical_count"]
            host["grid"] = st["grid"]
            if springs:
                cnt, part, rest = sim.dump_springs()
                host["springs"] = pinned_like(torch, {"count": cnt, "partner": part, "rest": rest})
            e2e_states.append((done, host))
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clock_rec = sampler.stop() if sampler else None
    sim_last_shape = sim.last_sweep_shape()  # the shapes of the last timed update (adaptive in dense states)
    launches = sim.kernel_launches() - launches0
    total_s = job_seconds(sum(step_ms) / 1e3, world, "cuda")
    value = job_rate(scene.n, steps, world, total_s)
    stage_ms = {STAGE_KEYS.get(k, k[5:]): v / steps for k, v in stage_sum.items()}

    rd = sim.read_particles(("dens",))
    rho0 = float(scene.params[4])
    dens_err = float(np.mean(np.abs(rd["dens"][:, 0] - rho0)) / rho0)
    spring_count = sim.spring_count() if springs else None

    # --- end to end through the C ABI with host buffers ---------------------
    # Every step loads one of the window's states from pinned host memory,
    # updates it and reads it back; each state takes an equal share of the
    # steps, after two untimed steps that let the sweep shapes settle on it.
    e2e_from = [u for u, _ in e2e_states]
    first = e2e_states[0][1]
    host_out = pinned_like(torch, {key: first[key] for key in STATE_KEYS})
    h2d = sum(first[key].nbytes for key in STATE_KEYS)
    springs_out = None
    if springs:
        springs_out = pinned_like(torch, dict(first["springs"]))
        h2d += sum(a.nbytes for a in first["springs"].values())

    def e2e_step(host):
        sim.load_state(host)
        if springs:
            sp = host["springs"]
            sim.load_springs(sp["count"], sp["partner"], sp["rest"])
        sim.update(dt)
        sim.dump_state(out=host_out)
        if springs:
            sim.dump_springs(out=springs_out)

    per_state = max(1, -(-e2e_steps // len(e2e_states)))
    e2e_local = 0.0
    for _, host in e2e_states:
        for _ in range(2):
            e2e_step(host)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(per_state):
            e2e_step(host)
        e2e_local += time.perf_counter() - t0
    e2e_steps = per_state * len(e2e_states)
    if world > 1:
        dist.barrier()
    e2e_s = job_seconds(e2e_local, world, "cuda")
    e2e_value = job_rate(scene.n, e2e_steps, world, e2e_s)
    sim.close()

    hbm, peak_kind = measured_peaks()
    visc_k, delta_k = sweep_kernels(sim_last_shape)
    if stage_ms["delta_positions"] >= stage_ms["viscosity_forces"]:
        kern, kms = delta_k, stage_ms["delta_positions"]
    else:
        kern, kms = visc_k, stage_ms["viscosity_forces"]
    alg = SWEEP_BYTES_PER_PARTICLE * scene.n
    achieved = alg / (kms / 1e3) / 1e9
    step_bytes = STEP_BYTES_SPRINGS if springs else STEP_BYTES_PLAIN
    mean_ms = statistics.mean(step_ms)
    step_gbs = step_bytes * scene.n / (mean_ms / 1e3) / 1e9
    out = {
        "workload": desc, "value": value, "unit": UNIT, "ms_per_step": mean_ms, "steps": steps, "warmup": warmup,
        "particles": scene.n, "springs": springs, "gpu_launches": int(launches),
        "sweep_shape": {"viscosity_warps": tuned[0], "viscosity_blocks": tuned[1], "delta_warps": tuned[2],
                        "delta_blocks": tuned[3],
                        "last_update": {"viscosity_warps": sim_last_shape[0], "viscosity_blocks": sim_last_shape[1],
                                        "delta_warps": sim_last_shape[2], "delta_blocks": sim_last_shape[3]},
                        "note": "autotuned after the warm-up; in dense states (long neighbour lists, crowded "
                                "cells) the library runs the staging-safe shapes instead (sph_set_adaptive_shapes)"},
        "stage_ms": stage_ms, "density_error": dens_err,
        "restarts": {"after_updates": restart_after, "count": restarts,
                     "why": "the collapsing 1024x1024 column exceeds the reference's 1,000-neighbour capacity "
                            "(sph.h:69) after ~110 updates; the scene is reloaded from its update-3 state, "
                            "outside the timed region"} if restart_after is not None else None,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(h2d),
                "steps": e2e_steps,
                "states": "the states after updates %s of the timed window, an equal share of the steps each "
                          "(after two untimed steps per state), loaded from pinned host memory every step"
                          % ", ".join(str(u) for u in e2e_from)},
        "roofline": {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": profile_traffic(kern, scene.n),
                     "algorithmic_bytes": alg, "kernel_ms": kms,
                     "step": {"bytes_per_particle_step": step_bytes, "achieved": step_gbs,
                              "frac": step_gbs / hbm}},
    }
    if springs:
        out["spring_count"] = spring_count
    if clock_rec is not None:
        out["clocks"] = clock_rec
    return out


def long_run(torch, pkg, workload: str, device: int, steps: int, block: int = 100):
    """A free run of `steps` updates from the scene's start (config 2 is
    specified over 1,000 steps): event-timed in blocks of `block` updates on
    the simulation's stream, after the autotuner has picked the sweep shapes
    on the scene's first updates.  Reports the mean over the whole run and
    per block, so that the cost of the later, denser states shows."""
    scene, springs, _ = make_scene(workload)
    sim = pkg.Simulation(scene.domain(), device=device)
    scene.apply(sim)
    if springs:
        sim.set_springs(True, **SPRINGS)
    dt = float(scenes_module().DT)
    stream = torch.cuda.ExternalStream(sim.stream())
    for _ in range(3):
        sim.update(dt)
    sim.autotune(dt)
    blocks = []
    done = 3
    while done < steps:
        k = min(block, steps - done)
        with torch.cuda.stream(stream):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        for _ in range(k):
            sim.update(dt)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        blocks.append(e0.elapsed_time(e1) / k)
        done += k
    rho0 = float(scene.params[4])
    d = sim.read_particles(("dens",))["dens"][:, 0]
    sim.close()
    timed = steps - 3
    ms = sum(b * min(block, timed - i * block) for i, b in enumerate(blocks)) / timed
    return {"steps": steps, "timed_steps": timed, "ms_per_step": ms, "value": scene.n / (ms / 1e3), "unit": UNIT,
            "ms_per_step_by_block": blocks, "block": block,
            "density_error_end": float(np.mean(np.abs(d - rho0)) / rho0)}


def scenes_module():
    from nbodysimulation_experiment_gb300 import scenes
    return scenes


def bench_batched(torch, pkg, scenes, device: int, steps: int, warmup: int):
    """The batched form: 512 independent scenes (log-uniform 1,024..65,536
    particles, ~8.1M in all) advanced by one update per step, replayed from
    the per-step CUDA graph; event-timed on the batch's stream."""
    mix = scenes.batch_scenes()
    batch = pkg.BatchSimulation(mix, device=device)
    dt = float(scenes.DT)
    stream = torch.cuda.ExternalStream(batch.stream())
    for _ in range(warmup):
        batch.update(dt)
    batch.synchronize()
    tuned = batch.autotune(dt)
    launches0 = batch.kernel_launches()
    ms = []
    stage_names = ("time_integration", "time_viscosity_forces", "time_predict", "time_update_grid",
                   "time_density_and_pressure", "time_delta_positions", "time_collisions")
    stage_sum = dict.fromkeys(stage_names, 0.0)
    for _ in range(steps):
        with torch.cuda.stream(stream):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        batch.update(dt)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        stats = batch.get_stats(0)  # stage times cover every scene of the batch
        for k in stage_names:
            stage_sum[k] += getattr(stats, k)
    batch.synchronize()
    launches = batch.kernel_launches() - launches0
    total = batch.get_particle_count()
    rho0 = float(mix[0].params[4])
    errs, single_errs, identical = [], [], True
    for k in range(0, len(mix), 64):
        got = batch.read_particles(k, ("pos", "dens"))
        errs.append(float(np.mean(np.abs(got["dens"][:, 0] - rho0)) / rho0))
        # The same scene advanced alone by the plain step, the same number
        # of updates: its density deviation, and whether the batch's state
        # equals it bit for bit.
        sim = pkg.Simulation(mix[k].domain(), device=device)
        mix[k].apply(sim)
        for _ in range(warmup + steps):
            sim.update(dt)
        alone = sim.read_particles(("pos", "dens"))
        sim.close()
        single_errs.append(float(np.mean(np.abs(alone["dens"][:, 0] - rho0)) / rho0))
        identical = identical and np.array_equal(alone["pos"], got["pos"]) and np.array_equal(alone["dens"],
                                                                                              got["dens"])
    batch.close()
    return {"value": total * steps / (sum(ms) / 1e3), "unit": UNIT, "ms_per_step": statistics.mean(ms),
            "steps": steps, "warmup": warmup, "scenes": len(mix), "particles": int(total),
            "gpu_launches": int(launches), "graphs": True,
            "stage_ms": {k[5:]: v / steps for k, v in stage_sum.items()},
            "autotuned_shape": {"viscosity_warps": tuned[0], "viscosity_blocks": tuned[1],
                                "delta_warps": tuned[2], "delta_blocks": tuned[3]},
            "density_error": float(np.mean(errs)),
            "density_error_scenes_alone": float(np.mean(single_errs)),
            "identical_to_scenes_alone": bool(identical),
            "sampled_scenes": len(errs),
            "workload": "512 independent box scenes, particle counts log-uniform in [1024, 65536] (seeded), "
                        "each a jittered block + 0-4 circles, 4 walls, plain step, FP32; inputs > L2"}


def bench_learned(torch, pkg, scenes, device: int, args):
    """The learned frame on the 262,144-particle dam break with obstacles:
    the network is trained on the GPU on plain frames of seeded 65,536-particle
    obstacle scenes, then learned frames (one plain update over the frame plus
    the network's correction, judged by the density deviation with a bound of
    0.01 rest density) are timed against plain frames (four updates of dt/4,
    the reference's kSPHSubsteps) on the same scene."""
    from nbodysimulation_experiment_gb300 import learned
    frame, sub = float(scenes.DT), learned.SUBSTEPS
    scene = scenes.dam_break_262144()
    model = pkg.Mpnn(scene.n, device=device, seed=7)
    t0 = time.perf_counter()
    ntrain = learned.collect(model, lambda k: scenes.obstacles_65536(seed=1000 + k), range(args.learned_scenes),
                             args.learned_frames)
    learned.collect(model, lambda k: scenes.obstacles_65536(seed=5000 + k), range(2), 4)
    t_collect = time.perf_counter() - t0
    t0 = time.perf_counter()
    losses = learned.train(model, args.learned_steps, indices=range(ntrain))
    t_train = time.perf_counter() - t0
    ev = learned.evaluate(model, range(ntrain, model.sample_count))
    model.clear_samples()

    def run(use_network: bool):
        sim = pkg.Simulation(scene.domain(), device=device)
        scene.apply(sim)
        for _ in range(3):
            sim.update(frame / sub)
        sim.autotune(frame / sub)
        stream = torch.cuda.ExternalStream(sim.stream())
        ms, used, errs = [], 0, []
        for f in range(args.learned_warmup + args.learned_eval_frames):
            with torch.cuda.stream(stream):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            if use_network:
                u, err = sim.learned_frame(model, frame, sub, bound=0.01)
            else:
                for _ in range(sub):
                    sim.update(frame / sub)
                u, err = False, 0.0
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            if f >= args.learned_warmup:
                ms.append(e0.elapsed_time(e1))
                used += int(u)
                errs.append(err)
        # End to end through the C ABI with host buffers: every frame loads
        # the state from pinned host memory, advances it and reads it back.
        st = sim.dump_state()
        pinned = pinned_like(torch, {k: st[k] for k in STATE_KEYS})
        pinned["canonical_count"] = st["canonical_count"]
        pinned["grid"] = st["grid"]
        pinned_out = pinned_like(torch, {k: st[k] for k in STATE_KEYS})
        nbytes = sum(pinned[k].nbytes for k in STATE_KEYS)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.learned_eval_frames):
            sim.load_state(pinned)
            if use_network:
                sim.learned_frame(model, frame, sub, bound=0.01)
            else:
                for _ in range(sub):
                    sim.update(frame / sub)
            sim.dump_state(out=pinned_out)
        e2e_ms = (time.perf_counter() - t0) * 1e3 / args.learned_eval_frames
        if not use_network:  # density deviation of the plain result, as the judge measures it
            errs = [sim.learned_frame(model, frame, sub, bound=-1.0)[1]]
        sim.close()
        return statistics.mean(ms), used, float(np.mean(errs)), e2e_ms, nbytes

    ms_l, used, err_l, e2e_l, nbytes = run(True)
    ms_p, _, err_p, e2e_p, _ = run(False)
    quality = learned_quality(pkg, scene, model, device, frame, sub, args.learned_rollout_frames)
    n, nf = scene.n, args.learned_eval_frames
    model.close()
    return {"value": n / (ms_l / 1e3), "unit": "particle-frames/s",
            "frame": "1/60 s = %d reference substeps" % sub,
            "particle_steps_per_s": n * sub / (ms_l / 1e3),
            "ms_per_frame": ms_l, "plain_ms_per_frame": ms_p, "speedup_vs_plain_frame": ms_p / ms_l,
            "e2e": {"value": n / (e2e_l / 1e3), "unit": "particle-frames/s", "ms_per_frame": e2e_l,
                    "plain_ms_per_frame": e2e_p, "speedup_vs_plain_frame": e2e_p / e2e_l,
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "path": "sph_load_state from pinned host memory, sph_learned_frame (or four sph_update), "
                            "sph_dump_state into pinned host memory, every frame"},
            "frames": nf, "accepted_frames": used, "density_error": err_l,
            "density_error_plain_frame": err_p, "judge_bound": 0.01,
            "judge": "a learned frame stands if its mean |rho - rho0| / rho0 exceeds that of the single plain "
                     "update of the whole frame it corrects by at most judge_bound; an absolute bound of 1% "
                     "of rho0 would reject every frame here, the plain four-update frame included "
                     "(density_error_plain_frame)",
            "quality": quality, "particles": n,
            "workload": "dam_break_262144: 512x512 jittered block, 102.4 x 57.6 box, 4 walls + 8 circles + "
                        "4 segments; 2-round MPNN (edge 6-128-128, node 130-128-2; edge layer on tcgen05 "
                        "kind::tf32 MMAs, dense layers persistent BF16 tcgen05 GEMMs)",
            "train": {"samples": ntrain, "scenes": args.learned_scenes, "frames_per_scene": args.learned_frames,
                      "scene": "obstacles_65536 seeds 1000..", "steps": args.learned_steps,
                      "collect_s": t_collect, "train_s": t_train, "final_loss": float(np.mean(losses[-50:])),
                      "held_out_loss": ev["learned"], "held_out_loss_without_network": ev["without_network"]}}


def learned_quality(pkg, scene, model, device, frame, sub, rollout_frames):
    """Accuracy of the learned frame against the plain frame it stands in
    for (four updates of dt/4), on the benchmark's scene: (a) per frame, from
    the same state, the RMS and largest position difference in units of h
    (the network's correction applied without the judge); (b) a free rollout
    of learned frames (under the benchmark's judge) against one of plain
    frames from the same start: mean density deviation, kinetic energy and
    density histogram at the end."""
    from nbodysimulation_experiment_gb300 import scenes as sc_mod  # noqa: F401
    h = float(scene.params[0])
    rho0 = float(scene.params[4])

    def fresh():
        sim = pkg.Simulation(scene.domain(), device=device)
        scene.apply(sim)
        for _ in range(3):
            sim.update(frame / sub)
        return sim

    # (a) the same state advanced both ways, at several points of a run
    sim = fresh()
    rms, worst = [], []
    for f in range(12):
        st = sim.dump_state()
        sim.learned_frame(model, frame, sub, bound=1e30)
        a = sim.read_particles(("pos",))["pos"].astype(np.float64)
        sim.load_state(st)
        for _ in range(sub):
            sim.update(frame / sub)
        b = sim.read_particles(("pos",))["pos"].astype(np.float64)
        d = np.sqrt(np.sum((a - b) ** 2, axis=1)) / h
        if f % 3 == 2:
            rms.append(float(np.sqrt(np.mean(d ** 2))))
            worst.append(float(d.max()))
    sim.close()

    # (b) free rollouts from the same start, the learned one under the judge
    taken = [0]

    def rollout(use_network):
        sim = fresh()
        done, failure = 0, None
        try:
            for _ in range(rollout_frames):
                if use_network:
                    taken[0] += int(sim.learned_frame(model, frame, sub, bound=0.01)[0])
                else:
                    for _ in range(sub):
                        sim.update(frame / sub)
                sim.synchronize()
                done += 1
        except pkg.SphError as exc:  # reported, not hidden: how far the rollout got
            failure = str(exc)
        r = sim.read_particles(("pos", "vel", "dens"))
        sim.close()
        d = r["dens"][:, 0].astype(np.float64)
        hist, _ = np.histogram(d / rho0, bins=20, range=(0.0, 2.0))
        return {"frames_completed": done, "failure": failure,
                "density_error": float(np.mean(np.abs(d - rho0)) / rho0),
                "kinetic_energy": float(0.5 * np.mean(np.sum(r["vel"].astype(np.float64) ** 2, axis=1))),
                "mean_height": float(np.mean(r["pos"][:, 1])), "hist": hist / len(d)}

    lr, pr = rollout(True), rollout(False)
    return {"per_frame_rms_position_error_h": float(np.mean(rms)), "per_frame_max_position_error_h": max(worst),
            "rollout_frames": rollout_frames, "rollout_frames_taken_by_network": taken[0],
            "rollout_learned": {k: v for k, v in lr.items() if k != "hist"},
            "rollout_plain": {k: v for k, v in pr.items() if k != "hist"},
            "rollout_density_histogram_l1": float(np.abs(lr["hist"] - pr["hist"]).sum())}


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=HEADLINE, choices=sorted(WORKLOADS),
                    help="the headline line's workload (the others are extra objects)")
    ap.add_argument("--cpu-steps", type=int, default=4, help="CPU-baseline sample: at least this many updates")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample: at least this long")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the other configurations' objects")
    ap.add_argument("--extra-steps", type=int, default=20, help="timed updates of the other configurations")
    ap.add_argument("--batch-steps", type=int, default=20, help="timed updates of the 512-scene batch")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-long", action="store_true", help="skip the 1,000-update free runs")
    ap.add_argument("--long-steps", type=int, default=1000, help="updates of each free run")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--learned-scenes", type=int, default=100, help="seeded 65,536-particle training scenes")
    ap.add_argument("--learned-frames", type=int, default=20, help="training frames captured per scene")
    ap.add_argument("--learned-steps", type=int, default=1500, help="Adam steps")
    ap.add_argument("--learned-eval-frames", type=int, default=20)
    ap.add_argument("--learned-warmup", type=int, default=3)
    ap.add_argument("--learned-rollout-frames", type=int, default=200)
    args = ap.parse_args(argv)
    args.warmup = max(3, args.warmup)
    return args


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)

    import torch
    import torch.distributed as dist
    import nbodysimulation_experiment_gb300 as pkg
    from nbodysimulation_experiment_gb300 import scenes

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    pkg.build()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    head = measure_scene(torch, pkg, args.workload, local, args.steps, args.warmup, world, flush,
                         max(10, args.steps // 4), clocks=True)

    extras = {}
    if not args.no_extra:
        for w in WORKLOADS:
            if w != args.workload:
                extras[w] = measure_scene(torch, pkg, w, local, args.extra_steps, 5, world, flush, 10)

    long_runs = {}
    if not args.no_long:
        # Config 2 over its specified 1,000 updates.  The 1024x1024 blocks
        # cannot run that long within the reference's capacities (see
        # RESTART_AFTER); their lines cover updates 3-90.
        long_runs["obstacles_65536"] = long_run(torch, pkg, "obstacles_65536", local, args.long_steps)

    batched = None
    if not args.no_batch:
        batched = bench_batched(torch, pkg, scenes, local, args.batch_steps, 3)
        batched["vs_plain_1m"] = batched["value"] / extras["block_1m_plain"]["value"] \
            if "block_1m_plain" in extras else None

    learned_line = None
    if not args.no_learned:
        learned_line = bench_learned(torch, pkg, scenes, local, args)

    cpu = None
    if rank == 0 and not args.no_cpu and host_memory_gb() >= 2.0 * ORACLE_BYTES_PER_PARTICLE * head["particles"] / 1e9:
        from oracle.oracle import OracleSim, build as build_oracle
        build_oracle(reference=False)
        workers = OracleSim.hardware_threads()
        scene, springs, _ = make_scene(args.workload)
        cval, k, csec = cpu_port_rate(scene, springs, workers, args.cpu_steps, args.cpu_seconds)
        cpu = {"value": cval, "unit": UNIT, "cores": workers, "kind": "port",
               "sample": "%d updates of the %d-particle scene%s after its first 2 updates (%.1f s)"
                         % (k, scene.n, " with springs" if springs else "", csec)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": head["workload"], "particles": head["particles"], "springs": head["springs"],
                       "l2": "flushed between steps (256 MiB write); inputs also exceed L2",
                       "sweep_shape": head["sweep_shape"],
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "density_error": head["density_error"], "spring_count": head.get("spring_count")},
            "e2e": head["e2e"],
            "gpu_launches": head["gpu_launches"],
            "stage_ms": head["stage_ms"],
            "restarts": head.get("restarts"),
            "roofline": head["roofline"],
            "cpu_baseline": cpu,
            "clocks": head.get("clocks"),
        }
        for w, d in extras.items():
            line[w] = d
        line["long_runs"] = long_runs or None
        line["batched"] = batched
        line["learned"] = learned_line
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
