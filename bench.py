"""Benchmark of the GB300 Demo4 SPH step (one JSON line on rank 0).

Workload (one "step" = one ``Update`` of the whole scene): ``obstacles_65536``
-- a 256x256 jittered block (65,536 particles, spacing h/6) in a 51.2 x 28.8
box with four walls, eight seeded circles (radii 2h..6h) and four seeded line
segments, gravity (0, -10), the reference's sph.h constants, FP32.

* ``value``: particle-steps/s with the scene resident in HBM; each timed step
  is bracketed by CUDA events on the simulation's stream, and L2 is flushed
  (a 256 MiB write) between steps, outside the events.
* ``e2e``: the same metric through the C ABI with host buffers: every step
  loads the full state from pinned host memory (``sph_load_state``), updates
  and reads the full state back into pinned host memory (``sph_dump_state``).
* ``roofline``: the dominant kernel (the ordered delta sweep) against the
  measured HBM copy bandwidth; achieved = algorithmic bytes (24 B per
  particle: read position and pressure, write position) / its event-timed
  duration.
* ``cpu_baseline``: the CPU restatement of the reference step (oracle/),
  multithreaded like the reference's ThreadPool on all host cores, on a
  bounded sample of the same workload.

Further objects in the same line (forms of the step beyond the reference):

* ``batched``: 512 independent scenes (log-uniform 1,024..65,536 particles,
  ~8.1M in all) advanced by one update per step from the per-step CUDA graph,
  sweep shapes chosen by the autotuner.
* ``block_1m``: the 1,048,576-particle block, plain and with viscoelastic
  springs.
* ``learned``: the message-passing network trained on the GPU on plain
  frames of seeded 65,536-particle scenes, then learned frames on a
  262,144-particle dam break with obstacles against plain frames (four
  updates of dt/4), under the density-deviation judge.

``--impl reference`` times that CPU implementation alone (rank 0 only).
Multi-GPU runs are independent replicas (the step does not shard).
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
DELTA_BYTES_PER_PARTICLE = 24  # read pos 8 + pressure 8, write pos 8
WORKLOAD = ("obstacles_65536: 65,536-particle jittered block (spacing h/6) in a 51.2 x 28.8 box, "
            "4 walls + 8 circles + 4 segments, plain Demo4 step (viscosity on, springs off), FP32")


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


def profile_traffic(n_particles: int):
    """DRAM bytes per launch of the delta sweep from the committed ncu
    summary (captured on a smaller case, scaled by particle count)."""
    path = os.path.join(ROOT, "profiles", "k_delta_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_particle"]) * n_particles
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


def cpu_baseline(scene, state_gpu, steps: int, workers: int):
    """Time the CPU restatement (multithreaded like the reference) on a
    bounded sample: `steps` updates from the GPU's mid-run state."""
    from oracle.oracle import OracleSim
    from oracle import state as ostate
    orc = OracleSim(scene.oracle_domain(OracleSim), fp64=False, workers=workers)
    scene.apply(orc)
    orc.set_state(ostate.to_reference_state(state_gpu))
    orc.update(float(scene_dt()))  # warm the pool and caches
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.update(float(scene_dt()))
    dt = time.perf_counter() - t0
    orc.close()
    return scene.n * steps / dt, dt


def scene_dt():
    from nbodysimulation_experiment_gb300 import scenes
    return scenes.DT


def run_reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from nbodysimulation_experiment_gb300 import scenes
    from oracle.oracle import OracleSim, build as build_oracle
    build_oracle(reference=True)
    scene = scenes.obstacles_65536()
    workers = OracleSim.hardware_threads()
    orc = OracleSim(scene.oracle_domain(OracleSim), fp64=False, workers=workers)
    scene.apply(orc)
    orc.update(float(scenes.DT))  # first update (AddParticle order)
    per = max(1, args.cpu_steps // max(1, args.steps))
    for _ in range(args.warmup):
        orc.update(float(scenes.DT))
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for _ in range(per):
            orc.update(float(scenes.DT))
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = scene.n * per * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / (per * args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": {"workload": WORKLOAD, "particles": scene.n},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                         "sample": "%d updates of the %d-particle scene per step, %d steps, after %d warm-up "
                                   "updates" % (per, scene.n, args.steps, args.warmup + 1)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


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
    errs = []
    for k in range(0, len(mix), 64):
        d = batch.read_particles(k, ("dens",))["dens"][:, 0]
        errs.append(float(np.mean(np.abs(d - rho0)) / rho0))
    batch.close()
    return {"value": total * steps / (sum(ms) / 1e3), "unit": UNIT, "ms_per_step": statistics.mean(ms),
            "steps": steps, "warmup": warmup, "scenes": len(mix), "particles": int(total),
            "gpu_launches": int(launches), "graphs": True,
            "stage_ms": {k[5:]: v / steps for k, v in stage_sum.items()},
            "autotuned_shape": {"viscosity_warps": tuned[0], "viscosity_blocks": tuned[1],
                                "delta_warps": tuned[2], "delta_blocks": tuned[3]},
            "density_error": float(np.mean(errs)),
            "workload": "512 independent box scenes, particle counts log-uniform in [1024, 65536] (seeded), "
                        "each a jittered block + 0-4 circles, 4 walls, plain step, FP32; inputs > L2"}


def bench_block_1m(torch, pkg, scenes, device: int, steps: int, warmup: int, springs: bool):
    """The 1,048,576-particle block (1024x1024 jittered lattice in a
    204.8 x 115.2 box, four walls), plain or with viscoelastic springs
    (yield ratio 0.1, plasticity 0.3, stiffness 0.3, at most 16 per
    particle); event-timed updates on the simulation's stream."""
    scene = scenes.block_1m()
    sim = pkg.Simulation(scene.domain(), device=device)
    scene.apply(sim)
    if springs:
        sim.set_springs(True, yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    dt = float(scenes.DT)
    stream = torch.cuda.ExternalStream(sim.stream())
    for _ in range(warmup):
        sim.update(dt)
    sim.synchronize()
    tuned = sim.autotune(dt)
    ms, spring_ms = [], []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        sim.update(dt)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        spring_ms.append(sim.get_stats().time_neighbor_search)
    out = {"value": scene.n * steps / (sum(ms) / 1e3), "unit": UNIT, "ms_per_step": statistics.mean(ms),
           "steps": steps, "warmup": warmup, "particles": scene.n, "springs": springs,
           "autotuned_shape": {"viscosity_warps": tuned[0], "viscosity_blocks": tuned[1],
                               "delta_warps": tuned[2], "delta_blocks": tuned[3]}}
    if springs:
        out["spring_phase_ms"] = statistics.mean(spring_ms)
        out["spring_count"] = sim.spring_count()
    sim.close()
    return out


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
        if not use_network:  # density deviation of the plain result, as the judge measures it
            errs = [sim.learned_frame(model, frame, sub, bound=-1.0)[1]]
        sim.close()
        return statistics.mean(ms), used, float(np.mean(errs))

    ms_l, used, err_l = run(True)
    ms_p, _, err_p = run(False)
    n, nf = scene.n, args.learned_eval_frames
    model.close()
    return {"value": n / (ms_l / 1e3), "unit": "particle-frames/s",
            "frame": "1/60 s = %d reference substeps" % sub,
            "particle_steps_per_s": n * sub / (ms_l / 1e3),
            "ms_per_frame": ms_l, "plain_ms_per_frame": ms_p, "speedup_vs_plain_frame": ms_p / ms_l,
            "frames": nf, "accepted_frames": used, "density_error": err_l,
            "density_error_plain_frame": err_p, "judge_bound": 0.01, "particles": n,
            "workload": "dam_break_262144: 512x512 jittered block, 102.4 x 57.6 box, 4 walls + 8 circles + "
                        "4 segments; 2-round MPNN (edge 6-128-128, node 130-128-2, BF16 tcgen05 GEMMs)",
            "train": {"samples": ntrain, "scenes": args.learned_scenes, "frames_per_scene": args.learned_frames,
                      "scene": "obstacles_65536 seeds 1000..", "steps": args.learned_steps,
                      "collect_s": t_collect, "train_s": t_train, "final_loss": float(np.mean(losses[-50:])),
                      "held_out_loss": ev["learned"], "held_out_loss_without_network": ev["without_network"]}}


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=60, help="CPU-baseline sample size in updates")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-steps", type=int, default=20, help="timed updates of the 512-scene batch")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--block-steps", type=int, default=10, help="timed updates of the 1M-particle block")
    ap.add_argument("--no-block", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--learned-scenes", type=int, default=100, help="seeded 65,536-particle training scenes")
    ap.add_argument("--learned-frames", type=int, default=20, help="training frames captured per scene")
    ap.add_argument("--learned-steps", type=int, default=1500, help="Adam steps")
    ap.add_argument("--learned-eval-frames", type=int, default=20)
    ap.add_argument("--learned-warmup", type=int, default=3)
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

    scene = scenes.obstacles_65536()
    sim = pkg.Simulation(scene.domain(), device=local)
    scene.apply(sim)
    dt = float(scenes.DT)
    stream = torch.cuda.ExternalStream(sim.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        sim.update(dt)
    sim.synchronize()
    tuned = sim.autotune(dt)

    # --- device-resident timed region -------------------------------------
    launches0 = sim.kernel_launches()
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    step_ms, delta_ms = [], []
    stage_names = ("time_integration", "time_viscosity_forces", "time_predict", "time_update_grid",
                   "time_neighbor_search", "time_density_and_pressure", "time_delta_positions", "time_collisions")
    stage_sum = dict.fromkeys(stage_names, 0.0)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        sim.update(dt)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        stats = sim.get_stats()
        delta_ms.append(stats.time_delta_positions)
        for k in stage_names:
            stage_sum[k] += getattr(stats, k)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = sampler.stop()
    launches = sim.kernel_launches() - launches0 - 0  # get_stats launches nothing
    total_s = job_seconds(sum(step_ms) / 1e3, world, "cuda")
    value = job_rate(scene.n, args.steps, world, total_s)

    # density deviation from the rest density at the end of the run
    rd = sim.read_particles(("dens",))
    rho0 = float(scene.params[4])
    dens_err = float(np.mean(np.abs(rd["dens"][:, 0] - rho0)) / rho0)

    # --- end to end through the C ABI with host buffers --------------------
    st = sim.dump_state()
    pinned = {}
    for k in ("pos", "prev", "vel", "acc", "dens", "press", "id", "cell", "cell_start", "cell_count"):
        a = st[k]
        t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32, pin_memory=True)
        arr = t.numpy()
        arr[...] = a
        pinned[k] = arr
    pinned["canonical_count"] = st["canonical_count"]
    pinned["grid"] = st["grid"]
    # The step's result is read back into pinned host memory as well.
    pinned_out = {}
    for k in ("pos", "prev", "vel", "acc", "dens", "press", "id", "cell", "cell_start", "cell_count"):
        a = st[k]
        pinned_out[k] = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32,
                                    pin_memory=True).numpy()
    e2e_steps = max(10, args.steps // 4)
    h2d = sum(pinned[k].nbytes for k in ("pos", "prev", "vel", "acc", "dens", "press", "id", "cell",
                                        "cell_start", "cell_count"))
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.load_state(pinned)
        sim.update(dt)
        out = sim.dump_state(out=pinned_out)
    e2e_s = job_seconds(time.perf_counter() - t0, world, "cuda")
    e2e_value = job_rate(scene.n, e2e_steps, world, e2e_s)

    hbm, peak_kind = measured_peaks()
    mean_delta_s = statistics.mean(delta_ms) / 1e3
    achieved = DELTA_BYTES_PER_PARTICLE * scene.n / mean_delta_s / 1e9
    traffic = profile_traffic(scene.n)

    batched = None
    if not args.no_batch:
        batched = bench_batched(torch, pkg, scenes, local, args.batch_steps, 3)
        batched["vs_plain"] = batched["value"] / value

    block = None
    if not args.no_block:
        block = {"plain": bench_block_1m(torch, pkg, scenes, local, args.block_steps, 3, False),
                 "springs": bench_block_1m(torch, pkg, scenes, local, args.block_steps, 3, True)}

    learned_line = None
    if not args.no_learned:
        learned_line = bench_learned(torch, pkg, scenes, local, args)

    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle.oracle import OracleSim, build as build_oracle
        build_oracle(reference=False)
        workers = OracleSim.hardware_threads()
        cval, csec = cpu_baseline(scene, st, args.cpu_steps, workers)
        cpu = {"value": cval, "unit": UNIT, "cores": workers, "kind": "port",
               "sample": "%d updates of the %d-particle scene from the GPU's state after %d updates "
                         "(%.1f s)" % (args.cpu_steps, scene.n, args.warmup, csec)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "particles": scene.n, "l2": "flushed between steps (256 MiB write)",
                       "sweep_shape": {"viscosity_warps": tuned[0], "viscosity_blocks": tuned[1],
                                       "delta_warps": tuned[2], "delta_blocks": tuned[3]},
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "density_error": dens_err},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(h2d)},
            "gpu_launches": int(launches),
            "stage_ms": {k[5:]: v / args.steps for k, v in stage_sum.items()},
            "roofline": {"bound": "hbm", "kernel": "k_delta", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": traffic,
                         "algorithmic_bytes": DELTA_BYTES_PER_PARTICLE * scene.n,
                         "kernel_ms": 1e3 * mean_delta_s},
            "cpu_baseline": cpu,
            "batched": batched,
            "block_1m": block,
            "learned": learned_line,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    sim.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
