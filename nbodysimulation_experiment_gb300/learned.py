"""Training and use of the learned frame (``Mpnn``; no counterpart in the
reference).

A learned frame of length dt is one plain update over the whole frame,
corrected by the network towards the reference's ``substeps`` updates of
dt / substeps (kSPHSubsteps, NBodySimulation/sph.h:32-34), and judged by the
plain method's density deviation (``Simulation.learned_frame``).  Training
samples are plain frames captured from seeded scenes; training runs on the
GPU through the library's own forward and backward kernels.
"""
from __future__ import annotations

import time
from typing import Callable, Dict, Iterable, List

import numpy as np

from . import scenes
from .simulation import Mpnn, Simulation

FRAME = float(scenes.DT)
SUBSTEPS = 4


def collect(model: Mpnn, make_scene: Callable[[int], "scenes.Scene"], seeds: Iterable[int], frames: int,
            warm: int = 3, substeps: int = SUBSTEPS, frame_dt: float = FRAME) -> int:
    """Capture ``frames`` consecutive plain frames from each seeded scene
    (after ``warm`` plain updates of frame_dt / substeps); returns the
    number of samples the model then holds."""
    for seed in seeds:
        scene = make_scene(seed)
        sim = Simulation(scene.domain())
        scene.apply(sim)
        for _ in range(warm):
            sim.update(frame_dt / substeps)
        for _ in range(frames):
            model.capture(sim, frame_dt, substeps)
        sim.close()
    return model.sample_count


def train(model: Mpnn, steps: int, lr: float = 1e-3, decay_at: float = 0.66, decay: float = 0.3,
          indices: Iterable[int] = None, seed: int = 0) -> List[float]:
    """Adam steps over the samples in a seeded random order; the learning
    rate drops by ``decay`` after ``decay_at`` of the steps.  Returns the
    per-step losses."""
    idx = list(indices) if indices is not None else list(range(model.sample_count))
    rng = np.random.default_rng(seed)
    order = []
    losses = []
    for it in range(steps):
        if not order:
            order = list(rng.permutation(idx))
        rate = lr if it < decay_at * steps else lr * decay
        losses.append(model.train_step(int(order.pop()), rate))
    return losses


def evaluate(model: Mpnn, indices: Iterable[int]) -> Dict[str, float]:
    """Mean loss of the network and of the uncorrected plain update (u = 0)
    on the given samples (squared error of the correction in units of h^2)."""
    idx = list(indices)
    learned = float(np.mean([model.eval(k) for k in idx]))
    base = float(np.mean([np.mean(np.sum(model.sample(k)["target"].astype(np.float64) ** 2, axis=1))
                          for k in idx]))
    return {"learned": learned, "without_network": base}
