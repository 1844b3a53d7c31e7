"""Seeded synthetic scenes for the Demo4 step.

The reference builds scenes through its simulation interface
(``DemoApplication::LoadScenario``, NBodySimulation/app.cpp:477-534):
reset stats, clear, set gravity and parameters, add bodies, add particles.
``Scene.apply`` does the same on any object with that interface.  Particle
jitter here comes from a seeded NumPy generator instead of ``rand()``
(vecmath.h:317-322) so that scenes are reproducible across machines.

Scenes:

* ``dam_break_4096``   -- 64x64 jittered lattice (spacing h/6 = 0.05, uniform
  jitter +-0.1h per axis) at the lower left of the reference's 10 x 5.625 box,
  four walls, gravity (0, -10), the reference's sph.h constants.
* ``obstacles_65536``  -- 256x256 jittered block in a 51.2 x 28.8 box (16:9),
  four walls, 8 seeded circles with radii in [2h, 6h] and 4 seeded line
  segments, all outside the block.
* ``block_1m``         -- 1024x1024 jittered block in a 204.8 x 115.2 box.
* ``dam_break_262144`` -- 512x512 block in a 102.4 x 57.6 box with 8 circles
  and 4 segments (the learned frame's workload).
* ``batch_scenes``     -- 512 independent boxes with log-uniform particle
  counts in [1,024, 65,536], each a jittered block plus 0-4 circles.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional, Tuple

import numpy as np

H = np.float32(6.0) * np.float32(0.05)       # kSPHKernelHeight (sph.h:36)
SPACING = H / np.float32(6.0)                 # Dambreak spacing (sph.h:329)
DT = np.float32(1.0) / np.float32(60.0)       # kSPHDeltaTime (sph.h:33)


def f32(x) -> float:
    return float(np.float32(x))


def scenario_params(kernel_height=H, cell_size=H, spacing=SPACING, near_stiffness=np.float32(6.0)) -> np.ndarray:
    """SPHParameters as the scenario table stores it: the 8-argument
    constructor keeps kSPHKernelHeight and kSPHRestDensity whatever is passed
    (sph.h:112-122)."""
    h = np.float32(6.0) * np.float32(0.05)
    return np.array([h, cell_size, spacing, np.float32(1.0) / np.float32(kernel_height), 20.0, 0.6,
                     near_stiffness, 0.5, 0.3], np.float32)


@dataclasses.dataclass
class Scene:
    name: str
    width: float
    height: float
    positions: np.ndarray                      # (n, 2) float32, AddParticle order
    planes: List[Tuple[float, float, float]]   # normal x, normal y, distance
    circles: List[Tuple[float, float, float]] = dataclasses.field(default_factory=list)
    segments: List[Tuple[float, float, float, float]] = dataclasses.field(default_factory=list)
    gravity: Tuple[float, float] = (0.0, -10.0)
    params: np.ndarray = dataclasses.field(default_factory=scenario_params)
    max_particles: Optional[int] = None

    @property
    def n(self) -> int:
        return len(self.positions)

    def domain(self):
        from .simulation import Domain, reference_domain
        d = reference_domain()
        d.width = self.width
        d.height = self.height
        d.max_particles = int(self.max_particles or max(self.n, 1))
        return d

    def oracle_domain(self, oracle_cls):
        d = oracle_cls.reference_domain()
        d.width = self.width
        d.height = self.height
        d.max_particles = int(self.max_particles or max(self.n, 1))
        return d

    def apply(self, sim) -> None:
        """LoadScenario order (app.cpp:479-527) on a GPU Simulation or an oracle."""
        gpu = hasattr(sim, "add_line_segment")
        sim.reset_stats()
        sim.clear_bodies()
        sim.clear_particles()
        sim.clear_emitters()
        sim.set_gravity(*self.gravity) if not gpu else sim.set_gravity(self.gravity)
        if gpu:
            from .simulation import Params
            sim.set_params(Params.from_array(self.params))
        else:
            sim.set_params(self.params)
        for nx, ny, d in self.planes:
            sim.add_plane((nx, ny), d) if gpu else sim.add_plane(nx, ny, d)
        for x, y, r in self.circles:
            sim.add_circle((x, y), r) if gpu else sim.add_circle(x, y, r)
        for ax, ay, bx, by in self.segments:
            sim.add_line_segment((ax, ay), (bx, by)) if gpu else sim.add_segment(ax, ay, bx, by)
        if gpu:
            sim.add_particles(self.positions)
        else:
            sim.add_particles(self.positions)


def box_planes(width: float, height: float) -> List[Tuple[float, float, float]]:
    """The four walls as LoadScenario derives them: distance = dot(normal,
    position) for CreatePlane(position, normal) (app.cpp:489-491,
    sph.h:183-190, 323-326)."""
    hw = np.float32(width) * np.float32(0.5)
    hh = np.float32(height) * np.float32(0.5)
    out = []
    for (nx, ny), (px, py) in (((0, 1), (0, -hh)), ((0, -1), (0, hh)), ((1, 0), (-hw, 0)), ((-1, 0), (hw, 0))):
        d = np.float32(nx) * np.float32(px) + np.float32(ny) * np.float32(py)
        out.append((float(nx), float(ny), float(d)))
    return out


def jittered_lattice(nx: int, ny: int, x0: float, y0: float, spacing=SPACING, jitter=np.float32(0.1) * H,
                     seed: int = 1234) -> np.ndarray:
    """Row-major lattice (y outer, x inner, like AddVolume) with uniform
    per-axis jitter in [-jitter, +jitter]."""
    rng = np.random.default_rng(seed)
    iy, ix = np.meshgrid(np.arange(ny, dtype=np.float32), np.arange(nx, dtype=np.float32), indexing="ij")
    p = np.stack([np.float32(x0) + ix.ravel() * np.float32(spacing),
                  np.float32(y0) + iy.ravel() * np.float32(spacing)], 1).astype(np.float32)
    p += rng.uniform(-float(jitter), float(jitter), p.shape).astype(np.float32)
    return p.astype(np.float32)


REF_WIDTH = 10.0
REF_HEIGHT = float(np.float32(10.0) / (np.float32(16.0) / np.float32(9.0)))


def dam_break_4096(seed: int = 1234) -> Scene:
    hh = np.float32(REF_HEIGHT) * np.float32(0.5)
    pos = jittered_lattice(64, 64, -4.9, float(-hh + np.float32(0.1)), seed=seed)
    return Scene("dam_break_4096", REF_WIDTH, REF_HEIGHT, pos, box_planes(REF_WIDTH, REF_HEIGHT))


def _block_scene(name: str, side: int, width: float, height: float, n_circles: int, n_segments: int,
                 seed: int, count: Optional[int] = None) -> Scene:
    """A side x side jittered block at the lower left of the box (the first
    ``count`` lattice points when given: rows of ``side``), walls, seeded
    circles and segments clear of the block."""
    hw, hh = width * 0.5, height * 0.5
    x0, y0 = -hw + 0.1, -hh + 0.1
    rows = side if count is None else -(-count // side)
    pos = jittered_lattice(side, rows, x0, y0, seed=seed)
    if count is not None:
        pos = np.ascontiguousarray(pos[:count])
    extent = float(max(side, rows)) * float(SPACING)
    rng = np.random.default_rng(seed + 1)
    block = (x0 - 0.2, y0 - 0.2, x0 + extent + 0.2, y0 + extent + 0.2)

    def clear_of_block(x, y, r):
        cx = min(max(x, block[0]), block[2])
        cy = min(max(y, block[1]), block[3])
        return (x - cx) ** 2 + (y - cy) ** 2 > (r + 0.3) ** 2

    circles = []
    r_max = min(6.0 * float(H), 0.2 * height)
    r_min = min(2.0 * float(H), 0.5 * r_max)
    attempts = 0
    while len(circles) < n_circles and attempts < 10000:
        attempts += 1
        r = float(rng.uniform(r_min, r_max))
        x = float(rng.uniform(-hw + r + 0.5, hw - r - 0.5))
        y = float(rng.uniform(-hh + r + 0.5, hh - r - 0.5))
        if clear_of_block(x, y, r) and all((x - a) ** 2 + (y - b) ** 2 > (r + c + 0.3) ** 2 for a, b, c in circles):
            circles.append((f32(x), f32(y), f32(r)))
    segments = []
    attempts = 0
    while len(segments) < n_segments and attempts < 10000:
        attempts += 1
        length = float(rng.uniform(1.5, min(4.0, 0.25 * width)))
        ang = float(rng.uniform(0, np.pi))
        x = float(rng.uniform(-hw + 0.5 * length + 0.5, hw - 0.5 * length - 0.5))
        y = float(rng.uniform(-hh + 0.5 * length + 0.5, hh - 0.5 * length - 0.5))
        ax, ay = x - 0.5 * length * np.cos(ang), y - 0.5 * length * np.sin(ang)
        bx, by = x + 0.5 * length * np.cos(ang), y + 0.5 * length * np.sin(ang)
        if clear_of_block(x, y, 0.5 * length):
            segments.append((f32(ax), f32(ay), f32(bx), f32(by)))
    return Scene(name, width, height, pos, box_planes(width, height), circles, segments)


def obstacles_65536(seed: int = 1234) -> Scene:
    return _block_scene("obstacles_65536", 256, 51.2, 28.8, 8, 4, seed)


def dam_break_262144(seed: int = 1234) -> Scene:
    """512x512 jittered block (262,144 particles) at the lower left of a
    102.4 x 57.6 box with four walls, 8 seeded circles and 4 segments."""
    return _block_scene("dam_break_262144", 512, 102.4, 57.6, 8, 4, seed)


def block_1m(seed: int = 1234) -> Scene:
    return _block_scene("block_1m", 1024, 204.8, 115.2, 0, 0, seed)


def scaled_block(side: int, seed: int = 1234, obstacles: bool = True) -> Scene:
    """A side x side block in a box four block-widths wide (16:9)."""
    extent = side * float(SPACING)
    width = max(16.0, 4.0 * extent)
    height = width * 9.0 / 16.0
    return _block_scene("block_%d" % (side * side), side, width, height, 8 if obstacles else 0,
                        4 if obstacles else 0, seed)


def block_n(count: int, seed: int = 1234, n_circles: int = 0, n_segments: int = 0) -> Scene:
    """``count`` particles as a near-square jittered block (rows of
    ceil(sqrt(count))) in a 16:9 box four block-widths wide (at least 16)."""
    side = int(np.ceil(np.sqrt(count)))
    extent = side * float(SPACING)
    width = max(16.0, 4.0 * extent)
    height = width * 9.0 / 16.0
    return _block_scene("block_n%d" % count, side, width, height, n_circles, n_segments, seed, count=count)


def batch_scenes(count: int = 512, seed: int = 4242, n_min: int = 1024, n_max: int = 65536) -> List[Scene]:
    """Independent box scenes for the batched step: particle counts
    log-uniform in [n_min, n_max], each a jittered block plus 0-4 seeded
    circles (no segments), all seeded from ``seed``."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(n_min), np.log(n_max), count))
    ns = np.clip(np.rint(ns).astype(np.int64), n_min, n_max)
    circles = rng.integers(0, 5, count)
    return [block_n(int(n), seed=seed * 1000 + k, n_circles=int(c)) for k, (n, c) in enumerate(zip(ns, circles))]


SCENES = {
    "dam_break_4096": dam_break_4096,
    "obstacles_65536": obstacles_65536,
    "block_1m": block_1m,
    "dam_break_262144": dam_break_262144,
}
