"""Headless replacement for Demo4's point render (demo4.cpp:453-532): the
particle colours (SPHGetParticleColor, sph.h:683-695) and the point image,
checked bit for bit against a NumPy restatement in FP32."""
import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes

pytestmark = pytest.mark.gpu

F = np.float32


def _clamp01(v):
    # std::max(std::min(v, 1.0f), 0.0f): comparisons as written (a NaN stays).
    lo = np.where(F(1.0) < v, F(1.0), v)
    return np.where(lo < F(0.0), F(0.0), lo).astype(F)


def _colors(rho0, dens, press, vel):
    r = press[:, 0] / F(-10.0)
    g = dens[:, 0] / F(rho0)
    b = np.sqrt(vel[:, 0] * vel[:, 0] + vel[:, 1] * vel[:, 1]) / F(10.0)
    return np.stack([_clamp01(r), _clamp01(g), _clamp01(b), np.ones_like(r)], axis=1).astype(F)


def _q8(x):
    y = (x * F(255.0) + F(0.5)).astype(F)
    ok = y >= F(1.0)
    return np.where(ok, np.floor(np.minimum(np.where(ok, y, F(0.0)), F(255.0))), 0).astype(np.uint64)


def _sim(steps=4):
    scene = scenes.scaled_block(32, seed=21)  # 1,024 particles with obstacles
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    for _ in range(steps):
        sim.update(float(scenes.DT))
    return scene, sim


def test_particle_colors_match_the_reference_formula():
    scene, sim = _sim()
    rd = sim.read_particles(("dens", "press", "vel"))
    got = sim.particle_colors()
    want = _colors(scene.params[4], rd["dens"], rd["press"], rd["vel"])
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert (got[:, 1] > 0).all()  # every particle has a density
    sim.close()


def test_point_image_draws_later_particles_over_earlier_ones():
    scene, sim = _sim()
    width, height = 400, 225
    img = sim.render_points(width, height)
    rd = sim.read_particles(("pos", "dens", "press", "vel"))
    c = _colors(scene.params[4], rd["dens"], rd["press"], rd["vel"])
    packed = _q8(c[:, 0]) | (_q8(c[:, 1]) << 8) | (_q8(c[:, 2]) << 16) | (_q8(c[:, 3]) << 24)
    dom = scene.domain()
    half_w, half_h = F(dom.width) * F(0.5), F(dom.height) * F(0.5)
    sx, sy = F(width) / F(dom.width), F(height) / F(dom.height)
    fx = ((rd["pos"][:, 0] + half_w) * sx).astype(F)
    fy = ((half_h - rd["pos"][:, 1]) * sy).astype(F)
    inside = (fx >= 0) & (fy >= 0) & (fx < width) & (fy < height)
    px = np.minimum(fx[inside].astype(np.int64), width - 1)
    py = np.minimum(fy[inside].astype(np.int64), height - 1)
    ids = np.nonzero(inside)[0].astype(np.uint64)
    keys = np.zeros((height, width), np.uint64)
    np.maximum.at(keys, (py, px), ((ids + np.uint64(1)) << np.uint64(32)) | packed[inside])
    want = (keys & np.uint64(0xffffffff)).astype(np.uint32).view(np.uint8).reshape(height, width, 4)
    assert np.array_equal(img, want)
    assert inside.sum() == len(fx)  # the box holds every particle
    assert (img[..., 3] == 255).sum() == len(np.unique(py * width + px))
    sim.close()
