"""The allocation-free entry point, through the C ABI, against the library's
regular update and against the oracle.

`sph_density_pressure_noalloc` exists for callers that cannot call
cudaMalloc (their memory belongs to another component's allocator or budget,
or they run in a loop that must not allocate): it takes device pointers for
positions and outputs and keeps its working memory in a fixed device array
inside the library.  Its densities and pressures must equal, bit for bit,
what one `sph_update` computes for the same freshly added, motionless
particles without gravity (the density pass sees exactly those positions and
the same neighbour lists), and what the oracle's first update computes.
Cases: two calls in a row with different particle sets (the shared working
array must carry nothing over), particles outside the box (clamped into the
edge cells), densely packed cells within the domain's capacities, no
particles, and inputs beyond the capacities (SPH_ERR_CAPACITY).

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes, simulation
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu


def _noalloc(lib, domain, params, pos_dev, n, dens_dev, press_dev, stream):
    fn = lib.sph_density_pressure_noalloc
    fn.argtypes = [ctypes.POINTER(simulation.Domain), ctypes.POINTER(simulation.Params), ctypes.c_void_p,
                   ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn(ctypes.byref(domain), ctypes.byref(params), pos_dev, n, dens_dev, press_dev, stream)


def _via_update(domain, params, positions):
    sim = pkg.Simulation(domain)
    sim.set_params(params)
    sim.set_gravity((0.0, 0.0))
    sim.add_particles(positions)
    sim.update(float(scenes.DT))
    out = sim.read_particles(("dens", "press"))
    sim.close()
    return out


def _via_oracle(params, positions):
    orc = OracleSim()
    orc.set_params(params.as_array())
    orc.set_gravity(0.0, 0.0)
    orc.add_particles(positions)
    orc.update(float(scenes.DT))
    st = orc.get_state(lists=False)
    orc.close()
    return {k: np.asarray(st[k], np.float32) for k in ("dens", "press")}


def _run(torch, lib, domain, params, pos):
    n = len(pos)
    stream = torch.cuda.current_stream().cuda_stream
    pos_dev = torch.from_numpy(pos).cuda()
    dens_dev = torch.full((n, 2), float("nan"), device="cuda")
    press_dev = torch.full((n, 2), float("nan"), device="cuda")
    rc = _noalloc(lib, domain, params, pos_dev.data_ptr(), n, dens_dev.data_ptr(), press_dev.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc, dens_dev.cpu().numpy(), press_dev.cpu().numpy()


def _positions(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-4.5, 4.5, n), rng.uniform(-2.5, 2.5, n)], 1).astype(np.float32)


def _outside(seed):
    """Particles in and beyond every edge of the 10 x 5.625 box."""
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-6.5, 6.5, 800), rng.uniform(-3.6, 3.6, 800)], 1).astype(np.float32)


def _packed(seed):
    """Two neighbouring cells packed with 350 and 300 particles (within the
    reference's 500 per cell and 1,000 per list) plus a sparse background."""
    rng = np.random.default_rng(seed)
    a = np.stack([rng.uniform(-0.19, 0.09, 350), rng.uniform(-1.90, -1.62, 350)], 1)
    b = np.stack([rng.uniform(0.11, 0.39, 300), rng.uniform(-1.90, -1.62, 300)], 1)
    return np.concatenate([a, b, _positions(500, seed + 1)]).astype(np.float32)


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch, pkg.load_library(), pkg.reference_domain(), pkg.Params.from_array(scenes.scenario_params())


@pytest.mark.parametrize("case", ["two_calls", "outside_box", "packed_cells"])
def test_density_pressure_noalloc_matches_update_and_oracle(env, case):
    torch, lib, domain, params = env
    sets = {"two_calls": [_positions(3000, 1), _positions(1500, 2)],
            "outside_box": [_outside(3)], "packed_cells": [_packed(4)]}[case]
    for pos in sets:
        rc, dens, press = _run(torch, lib, domain, params, pos)
        assert rc == simulation.SPH_OK, rc
        upd = _via_update(domain, params, pos)
        orc = _via_oracle(params, pos)
        for got, key in ((dens, "dens"), (press, "press")):
            assert np.array_equal(got, upd[key]), key
            assert np.array_equal(got, orc[key]), key


def test_density_pressure_noalloc_edge_sizes(env):
    torch, lib, domain, params = env
    # No particles: nothing to do, nothing touched.
    dummy = ctypes.c_void_p(16)
    assert _noalloc(lib, domain, params, dummy, 0, dummy, dummy, None) == simulation.SPH_OK
    # Sizes are checked before any pointer is used or any work is enqueued.
    assert _noalloc(lib, domain, params, dummy, 262145, dummy, dummy, None) == simulation.SPH_ERR_CAPACITY
    big = pkg.reference_domain()
    big.width, big.height = 600.0, 300.0  # 2000 x 1000 cells > 262,144
    assert _noalloc(lib, big, params, dummy, 10, dummy, dummy, None) == simulation.SPH_ERR_CAPACITY
    wide = pkg.reference_domain()
    wide.max_neighbors = 5000
    assert _noalloc(lib, wide, params, dummy, 10, dummy, dummy, None) == simulation.SPH_ERR_CAPACITY
    # A cell beyond the domain's 500 per cell: computed elsewhere, flagged.
    rng = np.random.default_rng(9)
    crowd = np.stack([rng.uniform(-0.19, 0.09, 520), rng.uniform(-1.90, -1.62, 520)], 1).astype(np.float32)
    rc, _, _ = _run(torch, lib, domain, params, crowd)
    assert rc == simulation.SPH_ERR_CAPACITY
    # The next call starts clean.
    pos = _positions(2000, 10)
    rc, dens, _ = _run(torch, lib, domain, params, pos)
    assert rc == simulation.SPH_OK
    assert np.array_equal(dens, _via_update(domain, params, pos)["dens"])
