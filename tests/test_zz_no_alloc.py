"""The allocation-free entry point, through the C ABI, against the library's
regular update.

`sph_density_pressure_noalloc` exists for callers that cannot call
cudaMalloc (their memory belongs to another component's allocator or budget,
or they run in a loop that must not allocate): it takes device pointers for
positions and outputs and keeps its working memory in a fixed device array
inside the library.  Its densities and pressures must equal what one
`sph_update` computes for the same freshly added, motionless particles (the
density pass sees exactly those positions and the same neighbour lists).
Two calls in a row with different particle sets check that the shared
working array carries nothing over from the previous call.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes, simulation

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5  # same single-step tolerance as the parity tests


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


def _positions(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-4.5, 4.5, n), rng.uniform(-2.5, 2.5, n)], 1).astype(np.float32)


def test_density_pressure_noalloc_matches_update_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = pkg.load_library()
    domain = pkg.reference_domain()
    params = pkg.Params.from_array(scenes.scenario_params())
    stream = torch.cuda.current_stream().cuda_stream
    for n, seed in ((3000, 1), (1500, 2)):
        pos = _positions(n, seed)
        ref = _via_update(domain, params, pos)
        pos_dev = torch.from_numpy(pos).cuda()
        dens_dev = torch.full((n, 2), float("nan"), device="cuda")
        press_dev = torch.full((n, 2), float("nan"), device="cuda")
        rc = _noalloc(lib, domain, params, pos_dev.data_ptr(), n, dens_dev.data_ptr(), press_dev.data_ptr(), stream)
        assert rc == simulation.SPH_OK, rc
        torch.cuda.synchronize()
        dens = dens_dev.cpu().numpy()
        press = press_dev.cpu().numpy()
        for got, want in ((dens, ref["dens"]), (press, ref["press"])):
            assert np.all(np.isfinite(got))
            err = np.max(np.abs(got.astype(np.float64) - want)) / np.max(np.abs(want))
            assert err <= REL_TOL, err


def test_density_pressure_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = pkg.load_library()
    domain = pkg.reference_domain()
    params = pkg.default_params()
    # Sizes are checked before any pointer is used or any work is enqueued.
    dummy = ctypes.c_void_p(16)
    rc = _noalloc(lib, domain, params, dummy, 262145, dummy, dummy, None)
    assert rc == simulation.SPH_ERR_CAPACITY
    big = pkg.reference_domain()
    big.width, big.height = 600.0, 300.0  # 2000 x 1000 cells > 262,144
    rc = _noalloc(lib, big, params, dummy, 10, dummy, dummy, None)
    assert rc == simulation.SPH_ERR_CAPACITY
