"""Failure paths and snapshots on the GPU, through the C ABI.

The reference asserts (Debug) or overruns memory (Release) where a cell or a
neighbour list exceeds its capacity (demo4.cpp:45, 199; sph.h:446), and
waits on its worker threads without a limit (threading.h:101-109).  The
library turns these into status codes; these tests drive each one without a
GPU fault:

* a bounded device-side wait that runs out: a test-only switch makes one
  sweep task never publish that it is done, with a 2 ms wait limit, so its
  dependants give up; the next synchronising call reports SPH_ERR_TIMEOUT,
  and after loading a saved state the simulation continues bit for bit as
  one that never failed;
* a cell beyond the grid update's 512-entry working array, and a 3x3 block
  beyond the 1,024-entry staging buffers: SPH_ERR_DEVICE_OVERFLOW (each is
  caught by the kernels' own capacity checks, which skip the work);
* snapshots: a dumped state (and spring tables) loaded into a fresh
  simulation updates exactly as the original; a state made by the oracle
  loads and updates as the oracle updates it.
"""
import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes
from nbodysimulation_experiment_gb300.simulation import (DELTA_WARPS, SPH_ERR_DEVICE_OVERFLOW, SPH_ERR_TIMEOUT,
                                                        VISC_WARPS, SphError)
from oracle import state as ostate
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu

DT = float(scenes.DT)
FIELDS = ("pos", "prev", "vel", "acc", "dens", "press", "id", "cell", "cell_start", "cell_count")


def _equal_states(a, b):
    for k in FIELDS:
        assert np.array_equal(a[k], b[k]), k
    assert a["canonical_count"] == b["canonical_count"]


def _lean(sim):
    base = sim.sweep_shape()
    sim.set_sweep_shape((VISC_WARPS[1], base[1], DELTA_WARPS[1], base[3]))


@pytest.mark.parametrize("sweep", [0, 1])
@pytest.mark.parametrize("lean", [False, True])
def test_wait_limit_reports_timeout_and_recovers(sweep, lean):
    scene = scenes.dam_break_4096()
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    for _ in range(3):
        sim.update(DT)
    if lean:
        _lean(sim)
    saved = sim.dump_state()
    # The next update from the saved state, without any failure.
    ref = pkg.Simulation(scene.domain())
    scene.apply(ref)
    ref.load_state(saved)
    if lean:
        _lean(ref)
    ref.update(DT)
    want = ref.dump_state()
    ref.close()

    sim.set_wait_limit(0.002)
    sim.test_hold_task(sweep, 0)  # the first task never reports done: its neighbours wait
    sim.update(DT)
    with pytest.raises(SphError) as e:
        sim.synchronize()
    assert e.value.status == SPH_ERR_TIMEOUT
    sim.test_hold_task(sweep, -1)
    sim.set_wait_limit(2.0)
    sim.load_state(saved)
    sim.update(DT)
    _equal_states(sim.dump_state(), want)
    sim.close()


def _cluster_sim(points):
    d = pkg.reference_domain()
    sim = pkg.Simulation(d)
    sim.set_gravity((0.0, -10.0))
    for nx, ny, dist in scenes.box_planes(scenes.REF_WIDTH, scenes.REF_HEIGHT):
        sim.add_plane((nx, ny), dist)
    sim.add_particles(points)
    return sim


def _square(n_side, x0, y0, size):
    g = (np.arange(n_side, dtype=np.float32) + 0.5) * np.float32(size / n_side)
    xx, yy = np.meshgrid(g + np.float32(x0), g + np.float32(y0))
    return np.stack([xx.ravel(), yy.ravel()], 1).astype(np.float32)


def test_cell_beyond_capacity_reports_overflow():
    # 24 x 24 = 576 particles inside one 0.3 x 0.3 cell (cells start at
    # x = -5 + 0.3 k, y = -2.8125 + 0.3 k): more than the 512 entries the
    # grid update holds per cell (the reference's own limit is 500).
    pts = _square(24, -5.0 + 0.3 * 16 + 0.02, -2.8125 + 0.3 * 3 + 0.02, 0.26)
    sim = _cluster_sim(pts)
    sim.update(DT)
    with pytest.raises(SphError) as e:
        sim.synchronize()
    assert e.value.status == SPH_ERR_DEVICE_OVERFLOW
    # The simulation stays usable: a fresh scene steps normally.
    sim.clear_particles()
    sim.add_particles(_square(10, -1.0, -2.0, 0.5))
    sim.update(DT)
    sim.synchronize()
    sim.close()


def test_block_beyond_staging_reports_overflow():
    # Three side-by-side cells of 20 x 20 = 400 particles each: every cell
    # fits the grid update, but the 3x3 block around the middle one lists
    # 1,200 entries, more than the 1,024 a block stages (and than the
    # reference's 1,000-entry neighbour list).
    x0, y0 = -5.0 + 0.3 * 15, -2.8125 + 0.3 * 3
    pts = np.concatenate([_square(20, x0 + 0.3 * k + 0.03, y0 + 0.03, 0.24) for k in range(3)])
    sim = _cluster_sim(pts)
    sim.update(DT)
    with pytest.raises(SphError) as e:
        sim.synchronize()
    assert e.value.status == SPH_ERR_DEVICE_OVERFLOW
    sim.close()


def test_load_state_round_trip():
    scene = scenes.obstacles_65536()
    a = pkg.Simulation(scene.domain())
    scene.apply(a)
    for _ in range(8):
        a.update(DT)
    st = a.dump_state()
    b = pkg.Simulation(scene.domain())
    scene.apply(b)  # bodies, gravity, parameters (the particles are replaced)
    b.load_state(st)
    _equal_states(b.dump_state(), st)
    for _ in range(3):
        a.update(DT)
        b.update(DT)
    _equal_states(a.dump_state(), b.dump_state())
    a.close()
    b.close()


def test_load_state_round_trip_with_springs():
    springs = dict(yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    scene = scenes.scaled_block(64, seed=12)
    a = pkg.Simulation(scene.domain())
    scene.apply(a)
    a.set_springs(True, **springs)
    for _ in range(10):
        a.update(DT)
    st, spr = a.dump_state(), a.dump_springs()
    assert spr[0].sum() > 0
    b = pkg.Simulation(scene.domain())
    scene.apply(b)
    b.set_springs(True, **springs)
    b.load_state(st)
    b.load_springs(*spr)
    for _ in range(2):
        a.update(DT)
        b.update(DT)
    _equal_states(a.dump_state(), b.dump_state())
    for x, y in zip(a.dump_springs(), b.dump_springs()):
        assert np.array_equal(x, y)
    a.close()
    b.close()


def test_load_oracle_made_state():
    """A state the oracle made (its own updates from the scene's start) loads
    into the library and updates as the oracle updates that state."""
    scene = scenes.dam_break_4096()
    orc = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(orc)
    for _ in range(5):
        orc.update(DT)
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    gx, gy = sim.grid
    ref = orc.get_state(lists=False)
    st = ostate.from_reference_state(ref, gx, gy)
    sim.load_state(st)
    got = sim.dump_state()
    for k in ("pos", "prev", "vel", "acc", "dens", "press"):
        assert np.array_equal(ostate.by_id(got, k), np.asarray(ref[k], np.float32)), k
    before = got
    orc.set_state(ostate.to_reference_state(before))
    orc.update(DT)
    sim.update(DT)
    res = ostate.compare_step(before, sim.dump_state(), orc.get_state(lists=False))
    assert res["cells_equal"] == 1.0 and res["pos_ulp"] == 0 and res["vel_ulp"] == 0, res
    sim.close()
    orc.close()


def test_invalid_state_and_springs_are_rejected_without_change():
    """sph_load_state and sph_load_springs check their input on the device;
    an invalid input returns SPH_ERR_INVALID_ARGUMENT and leaves the
    simulation as it was."""
    from nbodysimulation_experiment_gb300.simulation import SPH_ERR_INVALID_ARGUMENT
    springs = dict(yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    scene = scenes.scaled_block(32, seed=13)
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    sim.set_springs(True, **springs)
    for _ in range(4):
        sim.update(DT)
    st, spr = sim.dump_state(), sim.dump_springs()
    bad_cases = []
    for key, k, value in (("cell", 5, -1), ("id", 7, st["id"][8]), ("cell_count", int(np.argmax(st["cell_count"])),
                                                                     10 ** 6)):
        b = {kk: (np.array(vv, copy=True) if isinstance(vv, np.ndarray) else vv) for kk, vv in st.items()}
        b[key][k] = value
        bad_cases.append(b)
    moved = {kk: (np.array(vv, copy=True) if isinstance(vv, np.ndarray) else vv) for kk, vv in st.items()}
    moved["cell"][0] = (moved["cell"][0] + 1) % len(moved["cell_count"])  # outside its cell's range
    bad_cases.append(moved)
    for b in bad_cases:
        with pytest.raises(SphError) as e:
            sim.load_state(b)
        assert e.value.status == SPH_ERR_INVALID_ARGUMENT
        _equal_states(sim.dump_state(), st)
    cnt, part, rest = (np.array(a, copy=True) for a in spr)
    i = int(np.argmax(cnt))
    part[i, 0] = i  # a spring to itself
    with pytest.raises(SphError) as e:
        sim.load_springs(cnt, part, rest)
    assert e.value.status == SPH_ERR_INVALID_ARGUMENT
    for x, y in zip(sim.dump_springs(), spr):
        assert np.array_equal(x, y)
    cnt2 = np.array(spr[0], copy=True)
    cnt2[0] = 17
    with pytest.raises(SphError):
        sim.load_springs(cnt2, spr[1], spr[2])
    # A valid load still works and the run continues as the original.
    sim.load_state(st)
    sim.load_springs(*spr)
    sim.update(DT)
    sim.synchronize()
    sim.close()
