"""The C-ABI library builds, loads and exports every entry point that
include/sph_gb300.h declares (no GPU needed: nothing is computed)."""
import ctypes
import os
import re

import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import simulation

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(sph_[a-z_0-9]+)\s*\(", src, flags=re.M)
    return names


def test_header_declares_the_interface():
    names = declared_functions()
    for n in simulation.C_SYMBOLS:
        assert n in names, n


def test_library_exports_every_declared_symbol():
    pkg.build()
    lib = ctypes.CDLL(pkg.LIB_PATH)
    for n in declared_functions():
        assert hasattr(lib, n), n


def test_constants_match_the_reference():
    d = pkg.reference_domain()
    assert (d.width, d.height) == (10.0, 5.625)
    assert d.grid() == (33, 18)  # kSPHGridCountX/Y (sph.h:61-62)
    assert (d.max_particles, d.max_cell_particles, d.max_neighbors) == (10000, 500, 1000)
    p = pkg.default_params().as_array()
    assert p[0] == pytest.approx(0.3) and p[4] == 20.0 and p[5] == pytest.approx(0.6)


def test_create_without_gpu_fails_loudly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(pkg.SphError) as e:
        pkg.Simulation()
    assert e.value.status == simulation.SPH_ERR_NO_DEVICE


def test_dump_target_arrays_are_checked():
    """Caller-given dump arrays must match the state's sizes and types; the
    view then points at them (no device needed)."""
    import numpy as np
    n, n0, gx, gy = 5, 4, 3, 2
    out = {k: np.zeros((n, 2), np.float32) for k in ("pos", "prev", "vel", "acc", "dens", "press")}
    out.update(id=np.zeros(n, np.int32), cell=np.zeros(n, np.int32), cell_start=np.zeros(gx * gy, np.int32),
               cell_count=np.zeros(gx * gy, np.int32))
    st, v = simulation._state_view_of(out, n, n0, gx, gy)
    assert st is out and st["canonical_count"] == n0 and st["grid"] == (gx, gy)
    assert v.pos == out["pos"].ctypes.data and v.cell_count == out["cell_count"].ctypes.data
    assert v.count == n and v.canonical_count == n0
    for bad in ({"pos": np.zeros((n + 1, 2), np.float32)}, {"id": np.zeros(n, np.int64)},
                {"vel": np.zeros((2, n), np.float32).T}):
        with pytest.raises(ValueError):
            simulation._state_view_of({**out, **bad}, n, n0, gx, gy)
