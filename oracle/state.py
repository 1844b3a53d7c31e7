"""Test infrastructure: conversion between the GPU library's state dump and
the reference's full solver state, and parity comparisons.

Only tests, ``__graft_entry__.smoke()`` and the benchmark's CPU-baseline leg
use this module.

The GPU library keeps its state "canonical": the particles of cell c are the
consecutive numbers ``cell_start[c] .. cell_start[c]+cell_count[c]-1``;
numbers at or above ``canonical_count`` were added since the last update and
sit, in number order, at the end of their cell's array.  The reference's
``Demo4::ParticleSimulation`` state (demo4.h:122-162) holds the same thing
explicitly: per cell an index array, per particle its cell, its position in
the cell array and its neighbour list.  A particle's list is what
``NeighborSearch`` (demo4.cpp:183-206) built at the last update: the cell
arrays of the clamped 3x3 block, y-major then x -- which, between updates,
are the first ``cell_count`` members of each cell.  New particles have an
empty list (``ParticleIndex()``, demo4.cpp:148).
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np


def cell_arrays(gpu: Dict[str, np.ndarray]):
    """Per-cell index arrays (list of numpy arrays) of a GPU dump."""
    gx, gy = gpu["grid"]
    n = len(gpu["pos"])
    n0 = int(gpu["canonical_count"])
    start, count = gpu["cell_start"], gpu["cell_count"]
    cells = [np.arange(start[c], start[c] + count[c], dtype=np.int64) for c in range(gx * gy)]
    if n > n0:
        extra = np.arange(n0, n)
        owner = gpu["cell"][n0:]
        for c in np.unique(owner):
            cells[c] = np.concatenate([cells[c], extra[owner == c]])
    return cells


def to_reference_state(gpu: Dict[str, np.ndarray]) -> Dict[str, np.ndarray]:
    """Reference solver state (oracle ``set_state`` dict) for a GPU dump."""
    gx, gy = gpu["grid"]
    n = len(gpu["pos"])
    n0 = int(gpu["canonical_count"])
    cells = cell_arrays(gpu)
    cell = gpu["cell"].astype(np.int64)
    cxy = np.stack([cell % gx, cell // gx], 1).astype(np.int32)
    index_in_cell = np.zeros(n, np.uint64)
    for c, arr in enumerate(cells):
        if len(arr):
            index_in_cell[arr] = np.arange(len(arr), dtype=np.uint64)
    start, count = gpu["cell_start"], gpu["cell_count"]
    # One list per cell (all particles of a cell share it).
    block_list = {}
    nb_count = np.zeros(n, np.uint64)
    lists = []
    for c in range(gx * gy):
        if count[c] == 0:
            continue
        x, y = c % gx, c // gx
        parts = []
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                xx, yy = x + dx, y + dy
                if 0 <= xx < gx and 0 <= yy < gy:
                    c2 = yy * gx + xx
                    parts.append(np.arange(start[c2], start[c2] + count[c2], dtype=np.uint64))
        block_list[c] = np.concatenate(parts) if parts else np.zeros(0, np.uint64)
    order = []
    for k in range(n0):
        lst = block_list[int(cell[k])]
        nb_count[k] = len(lst)
        order.append(lst)
    nb_flat = np.concatenate(order) if order else np.zeros(0, np.uint64)
    cell_count = np.array([len(a) for a in cells], np.uint64)
    cell_flat = np.concatenate(cells).astype(np.uint64) if n else np.zeros(0, np.uint64)
    st = {k: np.asarray(gpu[k]) for k in ("pos", "prev", "acc", "vel", "dens", "press")}
    st.update(cell=cxy, index_in_cell=index_in_cell, nb_count=nb_count, nb_flat=nb_flat,
              cell_count=cell_count, cell_flat=cell_flat)
    return st


def reference_cells_by_id(ref: Dict[str, np.ndarray], ids: np.ndarray):
    """Reference cell arrays with particle numbers replaced by ids."""
    out = []
    off = 0
    for cnt in ref["cell_count"]:
        cnt = int(cnt)
        out.append(ids[ref["cell_flat"][off:off + cnt].astype(np.int64)])
        off += cnt
    return out


def gpu_cells_by_id(gpu: Dict[str, np.ndarray]):
    ids = gpu["id"].astype(np.int64)
    return [ids[a] for a in cell_arrays(gpu)]


def by_id(gpu: Dict[str, np.ndarray], key: str) -> np.ndarray:
    """A GPU dump array reordered into id (AddParticle) order."""
    out = np.empty_like(gpu[key])
    out[gpu["id"].astype(np.int64)] = gpu[key]
    return out


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """Normwise relative error max|a-b| / max|b| over all components."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    scale = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / (scale if scale > 0 else 1.0)


def ulp_diff(a: np.ndarray, b: np.ndarray) -> int:
    """Largest distance in units in the last place between two float32 arrays."""
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return int(np.max(np.abs(a - b))) if a.size else 0


def compare_step(gpu_before: Dict[str, np.ndarray], gpu_after: Dict[str, np.ndarray],
                 ref_after: Dict[str, np.ndarray]) -> Dict[str, float]:
    """Compare one GPU update with the reference's update of the same state.

    ``ref_after`` is in the numbering of ``gpu_before`` (the reference never
    renumbers); ``gpu_after`` is renumbered and is matched through ``id``.
    Returns per-field relative errors and ulp distances and whether the cell
    arrays are identical (as sequences of particle ids).
    """
    ids_before = gpu_before["id"].astype(np.int64)
    n = len(ref_after["pos"])
    if len(gpu_after["pos"]) != n:
        raise ValueError("particle counts differ: GPU %d, reference %d" % (len(gpu_after["pos"]), n))
    # Particles the update itself added (emitters) keep their AddParticle
    # index as number in the reference.
    ids_ref = np.concatenate([ids_before, np.arange(len(ids_before), n, dtype=np.int64)])
    out = {}
    for key in ("pos", "prev", "vel", "dens", "press"):
        ref = np.empty((n, 2), np.float32)
        ref[ids_ref] = np.asarray(ref_after[key], np.float32)
        mine = by_id(gpu_after, key)
        out[key + "_rel"] = rel_err(mine, ref)
        out[key + "_ulp"] = ulp_diff(mine, ref)
    ref_cells = reference_cells_by_id(ref_after, ids_ref)
    gpu_cells = gpu_cells_by_id(gpu_after)
    out["cells_equal"] = float(all(np.array_equal(a, b) for a, b in zip(ref_cells, gpu_cells)))
    out["cell_sets_equal"] = float(all(np.array_equal(np.sort(a), np.sort(b)) for a, b in zip(ref_cells, gpu_cells)))
    return out


def colour_rank_order(gx: int, gy: int) -> np.ndarray:
    """Cells in the library's numbering order: colour (y%3, x%3), then
    sub-colour ((y/3)%2, (x/3)%2), then row-major."""
    c = np.arange(gx * gy, dtype=np.int64)
    x, y = c % gx, c // gx
    key = (((y % 3) * 3 + (x % 3)) * 4 + ((y // 3) % 2) * 2 + ((x // 3) % 2)) * (1 << 26) + c
    return c[np.argsort(key, kind="stable")]


def from_reference_state(ref: Dict[str, np.ndarray], gx: int, gy: int) -> Dict[str, np.ndarray]:
    """A library state (``sph_load_state`` dict) holding the reference solver
    state ``ref`` (oracle ``get_state``), every particle canonical: particles
    are numbered cell by cell in the library's cell order, each cell's members
    in the reference's cell-array order; ``id`` keeps the reference's index.
    Valid where every particle has the list NeighborSearch builds from the
    current cell arrays, i.e. after an update without added particles."""
    n = len(ref["pos"])
    cnt = np.asarray(ref["cell_count"], np.int64)
    flat = np.asarray(ref["cell_flat"], np.int64)
    off = np.concatenate([[0], np.cumsum(cnt)])
    order = colour_rank_order(gx, gy)
    numbered = np.concatenate([flat[off[c]:off[c + 1]] for c in order]) if n else np.zeros(0, np.int64)
    start = np.zeros(gx * gy, np.int32)
    run = 0
    for c in order:
        start[c] = run
        run += int(cnt[c])
    cell = np.asarray(ref["cell"], np.int64)
    lin = (cell[:, 1] * gx + cell[:, 0]).astype(np.int32)
    st = {k: np.ascontiguousarray(np.asarray(ref[k], np.float32)[numbered]) for k in
          ("pos", "prev", "vel", "acc", "dens", "press")}
    st.update(id=numbered.astype(np.int32), cell=lin[numbered], cell_start=start,
              cell_count=cnt.astype(np.int32), canonical_count=n, grid=(gx, gy))
    return st
