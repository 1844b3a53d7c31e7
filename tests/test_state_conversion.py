"""Host logic: the canonical (cell-major) renumbering and the conversion of
a GPU-style state dump into the reference's explicit solver state.

Runs on the CPU against the oracle: the reference's own state after a few
updates is renumbered the way the GPU library renumbers, converted back, and
the neighbour lists and cell arrays must equal the reference's, relabelled.
"""
import numpy as np

from nbodysimulation_experiment_gb300 import scenes
from oracle import state as ostate
from oracle.oracle import OracleSim


def colour_rank(gx, gy):
    """The cell order of the GPU library (sph_api.cu, sph_create)."""
    cells = np.arange(gx * gy)
    x, y = cells % gx, cells // gx
    key = (((y % 3) * 3 + (x % 3)) * 4 + ((y // 3) % 2) * 2 + ((x // 3) % 2)) * (1 << 26) + cells
    order = np.argsort(key, kind="stable")
    return order


def canonical_dump(ref, gx, gy):
    """GPU-style dump of a reference state whose particles all have lists."""
    n = len(ref["pos"])
    counts = ref["cell_count"].astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(counts)])
    order = colour_rank(gx, gy)
    start = np.zeros(gx * gy, np.int64)
    run = 0
    for c in order:
        start[c] = run
        run += counts[c]
    new_of_old = np.zeros(n, np.int64)
    for c in range(gx * gy):
        members = ref["cell_flat"][offs[c]:offs[c + 1]].astype(np.int64)
        new_of_old[members] = start[c] + np.arange(len(members))
    dump = {}
    for k in ("pos", "prev", "vel", "acc", "dens", "press"):
        a = np.zeros((n, 2), np.float32)
        a[new_of_old] = ref[k]
        dump[k] = a
    dump["id"] = np.zeros(n, np.int32)
    dump["id"][new_of_old] = np.arange(n)
    cell_lin = ref["cell"][:, 1].astype(np.int64) * gx + ref["cell"][:, 0]
    dump["cell"] = np.zeros(n, np.int32)
    dump["cell"][new_of_old] = cell_lin
    dump["cell_start"] = start.astype(np.int32)
    dump["cell_count"] = counts.astype(np.int32)
    dump["canonical_count"] = n
    dump["grid"] = (gx, gy)
    return dump, new_of_old


def test_canonical_dump_roundtrip_reproduces_reference_lists():
    scene = scenes.dam_break_4096()
    orc = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(orc)
    for _ in range(8):
        orc.update(float(scenes.DT))
    ref = orc.get_state(lists=True)
    dump, new_of_old = canonical_dump(ref, orc.gx, orc.gy)
    back = ostate.to_reference_state(dump)
    n = len(ref["pos"])
    # Lists: particle old i -> new new_of_old[i]; entries relabelled.
    ref_off = np.concatenate([[0], np.cumsum(ref["nb_count"].astype(np.int64))])
    back_off = np.concatenate([[0], np.cumsum(back["nb_count"].astype(np.int64))])
    for i in range(0, n, 7):
        j = new_of_old[i]
        a = new_of_old[ref["nb_flat"][ref_off[i]:ref_off[i + 1]].astype(np.int64)]
        b = back["nb_flat"][back_off[j]:back_off[j + 1]].astype(np.int64)
        assert np.array_equal(a, b)
    # Cell arrays and index-in-cell agree after relabelling.
    assert np.array_equal(back["cell_count"], ref["cell_count"])
    assert np.array_equal(back["index_in_cell"][new_of_old], ref["index_in_cell"])


def test_relabelled_state_steps_identically_to_teacher_forcing():
    """Loading the converted state into the oracle and stepping reproduces the
    physics of the relabelled particles (no state is lost in conversion):
    the next step's neighbour sets and cell sets match the untouched run."""
    scene = scenes.dam_break_4096()
    orc = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(orc)
    for _ in range(5):
        orc.update(float(scenes.DT))
    ref = orc.get_state(lists=True)
    dump, new_of_old = canonical_dump(ref, orc.gx, orc.gy)
    orc2 = OracleSim(scene.oracle_domain(OracleSim))
    orc2.set_params(orc.get_params())
    orc2.set_gravity(0.0, -10.0)
    for nx, ny, d in scene.planes:
        orc2.add_plane(nx, ny, d)
    orc2.set_state(ostate.to_reference_state(dump))
    got = orc2.get_state(lists=False)
    for k in ("pos", "vel", "prev"):
        assert np.array_equal(got[k][new_of_old], ref[k])


def test_cell_arrays_with_appendix():
    # Two canonical particles in cell 0, one appended particle in cell 0 and
    # one in cell 3.
    dump = {
        "pos": np.zeros((4, 2), np.float32), "grid": (2, 2), "canonical_count": 2,
        "cell_start": np.array([0, 2, 2, 2], np.int32), "cell_count": np.array([2, 0, 0, 0], np.int32),
        "cell": np.array([0, 0, 3, 0], np.int32),
    }
    cells = ostate.cell_arrays(dump)
    assert list(cells[0]) == [0, 1, 3] and list(cells[3]) == [2] and len(cells[1]) == 0
