"""Host logic: seeded scene generation (CPU only)."""
import numpy as np
import pytest

from nbodysimulation_experiment_gb300 import scenes


@pytest.mark.parametrize("side", [8, 16, 24, 32, 64, 128])
def test_scaled_block_fits_box(side):
    sc = scenes.scaled_block(side, seed=side)
    assert sc.n == side * side
    hw, hh = sc.width / 2, sc.height / 2
    assert np.all(np.abs(sc.positions[:, 0]) < hw) and np.all(np.abs(sc.positions[:, 1]) < hh)
    assert len(sc.circles) == 8 and len(sc.segments) == 4
    for x, y, r in sc.circles:
        assert abs(x) + r < hw and abs(y) + r < hh


def test_named_scenes_are_seeded_and_reproducible():
    a = scenes.dam_break_4096()
    b = scenes.dam_break_4096()
    assert np.array_equal(a.positions, b.positions)
    assert a.n == 4096
    # 64x64 lattice at spacing h/6 = 0.05 with +-0.1h jitter, lower-left at
    # (-4.9, -2.7125) in the reference's 10 x 5.625 box.
    assert abs(a.positions[:, 0].min() - (-4.9)) <= 0.031
    assert abs(a.positions[:, 1].min() - (-2.7125)) <= 0.031
    ob = scenes.obstacles_65536()
    assert ob.n == 65536 and len(ob.circles) == 8 and len(ob.segments) == 4
    for _, _, r in ob.circles:
        assert 2 * 0.3 - 1e-6 <= r <= 6 * 0.3 + 1e-6


def test_box_planes_follow_load_scenario():
    planes = scenes.box_planes(10.0, 5.625)
    # distance = dot(normal, position) (app.cpp:489-491)
    assert planes[0] == (0.0, 1.0, -2.8125)
    assert planes[1] == (0.0, -1.0, -2.8125)
    assert planes[2] == (1.0, 0.0, -5.0)
    assert planes[3] == (-1.0, 0.0, -5.0)
