"""The wide viscosity sweep's two-lane schedule, checked on the CPU.

The sweep (k_viscosity<ViscWide>) runs one cell's particles k = 0, 1, ...
(list slots own + k of their shared stale list) as: the head of k (its pairs
before slot own + k - 1) in lockstep with the tail of k - 1 (its pairs after
slot own + k), then the middle of k (its pairs at slots own + k - 1 ..
own + k + 1).  This test restates that schedule in FP32 with every
interleaving of the two lanes chosen at random, and checks that it gives the
same velocities, bit for bit, as the reference's serial order
(demo4.cpp:223-237, sph.h:497-512): every velocity sees the pairs that touch
it in the same order.
"""
import numpy as np
import pytest

F = np.float32


def _geometry(pos, i, h):
    """In-range pairs of particle i over the whole list: (slot, nx, ny, 1 - q)."""
    out = []
    for e in range(len(pos)):
        rx, ry = F(pos[e, 0] - pos[i, 0]), F(pos[e, 1] - pos[i, 1])
        r2 = F(rx * rx + ry * ry)
        if not r2 < F(h * h):
            continue
        r = F(np.sqrt(r2))
        ln = r if r != F(0) else F(1)
        inv = F(F(1) / ln)
        out.append((e, F(rx * inv), F(ry * inv), F(F(1) - F(r * F(1 / h)))))
    return out


def _pair(vel, vi, g, sigma=F(0.5), beta=F(0.3), hdt=F(0.5 / 60)):
    """One pair of the viscosity chain: visc_pair's operations in FP32."""
    j, nx, ny, o = g
    vj = vel[j].copy()
    uu = F(F(F(vi[0] - vj[0]) * nx) + F(F(vi[1] - vj[1]) * ny))
    f = F(o * F(F(sigma * uu) + F(beta * F(uu * uu))))
    ix, iy = F(F(f * nx) * hdt), F(F(f * ny) * hdt)
    if uu > F(0):
        vi = np.array([F(vi[0] - ix), F(vi[1] - iy)], np.float32)
        vel[j] = np.array([F(ix + vj[0]), F(iy + vj[1])], np.float32)
    return vi


def _serial(pos, vel, own, cnt, h):
    vel = vel.copy()
    for k in range(cnt):
        i = own + k
        vi = vel[i].copy()
        for g in _geometry(pos, i, h):
            vi = _pair(vel, vi, g)
        vel[i] = vi
    return vel


def _two_lane(pos, vel, own, cnt, h, rng):
    vel = vel.copy()
    geo = [_geometry(pos, own + k, h) for k in range(cnt)]
    tail_vi = None
    for k in range(cnt + 1):
        head = [g for g in geo[k] if g[0] < own + k - 1] if k < cnt else []
        tail = [g for g in geo[k - 1] if g[0] > own + k] if k >= 1 else []
        vi_h = vel[own + k].copy() if k < cnt else None
        vi_t = tail_vi
        # The two lanes' steps in a random interleaving (lockstep is one of
        # them): they touch disjoint slots.
        steps = [("h", g) for g in head] + [("t", g) for g in tail]
        order = rng.permutation(len(steps))
        hi = ti = 0
        for idx in order:
            lane = steps[idx][0]
            if lane == "h":
                vi_h = _pair(vel, vi_h, head[hi])
                hi += 1
            else:
                vi_t = _pair(vel, vi_t, tail[ti])
                ti += 1
        if k >= 1:
            vel[own + k - 1] = vi_t  # particle k - 1 is finished
        if k < cnt:
            for g in geo[k]:
                if own + k - 1 <= g[0] <= own + k + 1:
                    vi_h = _pair(vel, vi_h, g)
            tail_vi = vi_h
    return vel


@pytest.mark.parametrize("seed", range(6))
def test_two_lane_schedule_equals_serial_order(seed):
    rng = np.random.default_rng(seed)
    h = F(0.3)
    # A 3x3 block of cells in list order; the task's cell is the fifth.
    counts = rng.integers(3, 9, 9)
    cnt = int(counts[4])
    own = int(counts[:4].sum())
    pos = []
    for c in range(9):
        cx, cy = c % 3, c // 3
        pos.append(np.stack([rng.uniform(cx, cx + 1, counts[c]), rng.uniform(cy, cy + 1, counts[c])], 1) * 0.3)
    pos = np.concatenate(pos).astype(np.float32)
    vel = rng.normal(0, 1, pos.shape).astype(np.float32)
    want = _serial(pos, vel, own, cnt, h)
    for _ in range(3):
        got = _two_lane(pos, vel, own, cnt, h, rng)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
