"""The pipelined delta sweep's schedule, checked on the CPU.

The pipelined shapes of k_delta evaluate particle k's pairs (producers)
while the summer finishes particle k - 1 (its ordered dx sum and final
position).  The one pair of k that needs x_{k-1} after that sum, (k, k-1),
is reserved in list order and evaluated by the summer right after the sum;
k's own (self) pair is kept aside so that no one sees x_k change before
reading it.  This test restates that schedule in FP32, with the two roles of
a phase in a random order, and checks it against the serial order of the
reference's DeltaPositions (demo4.cpp:239-255, sph.h:483-495) bit for bit.
"""
import numpy as np
import pytest

F = np.float32
H = F(0.3)
DT2 = F((1 / 60) ** 2)


def _half(xj, xk, r2, pk):
    """delta_half: D * 0.5 of one in-range pair in FP32."""
    rx, ry = F(xj[0] - xk[0]), F(xj[1] - xk[1])
    rij = F(np.sqrt(r2))
    ln = rij if rij != F(0) else F(1)
    inv = F(F(1) / ln)
    nx, ny = F(rx * inv), F(ry * inv)
    term = F(F(1) - F(rij * F(1 / H)))
    d = F(DT2 * F(F(pk[0] * term) + F(pk[1] * F(term * term))))
    return np.array([F(F(d * nx) * F(0.5)), F(F(d * ny) * F(0.5))], np.float32)


def _r2(xj, xk):
    rx, ry = F(xj[0] - xk[0]), F(xj[1] - xk[1])
    return F(F(rx * rx) + F(ry * ry))


def _serial(pos, press, own, cnt):
    x = pos.copy()
    for k in range(cnt):
        i = own + k
        xk = x[i].copy()
        dx = np.zeros(2, np.float32)
        after = xk.copy()
        for e in range(len(x)):
            xj = x[e].copy()
            r2 = _r2(xj, xk)
            if not r2 < F(H * H):
                continue
            h = _half(xj, xk, r2, press[i])
            moved = np.array([F(h[0] + xj[0]), F(h[1] + xj[1])], np.float32)
            if e == i:
                after = moved
            else:
                x[e] = moved
            dx = np.array([F(dx[0] - h[0]), F(dx[1] - h[1])], np.float32)
        x[i] = np.array([F(dx[0] + after[0]), F(dx[1] + after[1])], np.float32)
    return x


def _pipelined(pos, press, own, cnt, rng):
    x = pos.copy()
    halves = {}     # particle -> list of D/2 in list order (None = reserved)
    after = {}      # particle -> position after its self pair
    hres = None     # D/2 of the pending particle's reserved pair

    def produce(k):
        i, prev = own + k, own + k - 1 if k >= 1 else -1
        xk = x[i].copy()
        hs, aft = [], xk.copy()
        for e in range(len(x)):
            if e == prev:
                hs.append(None)  # (k, k-1): the summer evaluates it
                continue
            xj = x[e].copy()
            r2 = _r2(xj, xk)
            if not r2 < F(H * H):
                continue
            h = _half(xj, xk, r2, press[i])
            moved = np.array([F(h[0] + xj[0]), F(h[1] + xj[1])], np.float32)
            if e == i:
                aft = moved
            else:
                x[e] = moved
            hs.append(h)
        halves[k], after[k] = hs, aft

    def summer(k):
        """Finish particle k - 1, then evaluate the pair (k, k-1)."""
        nonlocal hres
        j = k - 1
        dx = np.zeros(2, np.float32)
        for h in halves[j]:
            h = hres if h is None else h
            dx = np.array([F(dx[0] - h[0]), F(dx[1] - h[1])], np.float32)
        xp = np.array([F(dx[0] + after[j][0]), F(dx[1] + after[j][1])], np.float32)
        x[own + j] = xp
        hres = np.zeros(2, np.float32)
        if k < cnt:
            xk = x[own + k].copy()
            r2 = _r2(xp, xk)
            if r2 < F(H * H):
                h = _half(xp, xk, r2, press[own + k])
                x[own + j] = np.array([F(h[0] + xp[0]), F(h[1] + xp[1])], np.float32)
                hres = h

    for k in range(cnt + 1):
        roles = []
        if k < cnt:
            roles.append(lambda k=k: produce(k))
        if k >= 1:
            roles.append(lambda k=k: summer(k))
        for r in rng.permutation(len(roles)):
            roles[r]()  # the two roles of a phase touch disjoint data
    return x


@pytest.mark.parametrize("seed", range(6))
def test_pipelined_schedule_equals_serial_order(seed):
    rng = np.random.default_rng(seed)
    counts = rng.integers(3, 9, 9)
    cnt = int(counts[4])
    own = int(counts[:4].sum())
    pos = []
    for c in range(9):
        cx, cy = c % 3, c // 3
        pos.append(np.stack([rng.uniform(cx, cx + 1, counts[c]), rng.uniform(cy, cy + 1, counts[c])], 1) * 0.3)
    pos = np.concatenate(pos).astype(np.float32)
    press = np.stack([rng.uniform(-2, 8, len(pos)), rng.uniform(0, 20, len(pos))], 1).astype(np.float32)
    want = _serial(pos, press, own, cnt)
    for _ in range(3):
        got = _pipelined(pos, press, own, cnt, rng)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
