"""Viscoelastic springs in the oracle, against an independent NumPy
restatement of the same rules (CPU only).

The reference has no springs; the oracle restates Clavet et al. 2005
("Particle-based viscoelastic fluid simulation", Algorithms 3 and 4) in a
deterministic parallel form: adjust and remove existing springs, add springs
between mutually nearest free candidates, then move every particle by -D/2 of
each of its springs from the positions before the phase (the library's
form).  It also applies the displacements in the paper's own serial form
(Algorithm 3: one spring at a time, positions updated at once).  Both are
pinned here against this independent restatement.

Isolation: viscosity, pressure, gravity and bodies are zero, so within one
update only prediction and the spring phase move particles, and the expected
positions and spring tables follow from the previous state alone.
"""
import numpy as np
import pytest

from nbodysimulation_experiment_gb300 import scenes
from oracle.oracle import OracleSim

F = np.float32
SLOTS = 16
YIELD, PLASTIC, KSPRING = F(0.1), F(0.3), F(0.3)


def _plastic(L, r, dt_alpha):
    d = YIELD * L
    if r > L + d:
        return F(L + dt_alpha * ((r - L) - d))
    if r < L - d:
        return F(L - dt_alpha * ((L - d) - r))
    return F(L)


def _spring_phase(x, count, partner, rest, tag, h, inv_h, dt, max_per=SLOTS, serial=False):
    """One spring phase on float32 positions x (n, 2).  ``serial`` applies
    the displacements as Clavet et al. 2005 write the loop (Algorithm 3):
    foreach spring ij, D from the current positions, x_i -= D/2, x_j += D/2,
    springs in order of their lower end's number, then slot order."""
    n = len(x)
    h2 = F(h * h)
    dt_alpha = F(dt * PLASTIC)
    dt2 = F(dt * dt)
    rij = (x[None, :, :] - x[:, None, :]).astype(F)           # x_j - x_i
    r2 = (rij[..., 0] * rij[..., 0] + rij[..., 1] * rij[..., 1]).astype(F)
    surv = []
    acc = []
    for i in range(n):
        keep = []
        for q in range(count[i]):
            p, L = int(partner[i, q]), F(rest[i, q])
            if r2[i, p] < h2:
                L = _plastic(L, F(np.sqrt(r2[i, p])), dt_alpha)
            if L <= h:
                keep.append((p, L))
        surv.append(keep)
        free = max_per - len(keep)
        existing = set(int(p) for p in partner[i, :count[i]])
        cand = [(r2[i, j], int(tag[j]), j) for j in range(n)
                if j != i and r2[i, j] < h2 and j not in existing]
        cand.sort()
        acc.append([j for _, _, j in cand[:max(free, 0)]])
    springs = []
    for i in range(n):
        lst = list(surv[i])
        for p in acc[i]:
            if i in acc[p]:
                L = _plastic(F(h), F(np.sqrt(r2[i, p])), dt_alpha)
                if L <= h:
                    lst.append((p, L))
        springs.append(lst)
    if serial:
        out = x.copy()
        for i in range(n):
            for p, L in springs[i]:
                if p <= i:
                    continue
                rx, ry = F(out[p, 0] - out[i, 0]), F(out[p, 1] - out[i, 1])
                r = F(np.sqrt(F(F(rx * rx) + F(ry * ry))))
                length = F(1) if r == 0 else r
                inv = F(F(1) / length)
                nx, ny = F(rx * inv), F(ry * inv)
                f = F(F(F(dt2 * KSPRING) * F(F(1) - F(L * inv_h))) * F(L - r))
                hx, hy = F(F(f * nx) * F(0.5)), F(F(f * ny) * F(0.5))
                out[i] = np.array([F(out[i, 0] - hx), F(out[i, 1] - hy)], F)
                out[p] = np.array([F(out[p, 0] + hx), F(out[p, 1] + hy)], F)
        return out, springs
    out = x.copy()
    for i in range(n):
        dx = np.zeros(2, F)
        for p, L in springs[i]:
            r = F(np.sqrt(r2[i, p]))
            length = F(1) if r == 0 else r
            inv = F(F(1) / length)
            nx, ny = F(rij[i, p, 0] * inv), F(rij[i, p, 1] * inv)
            f = F(F(F(dt2 * KSPRING) * F(F(1) - F(L * inv_h))) * F(L - r))
            dx[0] = F(dx[0] - F(F(f * nx) * F(0.5)))
            dx[1] = F(dx[1] - F(F(f * ny) * F(0.5)))
        out[i] = (dx + x[i]).astype(F)
    return out, springs


def _quiet_scene(side=14, seed=5):
    sc = scenes.scaled_block(side, seed=seed, obstacles=False)
    sc.planes = []
    sc.gravity = (0.0, 0.0)
    p = sc.params.copy()
    p[5] = 0.0   # stiffness
    p[6] = 0.0   # near stiffness
    p[7] = 0.0   # linear viscosity
    p[8] = 0.0   # quadratic viscosity
    sc.params = p
    return sc


@pytest.mark.parametrize("serial", [False, True])
def test_spring_phase_matches_restatement(serial):
    sc = _quiet_scene()
    orc = OracleSim(sc.oracle_domain(OracleSim))
    sc.apply(orc)
    orc.set_springs(True, YIELD, PLASTIC, KSPRING, SLOTS, serial=serial)
    dt = F(scenes.DT)
    h, inv_h = F(sc.params[0]), F(sc.params[3])
    n = sc.n
    count = np.zeros(n, np.int32)
    partner = np.full((n, SLOTS), -1, np.int32)
    rest = np.zeros((n, SLOTS), F)
    tag = np.arange(n)
    for step in range(4):
        before = orc.get_state(lists=False)
        x_star = (before["vel"].astype(F) * dt + before["pos"].astype(F)).astype(F)
        want_pos, want_springs = _spring_phase(x_star, count, partner, rest, tag, h, inv_h, dt, serial=serial)
        orc.update(float(dt))
        got = orc.get_state(lists=False)
        assert np.array_equal(got["pos"].astype(F), want_pos), step
        count, partner, rest = orc.get_spring_state()
        for i in range(n):
            assert count[i] == len(want_springs[i]), (step, i)
            for q, (p, L) in enumerate(want_springs[i]):
                assert partner[i, q] == p and rest[i, q] == L, (step, i, q)
    assert count.sum() > 0


def test_springs_are_symmetric_and_bounded():
    sc = scenes.scaled_block(20, seed=9)
    orc = OracleSim(sc.oracle_domain(OracleSim))
    sc.apply(orc)
    orc.set_springs(True, YIELD, PLASTIC, KSPRING, 12)
    for _ in range(8):
        orc.update(float(scenes.DT))
    count, partner, rest = orc.get_spring_state()
    h = F(sc.params[0])
    assert count.max() <= 12 and orc.spring_total() == count.sum() > 0
    for i in range(len(count)):
        for q in range(count[i]):
            j, L = partner[i, q], rest[i, q]
            assert 0 < L <= h
            back = [t for t in range(count[j]) if partner[j, t] == i]
            assert len(back) == 1 and rest[j, back[0]] == L


def test_springs_fp64_close_to_fp32():
    sc = scenes.scaled_block(16, seed=3)
    out = []
    for fp64 in (False, True):
        orc = OracleSim(sc.oracle_domain(OracleSim), fp64=fp64)
        sc.apply(orc)
        orc.set_springs(True, YIELD, PLASTIC, KSPRING, SLOTS)
        orc.update(float(scenes.DT))
        out.append(orc.get_state(lists=False)["pos"].astype(np.float64))
    err = np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[1])
    assert err < 1e-6, err
