"""Long rollouts: the GPU against the reference's update order, by statistics.

Each update is bit-identical to the reference's update of the same numbered
state (the parity tests); free-running, the GPU's renumbering changes the
order of the Gauss-Seidel sweeps relative to the reference's AddParticle
order, and a dam break is chaotic, so trajectories diverge particle by
particle.  Over hundreds of updates they are compared the way the physics
is: kinetic energy, mean height, the density histogram and the mean density
deviation (and, with springs, the spring count and mean rest length).  The
CPU side is the oracle in its single-worker (reference) order.
"""
import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import scenes
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu

DT = float(scenes.DT)


def _stats(pos, vel, dens, rho0):
    ke = 0.5 * np.mean(np.sum(np.asarray(vel, np.float64) ** 2, axis=1))
    hist, _ = np.histogram(dens[:, 0], bins=24, range=(0, 48))
    return {"ke": ke, "hist": hist / len(dens), "mean_y": float(np.mean(pos[:, 1])),
            "dev": float(np.mean(np.abs(dens[:, 0] - rho0)) / rho0)}


def test_dam_break_rollout_statistics():
    scene = scenes.dam_break_4096()
    gpu = pkg.Simulation(scene.domain())
    scene.apply(gpu)
    ref = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(ref)
    rho0 = float(scene.params[4])
    kes = []
    for step in range(1, 301):
        gpu.update(DT)
        ref.update(DT)
        if step % 30:
            continue
        g = gpu.read_particles(("pos", "vel", "dens"))
        r = ref.get_state(lists=False)
        a = _stats(g["pos"], g["vel"], g["dens"], rho0)
        b = _stats(r["pos"], r["vel"], r["dens"], rho0)
        kes.append((a["ke"], b["ke"]))
        if step <= 150:  # before the sloshing phase, energies track closely
            assert abs(a["ke"] - b["ke"]) <= 0.1 * b["ke"], (step, a["ke"], b["ke"])
        assert abs(a["mean_y"] - b["mean_y"]) <= 0.06, (step, a["mean_y"], b["mean_y"])
        assert np.abs(a["hist"] - b["hist"]).sum() <= 0.2, step
        assert abs(a["dev"] - b["dev"]) <= 0.02, (step, a["dev"], b["dev"])
    kg, kr = np.array(kes).T
    assert abs(kg.mean() - kr.mean()) <= 0.1 * kr.mean(), (kg.mean(), kr.mean())


def test_springs_rollout_statistics():
    scene = scenes.scaled_block(32, seed=21)
    gpu = pkg.Simulation(scene.domain())
    scene.apply(gpu)
    gpu.set_springs(True, yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    ref = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(ref)
    ref.set_springs(True, 0.1, 0.3, 0.3, 16)
    for step in range(1, 121):
        gpu.update(DT)
        ref.update(DT)
        if step % 20:
            continue
        cg, _, lg = gpu.dump_springs()
        cr, _, lr = ref.get_spring_state()
        ng, nr = gpu.spring_count(), ref.spring_total() // 2
        assert abs(ng - nr) <= 0.02 * nr, (step, ng, nr)
        mg = lg[cg[:, None] > np.arange(16)].mean()
        mr = lr[cr[:, None] > np.arange(16)].mean()
        assert abs(mg - mr) <= 0.03 * mr, (step, mg, mr)
        vg = gpu.read_particles(("vel",))["vel"]
        vr = ref.get_state(lists=False)["vel"]
        keg = 0.5 * np.mean(np.sum(vg.astype(np.float64) ** 2, 1))
        ker = 0.5 * np.mean(np.sum(vr ** 2, 1))
        assert abs(keg - ker) <= 0.1 * ker, (step, keg, ker)


def test_springs_rollout_against_the_papers_serial_form():
    """The library applies spring displacements from the positions before
    the phase (every particle at once); Clavet et al. 2005 (Algorithm 3)
    apply them one spring at a time with immediate position updates.  Over
    160 free updates of a 1,600-particle block the GPU's form and the
    oracle's serial form (in the oracle's own particle order) agree in
    spring count, mean rest length, kinetic energy, mean height and density
    histogram.  On the CPU the two forms alone (same order otherwise) differ
    by < 0.1% in spring count, < 0.05% in rest length, < 0.7% in kinetic
    energy and < 0.04 in histogram L1 over the same run."""
    springs = dict(yield_ratio=0.1, plasticity=0.3, stiffness=0.3, max_per_particle=16)
    scene = scenes.scaled_block(40, seed=31)
    gpu = pkg.Simulation(scene.domain())
    scene.apply(gpu)
    gpu.set_springs(True, **springs)
    ref = OracleSim(scene.oracle_domain(OracleSim))
    scene.apply(ref)
    ref.set_springs(True, serial=True, **springs)
    rho0 = float(scene.params[4])
    worst = {"springs": 0.0, "rest": 0.0, "ke": 0.0, "hist": 0.0, "y": 0.0}
    for step in range(1, 161):
        gpu.update(DT)
        ref.update(DT)
        if step % 20:
            continue
        cg, _, lg = gpu.dump_springs()
        cr, _, lr = ref.get_spring_state()
        ng, nr = gpu.spring_count(), ref.spring_total() // 2
        mg = lg[cg[:, None] > np.arange(16)].mean()
        mr = lr[cr[:, None] > np.arange(16)].mean()
        g = gpu.read_particles(("pos", "vel", "dens"))
        r = ref.get_state(lists=False)
        a = _stats(g["pos"], g["vel"], g["dens"], rho0)
        b = _stats(r["pos"], r["vel"], r["dens"], rho0)
        worst["springs"] = max(worst["springs"], abs(ng - nr) / nr)
        worst["rest"] = max(worst["rest"], abs(mg - mr) / mr)
        worst["ke"] = max(worst["ke"], abs(a["ke"] - b["ke"]) / b["ke"])
        worst["hist"] = max(worst["hist"], float(np.abs(a["hist"] - b["hist"]).sum()))
        worst["y"] = max(worst["y"], abs(a["mean_y"] - b["mean_y"]))
    print("library springs vs the paper's serial form, worst over 160 updates:", worst)
    # Measured on GB300: springs 0.5%, rest length 2.4%, kinetic energy 4.5%,
    # histogram 0.096 -- mostly the library's own sweep order (the rest
    # length drifts with the order of the density relaxation), not the form
    # of the spring application.
    assert worst["springs"] <= 0.02 and worst["rest"] <= 0.04 and worst["ke"] <= 0.1, worst
    assert worst["hist"] <= 0.15 and worst["y"] <= 0.06, worst
