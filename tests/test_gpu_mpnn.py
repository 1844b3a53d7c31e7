"""The learned frame on the GPU: its network against the FP64 oracle
(forward and every parameter gradient), training on samples of plain
frames, the judge and fallback, and what a trained network gains.

Samples come from the plain method: from a canonical state, one plain
update over the whole frame (dt = 1/60) gives the inputs x1 and
z0 = (x1 - x_prev) / h, and the target is (x4 - x1) / h with x4 the
positions after the reference's four substeps of dt/4.  The method without
the network is that single update (u = 0).
"""
import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import learned, scenes
from oracle import mpnn_ref

pytestmark = pytest.mark.gpu

FRAME = float(scenes.DT)
SUBSTEPS = 4
GRAD_TOL = 2e-2   # relative norm per parameter block (BF16 activations and weights)
FWD_TOL = 1e-2


def _sim(scene, warm=3):
    sim = pkg.Simulation(scene.domain())
    scene.apply(sim)
    for _ in range(warm):
        sim.update(FRAME / SUBSTEPS)
    return sim


def _oracle_case(sample):
    gx, gy = sample["grid"]
    start, count = sample["cell_start"], sample["cell_count"]
    n = len(sample["pos"])
    cell_of = np.zeros(n, np.int64)
    for c in np.nonzero(count)[0]:
        cell_of[start[c]:start[c] + count[c]] = c
    I, J = mpnn_ref.edges(sample["pos"], start, count, gx, gy, sample["h"], cell_of)
    return I, J


@pytest.mark.parametrize("edge_path", [pkg.Mpnn.EDGE_TENSOR_CORES, pkg.Mpnn.EDGE_CUDA_CORES])
def test_forward_and_gradients_match_oracle(edge_path):
    scene = scenes.scaled_block(20, seed=3)
    sim = _sim(scene)
    model = pkg.Mpnn(4096, seed=11)
    assert model.edge_path == pkg.Mpnn.EDGE_TENSOR_CORES  # the default
    model.edge_path = edge_path
    p = model.get_params()
    # Nonzero biases so that every parameter block is exercised.
    p = p + np.random.default_rng(0).normal(0, 0.02, p.shape).astype(np.float32)
    model.set_params(p)
    model.capture(sim, FRAME, SUBSTEPS)
    s = model.sample(0)
    I, J = _oracle_case(s)
    flat = model.get_params().astype(np.float64)
    u_ref, cache = mpnn_ref.forward(flat, s["pos"], s["z0"], I, J, s["h"], emulate_bf16=True)
    g_ref = mpnn_ref.backward(flat, cache, u_ref, s["target"].astype(np.float64), emulate_bf16=True)
    loss_gpu, u_gpu = model.eval(0, want_u=True)
    err_u = np.linalg.norm(u_gpu - u_ref) / np.linalg.norm(u_ref)
    assert err_u < FWD_TOL, err_u
    assert abs(loss_gpu - mpnn_ref.loss(u_ref, s["target"])) <= 1e-2 * loss_gpu
    loss2, g_gpu = model.gradient(0)
    assert abs(loss2 - loss_gpu) <= 1e-6 * max(loss_gpu, 1e-12)
    for rd, (gg, gr) in enumerate(zip(mpnn_ref.unpack(g_gpu.astype(np.float64)), mpnn_ref.unpack(g_ref))):
        for name in gr:
            num = np.linalg.norm(gg[name] - gr[name])
            den = np.linalg.norm(gr[name])
            assert den > 0, (rd, name)
            assert num / den < GRAD_TOL, (rd, name, num / den)
    model.close()
    sim.close()


def test_edge_layer_paths_agree_on_dense_and_isolated_particles():
    """The tensor-core edge layer against the CUDA-core one and the oracle
    on a dense cluster (spacing h/9: ~250 edges per particle, so a
    particle's run of columns spans two or three 128-column tiles, and ~80
    particles per cell, so a cell takes ten batches) plus three isolated
    particles (no edges: H = 0).  A frame of 1e-6 s keeps the captured
    positions at the lattice."""
    h = float(scenes.H)
    sim = pkg.Simulation(pkg.reference_domain())
    sim.set_params(pkg.Params.from_array(scenes.scenario_params()))
    for nx, ny, d in scenes.box_planes(scenes.REF_WIDTH, scenes.REF_HEIGHT):
        sim.add_plane((nx, ny), d)
    dense = scenes.jittered_lattice(36, 36, -3.0, -2.0, spacing=np.float32(h / 9.0), jitter=np.float32(0.02 * h), seed=5)
    lone = np.array([[3.0, 2.0], [3.8, -2.0], [4.5, 0.5]], np.float32)
    sim.add_particles(np.concatenate([dense, lone]))
    sim.update(1e-6)
    model = pkg.Mpnn(4096, seed=12)
    p = model.get_params()
    model.set_params(p + np.random.default_rng(1).normal(0, 0.02, p.shape).astype(np.float32))
    model.capture(sim, 1e-6, SUBSTEPS)
    s = model.sample(0)
    I, J = _oracle_case(s)
    deg = np.bincount(I, minlength=len(s["pos"]))
    assert deg.max() > 2 * 128 and np.count_nonzero(deg == 0) == 3, (deg.max(), np.count_nonzero(deg == 0))
    u_ref, _ = mpnn_ref.forward(model.get_params().astype(np.float64), s["pos"], s["z0"], I, J, s["h"],
                                emulate_bf16=True)
    out = {}
    for path in (pkg.Mpnn.EDGE_TENSOR_CORES, pkg.Mpnn.EDGE_CUDA_CORES):
        model.edge_path = path
        out[path] = model.eval(0, want_u=True)[1].astype(np.float64)
        err = np.linalg.norm(out[path] - u_ref) / np.linalg.norm(u_ref)
        assert err < FWD_TOL, (path, err)
    diff = np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[1])
    assert diff < 5e-3, diff  # same function, different summation order (then BF16 H)
    model.close()
    sim.close()


def _samples(model, scene, frames, warm=3):
    sim = _sim(scene, warm)
    for _ in range(frames):
        model.capture(sim, FRAME, SUBSTEPS)
    sim.close()


def test_training_reduces_the_loss():
    model = pkg.Mpnn(8192, seed=2)
    _samples(model, scenes.dam_break_4096(seed=1), 6)
    before = np.mean([model.eval(k) for k in range(model.sample_count)])
    # Weight gradients are summed with atomics, so the trajectory varies a
    # little from run to run; 400 steps leave a clear margin under one half.
    for it in range(400):
        model.train_step(it % model.sample_count, 1e-3)
    after = np.mean([model.eval(k) for k in range(model.sample_count)])
    assert after < 0.5 * before, (before, after)
    model.close()


def test_judge_falls_back_to_the_plain_frame():
    scene = scenes.scaled_block(24, seed=5)
    model = pkg.Mpnn(4096, seed=3)
    a, b = _sim(scene), _sim(scene)
    for _ in range(3):
        used, err = a.learned_frame(model, FRAME, SUBSTEPS, bound=-1.0)  # nothing passes
        assert not used and np.isfinite(err)
        for _ in range(SUBSTEPS):
            b.update(FRAME / SUBSTEPS)
    sa, sb = a.dump_state(), b.dump_state()
    for k in ("pos", "prev", "vel", "dens", "press", "id", "cell_start", "cell_count"):
        assert np.array_equal(sa[k], sb[k]), k
    used, err = a.learned_frame(model, FRAME, SUBSTEPS, bound=1e9)  # everything passes
    assert used and np.isfinite(err)
    st = a.dump_state()
    assert np.all(np.isfinite(st["pos"])) and np.array_equal(np.sort(st["id"]), np.arange(scene.n))
    a.close()
    b.close()


def test_judge_is_deterministic():
    """The judge's density deviation is summed in a fixed order: the same
    frame from the same state gives the same deviation and verdict, bit for
    bit, however often it is repeated."""
    scene = scenes.scaled_block(48, seed=7)
    model = pkg.Mpnn(4096, seed=4)
    sim = _sim(scene)
    st = sim.dump_state()
    seen = set()
    for _ in range(5):
        sim.load_state(st)
        used, err = sim.learned_frame(model, FRAME, SUBSTEPS, bound=1e9)
        seen.add((used, np.float32(err).tobytes()))
        after = sim.dump_state()["pos"].tobytes()
        seen.add(after)
    assert len(seen) == 2, "the learned frame or its judged deviation varied between repeats"
    sim.close()


def test_trained_network_gains_over_the_method_without_it():
    """Held-out frames: the trained network's correction beats the single
    plain update without it (u = 0) by a wide margin, and the judge takes
    learned frames."""
    model = pkg.Mpnn(8192, seed=4)
    train = learned.collect(model, lambda s: scenes.dam_break_4096(seed=s), (1, 2), 8)
    learned.collect(model, lambda s: scenes.dam_break_4096(seed=s), (3,), 4)
    learned.train(model, 600, indices=range(train))
    ev = learned.evaluate(model, range(train, model.sample_count))
    assert ev["learned"] < 0.5 * ev["without_network"], ev
    sim = _sim(scenes.dam_break_4096(seed=3), warm=3)
    used = [sim.learned_frame(model, FRAME, SUBSTEPS, bound=0.01)[0] for _ in range(10)]
    assert sum(used) >= 6, used
    sim.close()
    model.close()
