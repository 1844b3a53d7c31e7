"""The FP64 restatement of the learned frame's network (oracle/mpnn_ref.py):
its analytic backward pass against central finite differences (CPU only)."""
import numpy as np

from oracle import mpnn_ref


def _small_case(seed=0, n=60):
    rng = np.random.default_rng(seed)
    h = 0.3
    gx, gy = 5, 4
    pos = np.stack([rng.uniform(0, gx * h, n), rng.uniform(0, gy * h, n)], 1)
    cell = (np.minimum((pos[:, 1] / h).astype(int), gy - 1) * gx + np.minimum((pos[:, 0] / h).astype(int), gx - 1))
    order = np.argsort(cell, kind="stable")
    pos, cell = pos[order], cell[order]
    count = np.bincount(cell, minlength=gx * gy)
    start = np.concatenate([[0], np.cumsum(count)[:-1]])
    I, J = mpnn_ref.edges(pos, start, count, gx, gy, h, cell)
    z0 = rng.normal(0, 0.05, (n, 2))
    target = rng.normal(0, 0.05, (n, 2))
    return pos, z0, target, I, J, h


def test_edges_are_symmetric():
    pos, z0, target, I, J, h = _small_case(3)
    fwd = set(zip(I.tolist(), J.tolist()))
    assert fwd == set((j, i) for i, j in fwd) and len(fwd) == len(I)
    d = np.linalg.norm(pos[J] - pos[I], axis=1)
    assert np.all(d < h) and np.all(I != J)


def test_backward_matches_finite_differences():
    pos, z0, target, I, J, h = _small_case(1)
    flat = mpnn_ref.init_params(7)
    flat = flat + np.random.default_rng(2).normal(0, 0.02, flat.shape)  # nonzero biases too
    u, cache = mpnn_ref.forward(flat, pos, z0, I, J, h)
    grad = mpnn_ref.backward(flat, cache, u, target)
    rng = np.random.default_rng(4)
    idx = rng.choice(mpnn_ref.param_count(), 60, replace=False)
    # Every parameter block of both rounds gets probed.
    blocks = []
    off = 0
    for _ in range(mpnn_ref.ROUNDS):
        for name, shape in mpnn_ref._LAYOUT:
            size = int(np.prod(shape))
            if name == "W3":
                blocks.append(off + np.arange(mpnn_ref.HIDDEN) * mpnn_ref.NODE_IN_PAD + 5)
            else:
                blocks.append(off + np.arange(min(size, 4)))
            off += size
    idx = np.unique(np.concatenate([idx] + blocks))
    eps = 1e-6
    num = np.zeros(len(idx))
    for k, p in enumerate(idx):
        f1, f2 = flat.copy(), flat.copy()
        f1[p] += eps
        f2[p] -= eps
        l1 = mpnn_ref.loss(mpnn_ref.forward(f1, pos, z0, I, J, h)[0], target)
        l2 = mpnn_ref.loss(mpnn_ref.forward(f2, pos, z0, I, J, h)[0], target)
        num[k] = (l1 - l2) / (2 * eps)
    err = np.abs(num - grad[idx])
    scale = np.abs(num) + np.abs(grad[idx]) + 1e-9
    assert np.all((err / scale < 1e-4) | (err < 1e-10)), np.max(err / scale)


def test_padded_inputs_get_no_gradient():
    pos, z0, target, I, J, h = _small_case(5)
    flat = mpnn_ref.init_params(1)
    u, cache = mpnn_ref.forward(flat, pos, z0, I, J, h)
    grad = mpnn_ref.backward(flat, cache, u, target)
    for g in mpnn_ref.unpack(grad):
        assert np.all(g["W3"][:, mpnn_ref.NODE_IN:] == 0)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 65504.0, 1e-30])
    r = mpnn_ref.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # ties to even
    assert r[2] == 1.0078125
    assert abs(r[3] - -3.140625) < 1e-9


def test_tf32_rounding():
    """To nearest with ties away from zero, 10 explicit mantissa bits
    (cvt.rna.tf32.f32): the low 13 bits of the float32 are zero."""
    ulp = 2.0 ** -10
    x = np.array([1.0, 1.0 + ulp / 2, -(1.0 + ulp / 2), 1.0 + 1.5 * ulp, 1.0 + ulp / 2 - 2.0 ** -20, 0.1, 0.0])
    r = mpnn_ref.tf32(x)
    assert r[0] == 1.0
    assert r[1] == 1.0 + ulp and r[2] == -(1.0 + ulp)  # ties away from zero
    assert r[3] == 1.0 + 2 * ulp
    assert r[4] == 1.0
    assert abs(r[5] - 0.1) <= 0.1 * ulp / 2 and r[6] == 0.0
    bits = np.asarray(r, np.float32).view(np.uint32)
    assert np.all(bits & 0x1FFF == 0)
    assert np.array_equal(mpnn_ref.tf32(r), r)
