"""Test infrastructure (oracle): FP64 NumPy restatement of the learned
frame's message-passing network, forward and backward.

Only tests use this module.  The network has no counterpart in the
reference; this file defines its arithmetic, and the GPU kernels
(csrc/mpnn_kernels.cu, csrc/mpnn.cu) are checked against it.

Network (per round r = 0, 1, separate weights):
    edges      (i, j), j != i, |x_j - x_i| < h, j in the 3x3 cell block of i
    e_ij     = [d_x/h, d_y/h, r/h, (z_j - z_i)_x, (z_j - z_i)_y, (1 - r/h)^2]
    H_i      = (1/S) sum_j relu(W1 e_ij + b1)                       (128)
    M_i      = W2 H_i + (deg_i / S) b2                              (128)
    c_i      = relu(W3 [M_i, z_i, 0...] + b3)                       (128; input padded to 144)
    z_i     += W4 c_i + b4                                          (2)
with z^0 = v dt / h, output u = z^2 - z^0 and loss mean_i |u_i - t_i|^2.
``emulate_bf16=True`` rounds where the GPU rounds: to BF16 where it
stores BF16 (H, [M, z], c, the GEMM weights W2 and W3, and in the backward
pass da3 and dM), to TF32 the edge layer's inputs (the edge features, W1
and b1, which the tensor cores read as TF32).
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

HIDDEN = 128
EDGE_IN = 6
NODE_IN = 130
NODE_IN_PAD = 144
OUT = 2
ROUNDS = 2
S = 32.0

_LAYOUT = (("W1", (HIDDEN, EDGE_IN)), ("b1", (HIDDEN,)), ("W2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
           ("W3", (HIDDEN, NODE_IN_PAD)), ("b3", (HIDDEN,)), ("W4", (OUT, HIDDEN)), ("b4", (OUT,)))


def round_params() -> int:
    return sum(int(np.prod(s)) for _, s in _LAYOUT)


def param_count() -> int:
    return ROUNDS * round_params()


def unpack(flat: np.ndarray) -> List[Dict[str, np.ndarray]]:
    """Per-round views of the flat parameter vector (the library's order)."""
    out, off = [], 0
    for _ in range(ROUNDS):
        d = {}
        for name, shape in _LAYOUT:
            size = int(np.prod(shape))
            d[name] = flat[off:off + size].reshape(shape)
            off += size
        out.append(d)
    return out


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even) and back, through float32."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def tf32(x: np.ndarray) -> np.ndarray:
    """Round to TF32 (10 explicit mantissa bits), to nearest with ties away
    from zero (PTX cvt.rna.tf32.f32), through float32."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    mag = u & 0x7FFFFFFF
    mag = (mag + 0x1000) & 0x7FFFE000
    u = (u & 0x80000000) | mag
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def edges(pos, cell_start, cell_count, gx: int, gy: int, h: float, cell_of) -> Tuple[np.ndarray, np.ndarray]:
    """Directed edges (i, j) in the GPU's enumeration order: particle i's
    3x3 block of cells y-major, each cell in number order."""
    h2 = np.float32(h) * np.float32(h)
    I, J = [], []
    n = len(pos)
    p32 = pos.astype(np.float32)
    for i in range(n):
        c = int(cell_of[i])
        cx, cy = c % gx, c // gx
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                x, y = cx + dx, cy + dy
                if not (0 <= x < gx and 0 <= y < gy):
                    continue
                c2 = y * gx + x
                js = np.arange(cell_start[c2], cell_start[c2] + cell_count[c2])
                d = p32[js] - p32[i]
                r2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]
                keep = (r2 < h2) & (js != i)
                I.extend([i] * int(keep.sum()))
                J.extend(js[keep].tolist())
    return np.array(I, np.int64), np.array(J, np.int64)


def forward(flat, pos, z0, I, J, h, emulate_bf16=False):
    P = unpack(np.asarray(flat, np.float64))
    rnd = bf16 if emulate_bf16 else (lambda a: a)
    rnd_edge = tf32 if emulate_bf16 else (lambda a: a)
    n = len(pos)
    pos = pos.astype(np.float64)
    d = pos[J] - pos[I]
    r = np.sqrt((d * d).sum(1))
    deg = np.bincount(I, minlength=n).astype(np.float64)
    z = z0.astype(np.float64).copy()
    cache = {"I": I, "J": J, "d": d, "r": r, "deg": deg, "h": h, "rounds": []}
    for rd in range(ROUNDS):
        p = P[rd]
        dz = z[J] - z[I]
        q = r / h
        e = rnd_edge(np.stack([d[:, 0] / h, d[:, 1] / h, q, dz[:, 0], dz[:, 1], (1 - q) ** 2], 1))
        a = e @ rnd_edge(p["W1"]).T + rnd_edge(p["b1"])
        act = np.maximum(a, 0)
        H = np.zeros((n, HIDDEN))
        np.add.at(H, I, act)
        H = rnd(H / S)
        M = H @ rnd(p["W2"]).T + (deg / S)[:, None] * p["b2"]
        X3 = np.zeros((n, NODE_IN_PAD))
        X3[:, :HIDDEN] = M
        X3[:, HIDDEN:HIDDEN + 2] = z
        X3 = rnd(X3)
        pre = X3 @ rnd(p["W3"]).T + p["b3"]
        c = rnd(np.maximum(pre, 0))
        dzn = c @ p["W4"].T + p["b4"]
        cache["rounds"].append({"z": z.copy(), "e": e, "a": a, "H": H, "X3": X3, "c": c})
        z = z + dzn
    u = z - z0.astype(np.float64)
    return u, cache


def loss(u, target) -> float:
    return float(((u - target) ** 2).sum() / len(u))


def backward(flat, cache, u, target, emulate_bf16=False) -> np.ndarray:
    """Gradient of the loss with respect to the flat parameters."""
    P = unpack(np.asarray(flat, np.float64))
    grad = np.zeros(param_count())
    G = unpack(grad)
    rnd = bf16 if emulate_bf16 else (lambda a: a)
    rnd_edge = tf32 if emulate_bf16 else (lambda a: a)
    I, J, deg = cache["I"], cache["J"], cache["deg"]
    n = len(u)
    dz = 2.0 * (u - target) / n
    for rd in reversed(range(ROUNDS)):
        p, g, c_ = P[rd], G[rd], cache["rounds"][rd]
        c, X3, H, a, e = c_["c"], c_["X3"], c_["H"], c_["a"], c_["e"]
        g["W4"][...] = dz.T @ c
        g["b4"][...] = dz.sum(0)
        dc = dz @ p["W4"]
        da3 = rnd(dc * (c > 0))
        g["W3"][...] = da3.T @ X3
        g["b3"][...] = da3.sum(0)
        dX3 = da3 @ rnd(p["W3"])
        dM = rnd(dX3[:, :HIDDEN])
        dz_direct = dX3[:, HIDDEN:HIDDEN + 2]
        g["W2"][...] = dM.T @ H
        g["b2"][...] = ((deg / S)[:, None] * dM).sum(0)
        dH = dM @ rnd(p["W2"])
        da = (dH[I] / S) * (a > 0)
        g["W1"][...] = da.T @ e
        g["b1"][...] = da.sum(0)
        de = da @ rnd_edge(p["W1"])
        dz_edge = np.zeros((n, 2))
        np.add.at(dz_edge, J, de[:, 3:5])
        np.add.at(dz_edge, I, -de[:, 3:5])
        dz = dz + dz_direct + dz_edge
    return grad


def init_params(seed: int) -> np.ndarray:
    """Uniform(+-1/sqrt(fan_in)) weights, zero biases, output layer x0.1."""
    rng = np.random.default_rng(seed)
    flat = np.zeros(param_count())
    for p in unpack(flat):
        for name, fan in (("W1", EDGE_IN), ("W2", HIDDEN), ("W3", NODE_IN), ("W4", HIDDEN)):
            lim = 1.0 / np.sqrt(fan)
            p[name][...] = rng.uniform(-lim, lim, p[name].shape)
        p["W3"][:, NODE_IN:] = 0.0
        p["W4"] *= 0.1
    return flat
