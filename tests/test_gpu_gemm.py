"""The tcgen05 BF16 GEMM of the learned frame against PyTorch's FP32 matmul
of the same BF16 operands (products of BF16 values are exact in FP32, so the
two differ only by summation order), in each staging form: TMA with
persistent CTAs (several row tiles per CTA, B resident in shared memory,
double-buffered accumulator), plain loads, and TMA with one tile per CTA."""
import ctypes

import numpy as np
import pytest

import nbodysimulation_experiment_gb300 as pkg
from nbodysimulation_experiment_gb300 import simulation

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


def _gemm(lib, a, b, c, bias=None, relu=False, accumulate=False, splits=1, staging=0):
    fn = lib.sph_gemm_bf16
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 6 + [
        ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    m, k = a.shape
    n = b.shape[0]
    return fn(a.data_ptr(), b.data_ptr(), c.data_ptr(), m, n, k, a.stride(0), b.stride(0), c.stride(0),
              bias.data_ptr() if bias is not None else None, int(relu), int(accumulate), splits, staging, None)


@pytest.mark.parametrize("staging", [0, 1, 2])
@pytest.mark.parametrize("m,n,k", [(128, 128, 128), (256, 144, 144), (300, 16, 128), (128, 256, 64),
                                   (1000, 128, 48), (70000, 128, 144), (20000, 256, 128), (5000, 144, 256)])
def test_gemm_matches_fp32_reference(m, n, k, staging):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n + k)
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(n, device="cuda", generator=g)
    c = torch.full((m, n), float("nan"), device="cuda")
    assert _gemm(lib, a, b, c, bias=bias, relu=True, staging=staging) == simulation.SPH_OK
    torch.cuda.synchronize()
    want = torch.relu(a.float() @ b.float().T + bias)
    err = (c - want).norm() / want.norm()
    assert err < REL_TOL, float(err)


def test_gemm_with_leading_dimensions():
    """Operands that are column slices of wider arrays (leading dimension >
    K), as the network's backward pass uses them."""
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    g = torch.Generator(device="cuda").manual_seed(9)
    wide_a = torch.randn(384, 144, device="cuda", generator=g).to(torch.bfloat16)
    wide_b = torch.randn(128, 200, device="cuda", generator=g).to(torch.bfloat16)
    a, b = wide_a[:, :128], wide_b[:, :128]
    c = torch.zeros(384, 128, device="cuda")
    assert _gemm(lib, a, b, c) == simulation.SPH_OK
    torch.cuda.synchronize()
    want = a.float() @ b.float().T
    assert float((c - want).norm() / want.norm()) < REL_TOL


def test_gemm_split_k_accumulates():
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    g = torch.Generator(device="cuda").manual_seed(5)
    a = torch.randn(128, 8192, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(144, 8192, device="cuda", generator=g).to(torch.bfloat16)
    c = torch.ones(128, 144, device="cuda")
    assert _gemm(lib, a, b, c, accumulate=True, splits=8) == simulation.SPH_OK
    torch.cuda.synchronize()
    want = 1.0 + a.float() @ b.float().T
    err = (c - want).norm() / want.norm()
    assert err < REL_TOL, float(err)


def test_gemm_rejects_bad_shapes():
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    a = torch.zeros(128, 40, device="cuda", dtype=torch.bfloat16)
    b = torch.zeros(20, 40, device="cuda", dtype=torch.bfloat16)
    c = torch.zeros(128, 20, device="cuda")
    assert _gemm(lib, a, b, c) == simulation.SPH_ERR_INVALID_ARGUMENT  # N, K not multiples of 16


def test_gemm_persistent_equals_one_tile_per_cta():
    """The persistent and the one-tile-per-CTA TMA forms issue the same MMAs
    in the same order: identical results, bit for bit, over many tiles per
    CTA (M = 262,144: 2,048 row tiles) with bias, ReLU and a K tail."""
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    g = torch.Generator(device="cuda").manual_seed(5)
    m, n, k = 262144, 128, 144
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(n, device="cuda", generator=g)
    out = []
    for staging in (0, 2):
        c = torch.full((m, n), float("nan"), device="cuda")
        assert _gemm(lib, a, b, c, bias=bias, relu=True, staging=staging) == simulation.SPH_OK
        out.append(c)
    torch.cuda.synchronize()
    assert torch.equal(out[0], out[1])
