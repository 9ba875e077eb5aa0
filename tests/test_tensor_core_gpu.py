"""The radiance cache's tensor-core building block: one 128 x n x 64 BF16
product on the tcgen05 tensor cores (operands in the K-major shared-memory
layout, FP32 accumulator in tensor memory) against the same product in
float64 on the host.  The operands are BF16 values, so every product is exact
and only the FP32 accumulation rounds."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16(x):
    """round-to-nearest-even to BF16, kept as float32"""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("n", [16, 32, 64])
def test_tcgen05_gemm_matches_host(b200_device, n):
    import ospray_gb300 as og
    rng = np.random.default_rng(n)
    a = _bf16(rng.normal(size=(128, 64)))
    b = _bf16(rng.normal(size=(n, 64)))
    d = og.tensor_core_check(b200_device, a, b)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    np.testing.assert_allclose(d, ref, rtol=1e-5, atol=1e-4)


def test_tcgen05_gemm_layout_is_exact(b200_device):
    """A = identity rows, B = column-index pattern: every output element
    names which (row, column) the hardware paired, so a layout error shows
    as a permutation rather than noise."""
    import ospray_gb300 as og
    a = np.zeros((128, 64), np.float32)
    a[np.arange(128), np.arange(128) % 64] = 1.0
    b = np.tile(np.arange(64, dtype=np.float32) * 0.0 + 1.0, (64, 1)) * (np.arange(64, dtype=np.float32)[:, None] + 1)
    b = b * 0 + np.arange(64, dtype=np.float32)[None, :] + 1.0  # B[j][k] = k + 1
    d = og.tensor_core_check(b200_device, a, b)
    expect = (np.arange(128) % 64 + 1.0)[:, None] * np.ones((1, 64))
    np.testing.assert_array_equal(d, expect)
