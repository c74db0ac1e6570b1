"""The tensor-core (tcgen05) building block: hodlr_tc_selftest multiplies two
BF16 matrices with tcgen05.mma, operands in shared memory in the K-major
core-matrix layout, the FP32 accumulator in tensor memory.  Checked against
the exact product of the same BF16 values (FP64 on the host): only FP32
accumulation rounding separates them."""
import numpy as np
import pytest

from hodlrnd_gb300 import _lib

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """float32 -> BF16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def bf16_value(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("n,k", [(16, 16), (32, 32), (64, 16), (64, 64), (128, 48), (256, 128)])
def test_tc_product_matches_host(n, k):
    L = _lib.lib()
    rng = np.random.default_rng(n * 1000 + k)
    A = bf16_bits(rng.standard_normal((128, k)))
    B = bf16_bits(rng.standard_normal((n, k)))
    D = np.zeros((128, n), np.float32)
    _lib.check(L.hodlr_tc_selftest(A.ctypes.data, B.ctypes.data, n, k, D.ctypes.data))
    ref = bf16_value(A) @ bf16_value(B).T
    scale = np.abs(bf16_value(A)) @ np.abs(bf16_value(B)).T
    assert np.all(np.abs(D - ref) <= 1e-6 * scale + 1e-30)
