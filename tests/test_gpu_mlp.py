"""GPU: the tensor-core (tcgen05) building blocks of the radiance-cache MLP
against CPU products of the same bf16 operands."""
import ctypes

import numpy as np
import pytest

import mcrt_gb300 as M

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """Round-to-nearest-even float32 -> bf16 bit patterns."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("K,N", [(16, 16), (16, 64), (32, 48), (64, 64)])
@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_tensor_core_product(K, N, flags):
    rng = np.random.default_rng(K * 131 + N * 7 + flags)
    A = bf16_bits(rng.standard_normal((128, K)))
    B = bf16_bits(rng.standard_normal((N, K)))
    D = np.zeros((128, N), np.float32)
    L = M.lib()
    M.check(L.mcrt_mlp_gemm_probe(0, A.ctypes.data_as(ctypes.c_void_p), B.ctypes.data_as(ctypes.c_void_p), K, N,
                                  flags, D.ctypes.data_as(ctypes.c_void_p)))
    want = bf16_value(A).astype(np.float64) @ bf16_value(B).astype(np.float64).T
    err = np.abs(D - want).max()
    assert err <= 1e-4 * max(1.0, np.abs(want).max()), (err, D[:2, :4], want[:2, :4])
