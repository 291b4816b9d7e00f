"""The tcgen05 BF16 GEMM (tensor memory accumulator) the surrogate MLP uses,
against an FP64 product of the same BF16 values."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def _bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("M,K", [(128, 16), (128, 256), (512, 256), (256, 64), (128, 768)])
def test_tc_gemm_matches_fp64(M, K):
    from bldfm_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(M + K)
    A = _bf16_bits(rng.standard_normal((M, K)))
    B = _bf16_bits(rng.standard_normal((256, K)))
    D = np.zeros((M, 256), dtype=np.float32)
    st = lib.bldfm_tc_gemm_check(_lib.ptr(A), _lib.ptr(B), _lib.ptr(D), M, K)
    _lib.check(st, "tc_gemm_check")
    ref = _bf16_value(A) @ _bf16_value(B).T
    err = np.abs(D - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err
