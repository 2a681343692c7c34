"""The tensor-core GEMM (tcgen05.mma, bf16 operands in 128B-swizzled shared
memory, FP32 accumulator in tensor memory) against a plain FP32 product of the
same bf16 values."""
import numpy as np
import pytest

from multislice_gb300 import _abi

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    """Round-to-nearest-even bf16 bit patterns of float32 values."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def _bf16_value(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("M,N,K", [(128, 16, 64), (128, 64, 128), (256, 128, 192), (384, 256, 64),
                                   (128, 48, 320)])
def test_tc_gemm_matches_fp32_product(ctx, M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = _bf16_bits(rng.standard_normal((M, K)))
    B = _bf16_bits(rng.standard_normal((N, K)))
    D = np.zeros((M, N), np.float32)
    ctx._check(ctx._lib.msl_tc_gemm_bf16(ctx._h, A.ctypes.data, B.ctypes.data, D.ctypes.data, M, N, K))
    ref = _bf16_value(A).astype(np.float64) @ _bf16_value(B).astype(np.float64).T
    assert np.abs(D - ref).max() <= 1e-4 * np.abs(ref).max()


def test_tc_gemm_rejects_bad_shapes(ctx):
    A = np.zeros((100, 64), np.uint16)
    B = np.zeros((16, 64), np.uint16)
    D = np.zeros((100, 16), np.float32)
    rc = ctx._lib.msl_tc_gemm_bf16(ctx._h, A.ctypes.data, B.ctypes.data, D.ctypes.data, 100, 16, 64)
    assert rc == _abi.MSL_E_ARG
