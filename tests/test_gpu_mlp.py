"""The 5th-generation tensor-core building block (tcgen05.mma, accumulators in
tensor memory): BF16 x BF16 -> FP32 products against an exact CPU product of
the same BF16 values."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    """round-to-nearest-even BF16 bit patterns of float32 values"""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


@pytest.mark.parametrize("N,K", [(16, 16), (128, 16), (128, 128), (16, 128), (256, 64), (64, 256)])
def test_tc_gemm(ctx, N, K):
    import torch
    import ocfd
    from ocfd._abi import declare
    declare("ocfd_tc_gemm_bf16", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_void_p])
    rng = np.random.default_rng(N * 1000 + K)
    A = to_bf16_bits(rng.standard_normal((128, K)))
    B = to_bf16_bits(rng.standard_normal((N, K)))
    want = bf16_value(A) @ bf16_value(B).T
    dA = torch.from_numpy(A.view(np.int16).copy()).cuda()
    dB = torch.from_numpy(B.view(np.int16).copy()).cuda()
    dC = torch.zeros((128, N), dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    ocfd.check(ocfd.load().ocfd_tc_gemm_bf16(ctx.h, dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), N, K, st),
               "ocfd_tc_gemm_bf16")
    got = dC.cpu().numpy().astype(np.float64)
    # FP32 accumulation of K exact BF16 products
    tol = 1e-6 * np.abs(bf16_value(A)) @ np.abs(bf16_value(B)).T + 1e-30
    assert (np.abs(got - want) <= 8 * tol).all(), np.abs(got - want).max()
