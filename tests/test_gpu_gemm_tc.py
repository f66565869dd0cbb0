"""The BF16 tensor-core GEMM (tcgen05) of the proposal network's inference
against an FP64 product of the same BF16-rounded operands: ragged M, N, K,
bias and ReLU in the epilogue, argument checks."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16(x):
    """round-to-nearest-even to BF16, as float32"""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("M,N,K,bias,relu", [(128, 128, 64, False, False), (300, 200, 100, True, True),
                                             (7, 500, 128, False, False), (1000, 256, 560, True, True),
                                             (129, 129, 4, False, False)])
def test_gemm_bf16_matches_fp64(gpulib, cuda, M, N, K, bias, relu):
    import torch
    rng = np.random.Generator(np.random.PCG64(M * 7 + N + K))
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    b = rng.standard_normal(N).astype(np.float32) if bias else None
    dA, dB = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    db = torch.from_numpy(b).to(cuda) if bias else None
    C = torch.full((M, N), float("nan"), device=cuda)
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    rc = gpulib.gpuisac_nn_gemm_bf16(M, N, K, ctypes.c_float(0.5), dA.data_ptr(), K, dB.data_ptr(), K,
                                     db.data_ptr() if bias else None, int(relu), C.data_ptr(), N, err.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    want = 0.5 * (bf16(A).astype(np.float64) @ bf16(B).astype(np.float64).T)
    if bias:
        want += b
    if relu:
        want = np.maximum(want, 0.0)
    got = C.cpu().numpy()
    assert np.isfinite(got).all()
    assert np.abs(got - want).max() <= 1e-4 * max(np.abs(want).max(), 1.0), np.abs(got - want).max()


def test_gemm_bf16_rejects_unaligned(gpulib, cuda):
    import torch
    x = torch.zeros(64, device=cuda)
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    assert gpulib.gpuisac_nn_gemm_bf16(4, 4, 6, ctypes.c_float(1.0), x.data_ptr(), 6, x.data_ptr(), 6, None, 0,
                                       x.data_ptr(), 4, err.data_ptr(), None) == 2
    assert gpulib.gpuisac_nn_gemm_bf16(4, 4, 0, ctypes.c_float(1.0), x.data_ptr(), 4, x.data_ptr(), 4, None, 0,
                                       x.data_ptr(), 4, err.data_ptr(), None) == 2
