"""Pins the tcgen05 encodings the MLP kernels use (GPU): smem descriptors of
the canonical no-swizzle K-major and MN-major layouts, the kind::f16
(BF16 x BF16 -> FP32) instruction descriptor, and the TMEM placement of the
accumulator (M = 128: row m in lane m; M = 64: row m in lane
32 * (m // 16) + m % 16)."""

import pytest
import torch

pytestmark = pytest.mark.gpu

CASES = [(128, 64, 16, 0, 0), (128, 64, 64, 0, 0), (128, 16, 16, 0, 0), (128, 80, 128, 0, 0),
         (128, 128, 128, 0, 0), (128, 64, 64, 1, 0), (128, 64, 64, 0, 1), (128, 64, 128, 1, 1),
         (128, 80, 128, 1, 1), (64, 64, 128, 0, 0), (64, 80, 128, 1, 1), (64, 16, 32, 1, 0)]


@pytest.mark.parametrize("M,N,K,amn,bmn", CASES)
def test_tcgen05_bf16_gemm(cuda, M, N, K, amn, bmn):
    import tqf._lib as L
    g = torch.Generator(device=cuda).manual_seed(M * 1000 + N * 10 + K + amn * 7 + bmn * 3)
    A = torch.randn(M, K, device=cuda, generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device=cuda, generator=g).to(torch.bfloat16)
    out = torch.full((128, N), float("nan"), device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    L.call("tqf_tc_selftest", A.data_ptr(), B.data_ptr(), M, N, K, amn, bmn, out.data_ptr(), status.data_ptr(),
           L.stream_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    ref = A.float() @ B.float().T
    if M == 128:
        got = out
    else:
        lanes = torch.tensor([32 * (m // 16) + m % 16 for m in range(M)], device=cuda)
        got = out[lanes]
    torch.testing.assert_close(got, ref, rtol=1e-5, atol=1e-4)
