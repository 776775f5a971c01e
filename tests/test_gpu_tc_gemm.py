"""The surrogate's tcgen05 GEMM against torch's matmul of the same BF16 values (FP32
accumulation both ways; tolerance 1e-3 relative to the row's magnitude for FP32 output,
one BF16 rounding for BF16 output)."""
import pytest

pytestmark = pytest.mark.gpu

CASES = [(128, 32, 64, 1), (256, 64, 256, 1), (512, 128, 1152, 1), (1024, 256, 2304, 1), (384, 32, 320, 1),
         (256, 384, 3456, 1), (128, 128, 4096, 8)]


@pytest.mark.parametrize("M,N,K,splits", CASES)
def test_tc_gemm_matches_torch(rn, M, N, K, splits):
    import torch
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    P = (torch.randn(M, K, device="cuda", generator=g) * 0.5).to(torch.bfloat16)
    Q = (torch.randn(N, K, device="cuda", generator=g) * 0.5).to(torch.bfloat16)
    ref = P.float() @ Q.float().T
    got = rn.tc_gemm(P, Q, splits=splits)
    torch.cuda.synchronize()
    rn.synchronize()
    scale = ref.abs().amax(dim=1, keepdim=True) + 1.0
    assert ((got - ref).abs() / scale).max().item() < 1e-3


def test_tc_gemm_bf16_bias_relu(rn):
    import torch
    M, N, K = 256, 64, 576
    P = torch.randn(M, K, device="cuda").to(torch.bfloat16)
    Q = torch.randn(N, K, device="cuda").to(torch.bfloat16)
    b = torch.randn(N, device="cuda")
    ref = torch.relu(P.float() @ Q.float().T + b)
    got = rn.tc_gemm(P, Q, out_dtype=torch.bfloat16, bias=b, relu=True)
    torch.cuda.synchronize()
    assert torch.allclose(got.float(), ref.to(torch.bfloat16).float(), rtol=1e-2, atol=1e-2)


def test_tc_gemm_rejects_unsupported_shapes(rn):
    import torch
    P = torch.zeros(128, 64, device="cuda", dtype=torch.bfloat16)
    with pytest.raises(rn.RnError):
        rn.tc_gemm(P, torch.zeros(96, 64, device="cuda", dtype=torch.bfloat16))     # N 96
    with pytest.raises(rn.RnError):
        rn.tc_gemm(torch.zeros(100, 64, device="cuda", dtype=torch.bfloat16), P[:32])   # M not a multiple of 128
