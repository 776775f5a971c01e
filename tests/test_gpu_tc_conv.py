"""The implicit-GEMM 3x3 convolution against PyTorch's FP32 conv2d on the same BF16-rounded
operands (test harness only): FP32 accumulation of BF16 products, so the results agree to
FP32 rounding of the sums (relative 1e-3 of the output scale)."""
import pytest

pytestmark = pytest.mark.gpu

# (B, H, W, c0, c1, N): single and concatenated sources, 32- and 64-channel blocks, every
# tile shape (W = 128, 64, 32, 16, and a wide frame), N from 32 to 384
CASES = [
    (2, 16, 128, 32, 0, 32),
    (1, 32, 64, 64, 0, 64),
    (3, 16, 32, 128, 0, 128),
    (4, 16, 16, 256, 0, 256),
    (1, 8, 1920, 32, 64, 32),
    (2, 32, 32, 64, 128, 64),
    (2, 24, 256, 16, 0, 32),             # 16 input channels: the row-ring kernel only
    (1, 8, 128, 16, 0, 64),
    (1, 16, 16, 128, 256, 128),
    (1, 16, 64, 64, 0, 384),
    (2, 24, 48, 96, 0, 64),
]


def _ref(x0, x1, w, bias, relu):
    import torch
    import torch.nn.functional as F
    x = x0 if x1 is None else torch.cat([x0, x1], 3)
    B, H, W, Cin = x.shape
    N = w.shape[0]
    k = w[:, :9 * Cin].float().view(N, 3, 3, Cin).permute(0, 3, 1, 2)
    y = F.conv2d(x.float().permute(0, 3, 1, 2), k, bias, padding=1).permute(0, 2, 3, 1)
    return F.relu(y) if relu else y


@pytest.mark.parametrize("B,H,W,c0,c1,N", CASES)
def test_conv_matches_torch(rn, B, H, W, c0, c1, N):
    import torch
    g = torch.Generator(device="cuda").manual_seed(B * 1000 + H + W + c0 + c1 + N)
    x0 = torch.randn(B, H, W, c0, device="cuda", generator=g).to(torch.bfloat16)
    x1 = torch.randn(B, H, W, c1, device="cuda", generator=g).to(torch.bfloat16) if c1 else None
    cin = c0 + c1
    ldw = (9 * cin + 127) // 128 * 128
    w = torch.zeros(N, ldw, device="cuda", dtype=torch.bfloat16)
    w[:, :9 * cin] = (torch.randn(N, 9 * cin, device="cuda", generator=g) / (9 * cin) ** 0.5).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    out = rn.tc_conv3x3(x0, w, x1, bias=bias, relu=True)
    torch.cuda.synchronize()
    ref = _ref(x0, x1, w, bias, True)
    scale = ref.abs().max().item()
    err = (out - ref).abs().max().item()
    assert err <= 1e-3 * scale, (err, scale)


def test_conv_bf16_output_and_upsampled_copy(rn):
    import torch
    g = torch.Generator(device="cuda").manual_seed(9)
    x0 = torch.randn(2, 16, 32, 64, device="cuda", generator=g).to(torch.bfloat16)
    w = (torch.randn(128, 640, device="cuda", generator=g) / 24).to(torch.bfloat16)
    w[:, 576:] = 0
    out, up = rn.tc_conv3x3(x0, w, upsampled=True)
    torch.cuda.synchronize()
    ref = _ref(x0, None, w, None, False).to(torch.bfloat16)
    assert (out.float() - ref.float()).abs().max().item() <= 0.02 * ref.float().abs().max().item()
    want = out.repeat_interleave(2, 1).repeat_interleave(2, 2)
    assert torch.equal(up, want)


def test_conv_rejects_untileable_and_bad_channels(rn):
    import torch
    x = torch.zeros(1, 10, 24, 32, device="cuda", dtype=torch.bfloat16)      # W 24: TW 8, 16 rows > 10
    w = torch.zeros(32, 384, device="cuda", dtype=torch.bfloat16)
    with pytest.raises(rn.RnError):
        rn.tc_conv3x3(x, w)
    y = torch.zeros(1, 16, 16, 40, device="cuda", dtype=torch.bfloat16)       # 40 channels
    with pytest.raises(rn.RnError):
        rn.tc_conv3x3(y, torch.zeros(32, 384, device="cuda", dtype=torch.bfloat16))
    z = torch.zeros(1, 16, 64, 16, device="cuda", dtype=torch.bfloat16)       # 16 channels, 64-pixel rows
    with pytest.raises(rn.RnError):
        rn.tc_conv3x3(z, torch.zeros(32, 256, device="cuda", dtype=torch.bfloat16))


@pytest.mark.parametrize("B,H,W,c0,c1,N", [(2, 8, 128, 32, 0, 32), (1, 6, 256, 32, 0, 64), (1, 4, 1920, 32, 0, 32),
                                            (2, 8, 128, 32, 64, 32), (1, 5, 384, 64, 0, 64),
                                            # several row chunks per strip, a ragged last chunk
                                            (1, 37, 256, 32, 0, 32), (2, 70, 128, 32, 64, 32),
                                            (1, 333, 1920, 32, 0, 64)])
def test_conv_halo_tiles_match_the_general_kernel(rn, B, H, W, c0, c1, N):
    """Row tiles read from a ring of one-row boxes (conv_halo 1) accumulate the same K16 steps
    in the same order as the per-tap boxes (conv_halo 0): identical outputs, bias, ReLU and
    the upsampled copy included."""
    import torch
    saved = rn.tune_get("conv_halo")
    try:
        g = torch.Generator(device="cuda").manual_seed(B + H + W + c0 + c1 + N)
        x0 = torch.randn(B, H, W, c0, device="cuda", generator=g).to(torch.bfloat16)
        x1 = torch.randn(B, H, W, c1, device="cuda", generator=g).to(torch.bfloat16) if c1 else None
        cin = c0 + c1
        ldw = (9 * cin + 127) // 128 * 128
        w = torch.zeros(N, ldw, device="cuda", dtype=torch.bfloat16)
        w[:, :9 * cin] = (torch.randn(N, 9 * cin, device="cuda", generator=g) / (9 * cin) ** 0.5).to(torch.bfloat16)
        bias = torch.randn(N, device="cuda", generator=g)
        outs = []
        for halo in (0, 1):
            rn.tune_set("conv_halo", halo)
            o, u = rn.tc_conv3x3(x0, w, x1, bias=bias, relu=True, upsampled=True)
            f = rn.tc_conv3x3(x0, w, x1, bias=bias, relu=False)
            torch.cuda.synchronize()
            outs.append((o.clone(), u.clone(), f.clone()))
        for a, b in zip(*outs):
            assert torch.equal(a, b)
        ref = _ref(x0, x1, w, bias, False)
        assert (outs[1][2] - ref).abs().max().item() <= 1e-3 * ref.abs().max().item()
    finally:
        rn.tune_set("conv_halo", saved)


@pytest.mark.parametrize("B,H,W,c0,c1,N", [(2, 8, 128, 32, 0, 32), (1, 6, 256, 32, 0, 64), (1, 4, 1920, 16, 0, 32),
                                            (2, 8, 128, 32, 32, 32), (1, 5, 384, 64, 0, 64), (1, 1, 128, 32, 0, 32),
                                            (1, 2, 128, 16, 0, 64), (1, 37, 256, 32, 0, 32), (2, 70, 128, 32, 64, 32),
                                            (1, 333, 1920, 32, 0, 64), (3, 19, 640, 32, 16, 64),
                                            # output channels in slices of 32 (the weights of a
                                            # 64-wide slice do not fit; N beyond 64)
                                            (1, 8, 128, 128, 64, 64), (1, 37, 384, 128, 64, 64),
                                            (1, 6, 256, 64, 0, 128), (2, 9, 128, 32, 32, 256)])
def test_conv_fan_matches_row_by_row(rn, B, H, W, c0, c1, N):
    """Fan-out MMAs (conv_fan 1: one MMA of N = 3 x BN per input row, shift and channel step,
    feeding the three output rows that read the row) against the row-by-row MMAs (conv_fan 0):
    identical FP32 and BF16 outputs, bias, ReLU and the upsampled copy included, on frames of
    1 to 333 rows (items of 1 to 16 rows: the accumulator ring wraps inside an MMA). Shapes the
    row-by-row form cannot take (weights too large, N beyond 64) compare with the per-tap
    kernel, whose K steps run in the same order (tap, then channel)."""
    import torch
    saved = (rn.tune_get("conv_fan"), rn.tune_get("conv_halo"))
    try:
        rn.tune_set("conv_halo", 1)
        g = torch.Generator(device="cuda").manual_seed(7 * B + H + W + c0 + c1 + N)
        x0 = torch.randn(B, H, W, c0, device="cuda", generator=g).to(torch.bfloat16)
        x1 = torch.randn(B, H, W, c1, device="cuda", generator=g).to(torch.bfloat16) if c1 else None
        cin = c0 + c1
        ldw = (9 * cin + 127) // 128 * 128
        w = torch.zeros(N, ldw, device="cuda", dtype=torch.bfloat16)
        w[:, :9 * cin] = (torch.randn(N, 9 * cin, device="cuda", generator=g) / (9 * cin) ** 0.5).to(torch.bfloat16)
        bias = torch.randn(N, device="cuda", generator=g)
        outs = []
        for fan in (0, 1):
            rn.tune_set("conv_fan", fan)
            o, u = rn.tc_conv3x3(x0, w, x1, bias=bias, relu=True, upsampled=True)
            f = rn.tc_conv3x3(x0, w, x1, bias=bias, relu=False)
            torch.cuda.synchronize()
            outs.append((o.clone(), u.clone(), f.clone()))
        for a, b in zip(*outs):
            assert torch.equal(a, b), int((a != b).sum().item())
        ref = _ref(x0, x1, w, bias, False)
        assert (outs[1][2] - ref).abs().max().item() <= 1e-3 * ref.abs().max().item()
    finally:
        rn.tune_set("conv_fan", saved[0])
        rn.tune_set("conv_halo", saved[1])


@pytest.mark.parametrize("B,H,W,c0,c1,N", [(1, 8, 128, 32, 0, 64), (2, 21, 256, 64, 0, 64), (1, 5, 384, 32, 32, 64)])
def test_conv_fan_slices_of_32_match(rn, B, H, W, c0, c1, N):
    """64-channel layers as two 32-channel slices (conv_fan_bn 32: each CTA reloads the weights
    when its items cross into the next slice) give the 64-wide fan-out's outputs bit for bit."""
    import torch
    saved = (rn.tune_get("conv_fan"), rn.tune_get("conv_fan_bn"))
    try:
        rn.tune_set("conv_fan", 1)
        g = torch.Generator(device="cuda").manual_seed(11 * B + H + W + c0 + c1 + N)
        x0 = torch.randn(B, H, W, c0, device="cuda", generator=g).to(torch.bfloat16)
        x1 = torch.randn(B, H, W, c1, device="cuda", generator=g).to(torch.bfloat16) if c1 else None
        cin = c0 + c1
        ldw = (9 * cin + 127) // 128 * 128
        w = torch.zeros(N, ldw, device="cuda", dtype=torch.bfloat16)
        w[:, :9 * cin] = (torch.randn(N, 9 * cin, device="cuda", generator=g) / (9 * cin) ** 0.5).to(torch.bfloat16)
        bias = torch.randn(N, device="cuda", generator=g)
        outs = []
        for bn in (64, 32):
            rn.tune_set("conv_fan_bn", bn)
            o, u = rn.tc_conv3x3(x0, w, x1, bias=bias, relu=True, upsampled=True)
            f = rn.tc_conv3x3(x0, w, x1, bias=bias, relu=False)
            torch.cuda.synchronize()
            outs.append((o.clone(), u.clone(), f.clone()))
        for a, b in zip(*outs):
            assert torch.equal(a, b), int((a != b).sum().item())
    finally:
        rn.tune_set("conv_fan", saved[0])
        rn.tune_set("conv_fan_bn", saved[1])
