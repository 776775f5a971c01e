"""The learned surrogate's network against a PyTorch FP32 restatement of it (test harness
only): same weights, same inputs; the loss and every parameter's gradient must agree to the
precision BF16 activations allow (cosine similarity > 0.995, norm within 5%). Then a short
training run must lower the loss."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def torch_unet(params, x):
    """The surrogate's network in plain PyTorch FP32 (NCHW), from rn_unet_get_params' layout."""
    import torch
    import torch.nn.functional as F
    import rn_ao
    ws, o = [], 0
    for cin, cout in rn_ao.UNET_CONVS:
        n = cout * 9 * cin
        w = params[o:o + n].view(cout, 3, 3, cin).permute(0, 3, 1, 2)
        o += n
        b = params[o:o + cout]
        o += cout
        ws.append((w, b))
    wh, bh = params[o:o + 32], params[o + 32:o + 33]

    def conv(t, k):
        return F.relu(F.conv2d(t, ws[k][0], ws[k][1], padding=1))
    e0 = conv(conv(x, 0), 1)
    e1 = conv(conv(F.avg_pool2d(e0, 2), 2), 3)
    e2 = conv(conv(F.avg_pool2d(e1, 2), 4), 5)
    b3 = conv(conv(F.avg_pool2d(e2, 2), 6), 7)
    up = lambda t: F.interpolate(t, scale_factor=2, mode="nearest")
    d2 = conv(conv(torch.cat([e2, up(b3)], 1), 8), 9)
    d1 = conv(conv(torch.cat([e1, up(d2)], 1), 10), 11)
    d0 = conv(conv(torch.cat([e0, up(d1)], 1), 12), 13)
    z = (d0 * wh.view(1, 32, 1, 1)).sum(1) + bh
    return torch.sigmoid(z)


def _batch(B, H, W, seed):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.rand(B, H, W, 5, device="cuda", generator=g)
    x[..., 1:4] = x[..., 1:4] * 2 - 1
    y = (0.3 + 0.6 * x[..., 4] + 0.1 * torch.rand(B, H, W, device="cuda", generator=g)).clamp(0, 1)
    return x.contiguous(), y.contiguous()


def test_unet_gradients_match_torch(rn):
    import torch
    B, H, W = 8, 32, 32
    net = rn.UNet(B, H, W, seed=3)
    x, y = _batch(B, H, W, 1)
    loss = net.train_step(x, y, lr=0.0)          # gradients only
    g_ours = torch.from_numpy(net.get_grads())
    p = torch.from_numpy(net.get_params()).requires_grad_(True)
    xin = torch.zeros(B, 8, H, W)
    xin[:, :5] = x.cpu().permute(0, 3, 1, 2)
    out = torch_unet(p, xin)
    ref_loss = ((out - y.cpu()) ** 2).mean()
    ref_loss.backward()
    assert abs(loss - ref_loss.item()) <= 0.02 * ref_loss.item()
    import rn_ao
    o = 0
    for cin, cout in rn_ao.UNET_CONVS + [(32, 1)]:
        n = cout * 9 * cin + cout if cin != 32 or cout != 1 else 33
        a, b = g_ours[o:o + n], p.grad[o:o + n]
        o += n
        cos = torch.nn.functional.cosine_similarity(a, b, dim=0).item()
        ratio = (a.norm() / b.norm()).item()
        assert cos > 0.995 and abs(ratio - 1) < 0.05, (cin, cout, cos, ratio)


def test_unet_training_lowers_loss(rn):
    B, H, W = 8, 32, 32
    net = rn.UNet(B, H, W, seed=5)
    x, y = _batch(B, H, W, 2)
    first = net.train_step(x, y, lr=1e-3)
    for _ in range(60):
        last = net.train_step(x, y, lr=1e-3)
    assert last < 0.5 * first
    out = net.forward(x)
    import torch
    torch.cuda.synchronize()
    assert float(((out - y) ** 2).mean()) < first


def test_unet_param_roundtrip_and_shapes(rn):
    net = rn.UNet(2, 64, 64, seed=1)
    p = net.get_params()
    assert p.size == net.param_count and np.isfinite(p).all()
    net.set_params(p * 0.5)
    assert np.allclose(net.get_params(), p * 0.5)
    with pytest.raises(rn.RnError):
        rn.UNet(1, 24, 32)                       # not a multiple of 16
