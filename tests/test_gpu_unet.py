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


@pytest.mark.parametrize("B,H,W,explicit", [(8, 32, 32, True), (2, 128, 128, False)])
def test_unet_gradients_match_torch(rn, B, H, W, explicit):
    """32 x 32 runs on explicit im2col GEMMs (its deepest level cannot be tiled for the
    implicit convolution); 128 x 128 on the implicit-GEMM convolutions."""
    import torch
    net = rn.UNet(B, H, W, seed=3, explicit=explicit)
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
    norm, scale = net.last_grad_norm()                 # the library's global norm, unclipped
    assert abs(norm / p.grad.norm().item() - 1) < 0.05 and scale == 1.0
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


def test_unet_clipping_bounds_the_update(rn):
    """Clipping at ratio r limits the norm to r x the running mean of past clipped norms; the
    mean starts at the first norm, so the first step is scaled by r and the second (same
    batch, nearly the same weights) by r (0.99 + 0.01 r) n0 / n1."""
    B, H, W = 8, 32, 32
    net = rn.UNet(B, H, W, seed=7)
    x, y = _batch(B, H, W, 3)
    net.set_clip(0.5)
    net.train_step(x, y, lr=1e-7)
    n0, s0 = net.last_grad_norm()
    assert n0 > 0 and abs(s0 - 0.5) < 1e-6
    net.train_step(x, y, lr=1e-7)
    n1, s1 = net.last_grad_norm()
    assert abs(s1 - 0.5 * 0.995 * n0 / n1) < 1e-5
    net.set_clip(0.0)
    net.train_step(x, y, lr=1e-7)
    assert net.last_grad_norm()[1] == 1.0
    with pytest.raises(rn.RnError):
        net.set_clip(-1.0)


def test_unet_state_roundtrip_and_inference_mode(rn):
    import torch
    B, H, W = 8, 32, 32
    net = rn.UNet(B, H, W, seed=2)
    x, y = _batch(B, H, W, 4)
    for _ in range(3):
        net.train_step(x, y, lr=1e-3)
    state, step = net.get_state()
    assert step == 3 and state.size == 3 * net.param_count
    twin = rn.UNet(B, H, W, seed=99)
    twin.set_state(state, step)
    a, b = net.train_step(x, y, lr=1e-3), twin.train_step(x, y, lr=1e-3)
    # equal up to the order of floating-point atomics in the loss and head reductions
    assert abs(a - b) <= 1e-6 * abs(a)
    assert np.allclose(net.get_params(), twin.get_params(), rtol=1e-4, atol=1e-6)
    inf = rn.UNet(B, H, W, inference=True)
    inf.set_params(net.get_params())
    torch.testing.assert_close(inf.forward(x), net.forward(x), rtol=0, atol=0)
    with pytest.raises(rn.RnError):
        inf.train_step(x, y, lr=1e-3)


def test_unet_param_roundtrip_and_shapes(rn):
    net = rn.UNet(2, 64, 64, seed=1)
    p = net.get_params()
    assert p.size == net.param_count and np.isfinite(p).all()
    net.set_params(p * 0.5)
    assert np.allclose(net.get_params(), p * 0.5)
    with pytest.raises(rn.RnError):
        rn.UNet(1, 24, 32)                       # not a multiple of 16


def test_unet_implicit_and_explicit_convolutions_agree(rn):
    """The implicit-GEMM convolutions accumulate the same products in the same K order as the
    explicit im2col GEMMs: the forward is bit-identical, the gradients equal up to the order
    of the weight gradient's split-K atomics."""
    import torch
    B, H, W = 2, 128, 128
    imp = rn.UNet(B, H, W, seed=6)
    exp = rn.UNet(B, H, W, seed=6, explicit=True)
    x, y = _batch(B, H, W, 8)
    assert torch.equal(imp.forward(x), exp.forward(x))
    la, lb = imp.train_step(x, y, lr=0.0), exp.train_step(x, y, lr=0.0)
    assert abs(la - lb) <= 1e-6 * abs(la)
    ga, gb = imp.get_grads(), exp.get_grads()
    assert np.allclose(ga, gb, rtol=1e-3, atol=1e-6 * np.abs(gb).max())
    inf = rn.UNet(B, H, W, inference=True)
    inf.set_params(imp.get_params())
    assert torch.equal(inf.forward(x), imp.forward(x))


def test_unet_step_in_halves_and_data_parallel_average(rn):
    """rn_unet_backward + rn_unet_apply is rn_unet_train_step (up to the order of the loss and
    weight-gradient atomics); the flat gradient copy round-trips; and two data-parallel
    replicas that average their gradients (as the ranks' all-reduce does) take the same step
    bit for bit, with the gradient of the joint batch."""
    import torch
    import replicas
    B, H, W = 2, 128, 128
    a = rn.UNet(B, H, W, seed=8)
    b = rn.UNet(B, H, W, seed=8)
    x, y = _batch(B, H, W, 21)
    la = a.train_step(x, y, lr=1e-3)
    lb = b.backward(x, y)
    flat = torch.empty(b.grad_count, device="cuda")
    b.grads_to(flat)
    b.grads_from(flat)
    b.apply(1e-3)
    assert abs(la - lb) <= 1e-6 * abs(la)
    assert np.allclose(a.get_params(), b.get_params(), rtol=1e-4, atol=1e-6)
    # two replicas, one batch each, gradients averaged; a batch-4 network on both batches
    x1, y1 = _batch(B, H, W, 22)
    r0, r1 = rn.UNet(B, H, W, seed=9), rn.UNet(B, H, W, seed=9)
    both = rn.UNet(2 * B, H, W, seed=9)
    r0.backward(x, y)
    r1.backward(x1, y1)
    g0, g1 = torch.empty(r0.grad_count, device="cuda"), torch.empty(r1.grad_count, device="cuda")
    r0.grads_to(g0)
    r1.grads_to(g1)
    mean = (g0 + g1) / 2
    replicas.allreduce_mean_(mean, None)              # one rank: unchanged
    both.backward(torch.cat([x, x1]).contiguous(), torch.cat([y, y1]).contiguous())
    gb = torch.empty(both.grad_count, device="cuda")
    both.grads_to(gb)
    assert torch.allclose(mean, gb, rtol=1e-3, atol=1e-6 * gb.abs().max().item())
    r0.grads_from(mean)
    r1.grads_from(mean.clone())
    r0.apply(1e-3)
    r1.apply(1e-3)
    assert np.array_equal(r0.get_params(), r1.get_params())
