"""Host-side logic of the learned surrogate, on the CPU: the padded network shape, the
learning-rate schedule, the training scenes' densities, the confidence-band tile test, the
BF16 weight files and the RMSE."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_padded_shape():
    import surrogate as S
    assert S.padded_shape(2160, 3840) == (2176, 3840)
    for h, w in ((1080, 1920), (224, 384), (37, 101), (2160, 3840), (128, 128)):
        H, W = S.padded_shape(h, w)
        assert H >= h and W >= w and H % 16 == 0 and W % 16 == 0
        assert ((H // 8) * (W // 8)) % 128 == 0
        assert W - w < 16                                     # the width is only rounded up
        # the smallest such height (an awkward width can need a tall pad: 37 x 101 -> 512 x 112)
        assert H - 16 < h or (((H - 16) // 8) * (W // 8)) % 128 != 0


def test_lr_schedule():
    import surrogate as S
    peak, total = 1e-3, 1000
    assert S.lr_at(0, total, peak) == pytest.approx(peak / 100)
    assert S.lr_at(99, total, peak) == pytest.approx(peak)
    assert S.lr_at(100, total, peak) == pytest.approx(peak)
    assert S.lr_at(total, total, peak) == pytest.approx(0.0, abs=1e-12)
    after = [S.lr_at(s, total, peak) for s in range(100, total + 1, 50)]
    assert all(a >= b for a, b in zip(after, after[1:]))
    assert S.lr_at(550, total, peak) == pytest.approx(peak / 2)


def test_scene_densities():
    import surrogate as S
    assert S.scene_counts(5, "fixed") == (200, 50)
    draws = [S.scene_counts(s, "mixed") for s in range(1000, 1400)]
    assert draws == [S.scene_counts(s, "mixed") for s in range(1000, 1400)]      # seeded
    b = np.array([d[0] for d in draws])
    s = np.array([d[1] for d in draws])
    assert b.min() >= 200 and b.max() <= 10000 and s.min() >= 50 and s.max() <= 6000
    # log-uniform: the median near the geometric mean of the range
    assert abs(np.log(np.median(b)) - np.log(np.sqrt(200 * 10000))) < 0.4
    assert abs(np.log(np.median(s)) - np.log(np.sqrt(50 * 6000))) < 0.4
    with pytest.raises(ValueError):
        S.scene_counts(1, "dense")


def test_band_test_flags_only_tiles_outside_the_band():
    import torch
    import surrogate as S
    h, w = 40, 24                                       # 3 x 2 tiles, the last row and column ragged
    g = torch.Generator().manual_seed(3)
    ao4 = (torch.randint(0, 5, (h, w), generator=g).float() / 4)
    mask = torch.ones(h, w, dtype=torch.uint8)
    mask[32:, 16:] = 0                                  # one tile without coverage
    pred = ao4.clone()
    tiles = S.fallback_tiles(pred, ao4, mask, 4, 3.0)
    assert tiles.shape == (3, 2) and not bool(tiles.any())
    pred[:16, :16] = (ao4[:16, :16] + 0.5).clamp(max=1.0)   # far outside the band
    pred[16:32, 16:] += 0.002                           # well inside it
    pred[32:, 16:] = 0.0                                # uncovered: never flagged
    tiles = S.fallback_tiles(pred, ao4, mask, 4, 3.0)
    assert tiles.tolist() == [[True, False], [False, False], [False, False]]
    px = S.tiles_to_pixels(tiles, h, w)
    assert px.shape == (h, w) and int(px.sum()) == 256
    # a tile of constant 4-spp AO still has a floor on its band: 0.5 / sqrt(4 n)
    flat = torch.ones(h, w)
    tiles = S.fallback_tiles(flat - 0.01, flat, mask, 4, 3.0)
    assert not bool(tiles.any())


class _FakeNet:
    def __init__(self, n):
        self.p = np.random.default_rng(0).normal(0, 0.05, n).astype(np.float32)
        self.loaded = None

    def get_params(self):
        return self.p.copy()

    def set_params(self, p):
        self.loaded = np.asarray(p, np.float32).copy()


def test_bf16_weight_files(tmp_path):
    import rn_ao
    import surrogate as S
    n = sum(co * 9 * ci + co for ci, co in rn_ao.UNET_CONVS) + 33
    net = _FakeNet(n)
    S.save_weights(net, str(tmp_path / "w.npz"), {"steps": 7})
    meta = S.load_weights(net, str(tmp_path / "w.npz"))
    assert meta == {"steps": 7}
    # round to nearest even in BF16: the error is at most half a BF16 unit, ties go even
    a, b = net.p, net.loaded
    ulp = np.abs(a).view(np.uint32) & 0x7F800000
    half = (ulp.view(np.float32) * np.float32(2.0 ** -8))
    assert np.all(np.abs(a - b) <= half) and np.all((b.view(np.uint32) & 0xFFFF) == 0)
    tie = np.array([1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8], np.float32)      # halfway cases
    net2 = _FakeNet(2)
    net2.p = tie
    S.save_weights(net2, str(tmp_path / "t.npz"), {})
    S.load_weights(net2, str(tmp_path / "t.npz"))
    assert net2.loaded.tolist() == [1.0, 1.0 + 4 * 2.0 ** -8]
    # the committed weights hold the whole network
    for f in ("surrogate_bf16.npz", "surrogate_mixed_bf16.npz"):
        path = os.path.join(ROOT, "raw-native_gb300", "weights", f)
        net3 = _FakeNet(1)
        S.load_weights(net3, path)
        assert net3.loaded.size == n and np.isfinite(net3.loaded).all()


def test_rmse_over_covered_pixels():
    import torch
    import surrogate as S
    a = torch.tensor([[0.0, 1.0], [0.5, 0.25]])
    b = torch.tensor([[0.0, 0.0], [0.5, 0.75]])
    m = torch.tensor([[1, 0], [1, 1]], dtype=torch.uint8)
    assert S.rmse(a, b, m) == pytest.approx(np.sqrt(0.25 / 3))
    assert S.rmse(a, b, torch.zeros(2, 2, dtype=torch.uint8)) == 0.0
