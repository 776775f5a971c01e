"""The C ABI from plain C: tests/seam/c_abi_example.c compiles as strict C99 against
include/rn_ao.h, links with librn_ao.so, and without a GPU stops at rn_init with
RN_ERR_NO_DEVICE (exit 3, "unverifiable"), as the reference does without a device."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "raw-native_gb300")


def _cuda_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def example(tmp_path_factory):
    import rn_build
    rn_build.build_library()
    cc = shutil.which("gcc") or shutil.which("cc")
    out = str(tmp_path_factory.mktemp("cabi") / "ao_example")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "seam", "c_abi_example.c"), "-L" + PKG, "-lrn_ao",
                        "-Wl,-rpath," + PKG, "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.mark.skipif(_cuda_present(), reason="checks the behaviour without a GPU")
def test_c_caller_without_a_device(example):
    r = subprocess.run([example], capture_output=True, text=True, timeout=120)
    assert r.returncode == 3, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith("unverifiable")


@pytest.mark.gpu
def test_c_caller_frame_on_the_gpu(example):
    """The same C99 binary on a GPU: exit 0 and the frame's reconcile equal to the oracle's
    (pixels 4096; rmse, max error and verdict as printed; the lowest traced AO)."""
    import numpy as np
    from oracle import oracle as O
    r = subprocess.run([example], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    w = h = 64
    tris = np.array([-1, 0, -1, 1, 0, -1, 1, 0, 1, -1, 0, -1, 1, 0, 1, -1, 0, 1,
                     0.5, 0, -1, 0.5, 1, -1, 0.5, 1, 1, 0.5, 0, -1, 0.5, 1, 1, 0.5, 0, 1], np.float32).reshape(4, 9)
    xs = np.float32(-1.0) + (np.float32(2.0) * (np.arange(w, dtype=np.float32) + np.float32(0.5))) / np.float32(w)
    pos = np.zeros((h, w, 3), np.float32)
    pos[:, :, 0] = xs[None, :]
    pos[:, :, 2] = xs[:, None]
    nrm = np.zeros_like(pos)
    nrm[:, :, 1] = 1.0
    mask = np.ones((h, w), np.uint8)
    ao, _, _ = O.trace(pos, nrm, mask, tris, 16, 0.5, to_light=np.array([0, 1, 0], np.float32))
    ss = O.ssao(pos, nrm, mask, 24, 0.5)
    _, st = O.reconcile(ss, ao, mask, 0.12)
    want = "pixels %d rmse %.6f max_error %.6f verdict %s; lowest ray-traced AO %.4f" % (
        st["pixels"], st["rmse"], st["maxError"], "verified" if st["within"] else "refuted", float(ao.min()))
    assert st["pixels"] == 4096
    assert r.stdout.strip() == want, (r.stdout, want)
