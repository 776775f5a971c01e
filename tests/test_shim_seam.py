"""The C++ drop-in, checked where the raw-native tree is present: the shim (ao_shim.cpp,
accel_shim.cpp) compiles against the reference's own headers, links with the reference's
scene, rasterizer and arena sources in place of ray_ao.cpp / ssao.cpp / reconcile.cpp /
accel.cpp, and the resulting program reaches librn_ao.so. Without a GPU it must fail the way
the reference fails without a device: "unverifiable", exit 4. No compute runs on the CPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle import oracle as _O

REF = _O.reference_dir() or ""
PKG = os.path.join(ROOT, "raw-native_gb300")
REF_SOURCES = ["src/renderer/raster.cpp", "src/scene/scene.cpp", "src/core/arena.cpp", "src/renderer/bvh.cpp"]

pytestmark = pytest.mark.skipif(not REF,
                                reason="the raw-native tree is not on this host")


def _cuda_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def seam_binary(tmp_path_factory):
    import rn_build
    rn_build.build_library()
    out = str(tmp_path_factory.mktemp("seam") / "raw_native_ao_seam")
    cmd = [shutil.which("g++") or "g++", "-std=c++23", "-O2", "-ffp-contract=off", "-I" + REF,
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(PKG, "host"), "-o", out,
           os.path.join(ROOT, "tests", "seam", "seam_main.cpp"), os.path.join(PKG, "host", "ao_shim.cpp"),
           os.path.join(PKG, "host", "accel_shim.cpp")] + [os.path.join(REF, s) for s in REF_SOURCES] + \
          ["-L" + PKG, "-lrn_ao", "-Wl,-rpath," + PKG, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def test_shim_links_against_the_reference(seam_binary):
    assert os.path.exists(seam_binary)


@pytest.mark.skipif(_cuda_present(), reason="a GPU is present: the no-device path is not reachable")
def test_seam_without_gpu_is_unverifiable(seam_binary):
    r = subprocess.run([seam_binary, "64", "64"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 4, (r.returncode, r.stdout, r.stderr)
    assert "unverifiable" in r.stdout and "RN_ERR" not in r.stdout
