"""The C++ drop-in, checked where the raw-native tree is present: the shim (ao_shim.cpp,
accel_shim.cpp) compiles against the reference's own headers, links with the reference's
scene, rasterizer and arena sources in place of ray_ao.cpp / ssao.cpp / reconcile.cpp /
accel.cpp, and the resulting program reaches librn_ao.so. Without a GPU it must fail the way
the reference fails without a device: "unverifiable", exit 4. No compute runs on the CPU.

The `--gpu` seam: gpu_shim.cpp (raw::gpuInit / raw::renderGpu) in place of
src/renderer/gpu/gpu_renderer.cpp, linked with the reference's own src/tools/gpu_run.cpp,
gpu_reconcile.cpp, its CLI parser, frame graph, writers and certificates, under the CLI's
GPU branch; without a GPU it exits 4 and writes the "unverifiable" GPU certificate with the
library's reason, as the reference does on its null backend."""
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


# The reference sources the `--gpu` branch needs besides the shims (the link's closure):
# gpu_run.cpp, the CPU reference frame it renders beside the GPU's, the writers, the
# certificates and receipts, the CLI parser and the scenes it can load.
GPU_SEAM_SOURCES = [
    "src/assets/gltf.cpp", "src/assets/json.cpp", "src/cert/certificate.cpp", "src/cert/certificate_from.cpp",
    "src/core/arena.cpp", "src/core/image.cpp", "src/core/sha256.cpp", "src/core/version.cpp",
    "src/graph/frame_graph.cpp", "src/renderer/composite.cpp", "src/renderer/gpu_reconcile.cpp",
    "src/renderer/motion.cpp", "src/renderer/raster.cpp", "src/renderer/render.cpp", "src/scene/scene.cpp",
    "src/tools/channels_json.cpp", "src/tools/cli_params.cpp", "src/tools/gpu_run.cpp",
    "src/tools/model_manifest.cpp", "src/tools/model_scene.cpp", "src/tools/owned_build.cpp",
    "src/tools/owned_export.cpp", "src/tools/owned_hall.cpp", "src/tools/receipt.cpp", "src/tools/run.cpp"]


@pytest.fixture(scope="module")
def gpu_seam_binary(tmp_path_factory):
    import concurrent.futures as cf
    import rn_build
    rn_build.build_library()
    d = tmp_path_factory.mktemp("gpuseam")
    cxx = shutil.which("g++") or "g++"
    inc = ["-I" + REF, "-I" + os.path.join(REF, "third_party", "superstack"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(PKG, "host")]
    srcs = [os.path.join(REF, s) for s in GPU_SEAM_SOURCES] + [
        os.path.join(ROOT, "tests", "seam", "gpu_seam_main.cpp"), os.path.join(PKG, "host", "gpu_shim.cpp"),
        os.path.join(PKG, "host", "ao_shim.cpp"), os.path.join(PKG, "host", "accel_shim.cpp")]

    def compile_one(src):
        obj = str(d / (os.path.basename(os.path.dirname(src)) + "_" + os.path.basename(src) + ".o"))
        r = subprocess.run([cxx, "-std=c++23", "-O1", "-w", "-ffp-contract=off"] + inc + ["-c", src, "-o", obj],
                           capture_output=True, text=True)
        assert r.returncode == 0, (src, r.stderr[-3000:])
        return obj

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs))
    out = str(d / "raw_native_gpu_seam")
    r = subprocess.run([cxx, "-o", out] + objs + ["-L" + PKG, "-lrn_ao", "-Wl,-rpath," + PKG, "-lpthread"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def test_gpu_shim_links_with_the_reference_gpu_run(gpu_seam_binary):
    assert os.path.exists(gpu_seam_binary)


@pytest.mark.skipif(_cuda_present(), reason="a GPU is present: the no-device path is not reachable")
def test_gpu_seam_without_gpu_is_unverifiable(gpu_seam_binary, tmp_path):
    import json
    out = str(tmp_path / "run")
    r = subprocess.run([gpu_seam_binary, "--out", out, "--width", "64", "--height", "48"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 4, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith("gpu: ") and "gpu-certificate:" in r.stdout
    cert = json.load(open(os.path.join(out, "gpu_certificate.json")))
    text = json.dumps(cert)
    assert "unverifiable" in text and "cuda" in text


def test_shim_links_against_the_reference(seam_binary):
    assert os.path.exists(seam_binary)


@pytest.mark.skipif(_cuda_present(), reason="a GPU is present: the no-device path is not reachable")
def test_seam_without_gpu_is_unverifiable(seam_binary):
    r = subprocess.run([seam_binary, "64", "64"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 4, (r.returncode, r.stdout, r.stderr)
    assert "unverifiable" in r.stdout and "RN_ERR" not in r.stdout
