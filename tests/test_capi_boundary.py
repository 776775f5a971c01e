"""The drop-in boundary, checked without a GPU: librn_ao.so loads, exports every symbol
include/rn_ao.h declares, and fails loudly (RN_ERR_NO_DEVICE, never a CPU answer) when no
device is present."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rn_ao.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void)\s+(rn_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    import rn_ao
    if not os.path.exists(rn_ao.LIB_PATH):
        import rn_build
        rn_build.build_library()
    return rn_ao.lib()


def test_header_declares_the_exports():
    import rn_ao
    assert declared_symbols() == sorted(rn_ao.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.rn_ao_version() == 1


def _cuda_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_cuda_present(), reason="a GPU is present; the no-device path is not reachable")
def test_no_device_fails_loudly(lib):
    import rn_ao
    with pytest.raises(rn_ao.RnError) as e:
        rn_ao.init()
    assert e.value.code == 2
    a = np.zeros((2, 2), np.float32)
    m = np.ones((2, 2), np.uint8)
    with pytest.raises(rn_ao.RnError) as e:
        rn_ao.reconcile(a, a, m, 0.1)
    assert e.value.code == 2
    g = rn_ao.GBuffer(np.zeros((2, 2, 3), np.float32), np.zeros((2, 2, 3), np.float32), m)
    with pytest.raises(rn_ao.RnError):
        rn_ao.compute_ssao(g, 24, 2.0)
    st = rn_ao.Status()
    eye = (C.c_float * 3)(0, 0, 0)
    assert lib.rn_hybrid(None, None, None, eye, eye, 0, None, None, None, C.byref(st)) == 2


def test_argument_errors_before_any_device_work(lib):
    import rn_ao
    st = rn_ao.Status()
    # null arguments are rejected before the device is touched
    assert lib.rn_reconcile(None, None, None, 1, 1, C.c_float(0.1), 0, None, None, C.byref(st)) == 1
    assert b"null" in st.message
    assert lib.rn_accel_build(None, 5, 0, C.byref(C.c_void_p()), C.byref(st)) == 1
    assert lib.rn_ploc_build(None, 3, 16, 0, None, None, None, C.byref(st)) == 1
    assert lib.rn_closest(None, None, None, 4, 0, None, None, C.byref(st)) == 1


def test_host_and_device_arrays_do_not_mix():
    import rn_ao

    class FakeCuda:
        is_cuda = True
    with pytest.raises(rn_ao.RnError):
        rn_ao._Args(np.zeros(3, np.float32), FakeCuda())


def test_tuning_keys_without_a_device(lib, tmp_path, monkeypatch):
    """The launch-shape keys are host state: set, read back, loaded from a file (all or
    nothing), and refused with RN_ERR_INVALID for an unknown key or value."""
    import rn_ao
    saved = rn_ao.tune_all()
    try:
        assert set(saved) == set(rn_ao.TUNE_KEYS)
        for k, values in rn_ao.TUNE_KEYS.items():
            for v in values:
                rn_ao.tune_set(k, v)
                assert rn_ao.tune_get(k) == v
        with pytest.raises(rn_ao.RnError) as e:
            rn_ao.tune_set("trace_packet", 5)
        assert e.value.code == 1
        with pytest.raises(rn_ao.RnError):
            rn_ao.tune_set("no_such_key", 1)
        rn_ao.tune_set("trace_packet", 8)
        good = tmp_path / "good.txt"
        good.write_text("# picked\ntrace_packet = 16\n\nssao_tile_h=4   # comment\n")
        rn_ao.tune_load(str(good))
        assert rn_ao.tune_get("trace_packet") == 16 and rn_ao.tune_get("ssao_tile_h") == 4
        bad = tmp_path / "bad.txt"
        bad.write_text("trace_packet = 4\nconv_bn_max = 7\n")
        with pytest.raises(rn_ao.RnError):
            rn_ao.tune_load(str(bad))
        assert rn_ao.tune_get("trace_packet") == 16          # nothing of the bad file applied
        unknown = tmp_path / "unknown.txt"
        unknown.write_text("trace_packet = 4\nwarp_size = 64\n")
        with pytest.raises(rn_ao.RnError) as e:
            rn_ao.tune_load(str(unknown))
        assert "warp_size" in str(e.value)
        assert rn_ao.tune_get("trace_packet") == 16
        with pytest.raises(rn_ao.RnError):
            rn_ao.tune_load(str(tmp_path / "missing.txt"))
        # an environment variable keeps its key out of the file's reach
        monkeypatch.setenv("RN_TUNE_SSAO_TILE_H", "16")
        rn_ao.tune_set("ssao_tile_h", 8)
        rn_ao.tune_load(str(good))
        assert rn_ao.tune_get("ssao_tile_h") == 8 and rn_ao.tune_get("trace_packet") == 16
    finally:
        for k, v in saved.items():
            rn_ao.tune_set(k, v)


def test_package_tune_file_loads(lib):
    """The autotuner's committed file for GB300 names known keys with allowed values only."""
    import rn_ao
    saved = rn_ao.tune_all()
    try:
        rn_ao.tune_load(rn_ao.TUNE_FILE)
        keys = [ln.split("=")[0].strip() for ln in open(rn_ao.TUNE_FILE) if "=" in ln and not ln.startswith("#")]
        assert keys and set(keys) <= set(rn_ao.TUNE_KEYS)
        for ln in open(rn_ao.TUNE_FILE):
            if "=" in ln and not ln.startswith("#"):
                k, v = (x.strip() for x in ln.split("=", 1))
                assert rn_ao.tune_get(k) == int(v)
    finally:
        for k, v in saved.items():
            rn_ao.tune_set(k, v)


def test_autotuner_file_round_trip(lib, tmp_path):
    """A tune file the autotuner writes (every key, one line each, known values) loads back
    as written."""
    import rn_ao
    import autotune
    saved = rn_ao.tune_all()
    try:
        pick = {k: v[-1] for k, v in rn_ao.TUNE_KEYS.items()}
        path = tmp_path / "tune.txt"
        autotune.write_tune_file(str(path), pick, "test")
        lines = [ln for ln in path.read_text().splitlines() if ln and not ln.startswith("#")]
        assert len(lines) == len(rn_ao.TUNE_KEYS)
        for k, v in saved.items():
            rn_ao.tune_set(k, v)
        rn_ao.tune_load(str(path))
        assert rn_ao.tune_all() == pick
        assert autotune.read_tune_file(str(path)) == pick      # --merge reads what it wrote
    finally:
        for k, v in saved.items():
            rn_ao.tune_set(k, v)


@pytest.mark.skipif(_cuda_present(), reason="checks the behaviour without a GPU")
def test_device_info_and_gpu_renderer_without_a_device(lib):
    """rn_device_info and raw::gpuInit / raw::renderGpu (gpu_shim.cpp, through the stand-alone
    shim build) report no device instead of answering: gpu_run.cpp then exits 4."""
    import rn_ao
    with pytest.raises(rn_ao.RnError) as e:
        rn_ao.device_info()
    assert e.value.code == 2
    import rn_build
    shim = C.CDLL(rn_build.build_shim())
    msg = C.create_string_buffer(512)
    z = np.zeros(64, np.float32)
    p = z.ctypes.data_as(C.c_void_p)
    args = [8, 8, p, p, p, p, p, 0, None, 1, 2, C.c_float(0.12), 0] + [None] * 14 + [None, 0, msg, 512]
    assert shim.shim_render_gpu(*args) == -1
    assert msg.value.startswith(b"gpuInit: ")


@pytest.mark.skipif(_cuda_present(), reason="checks the behaviour without a GPU")
def test_path_tracer_arguments_and_no_device(lib):
    """rn_pt_scene_create rejects malformed scenes before touching a device (an index out of
    range, a texture that is not a power of two) and reports no device otherwise."""
    import rn_ao
    sc = dict(pos=np.zeros((3, 3), np.float32), nrm=np.zeros((3, 3), np.float32), uv=np.zeros((3, 2), np.float32),
              idx=np.array([[0, 1, 2]], np.uint32), tri_tex=np.zeros(1, np.uint32),
              tex_entries=np.array([[0, 4, 4]], np.uint32), texels=np.zeros(16, np.uint32),
              materials=np.array([[1, 0.5, 0, 0.5, 0, 0, 0]], np.float32), sun_dir=(0, 1, 0), sun_irr=(1, 1, 1),
              sky=(0, 0, 0))
    with pytest.raises(rn_ao.RnError) as e:
        rn_ao.PtScene(dict(sc, idx=np.array([[0, 1, 3]], np.uint32)))
    assert e.value.code == 1 and "out of range" in e.value.message
    with pytest.raises(rn_ao.RnError) as e:
        rn_ao.PtScene(dict(sc, tex_entries=np.array([[0, 3, 4]], np.uint32)))
    assert e.value.code == 1 and "powers of two" in e.value.message
    with pytest.raises(rn_ao.RnError) as e:
        rn_ao.PtScene(sc)
    assert e.value.code == 2
