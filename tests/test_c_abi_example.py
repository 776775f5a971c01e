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
