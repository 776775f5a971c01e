"""Build librn_ao.so (the sm_103a AO path) in place.

Each CUDA translation unit compiles in parallel with nvcc for sm_103a only; the objects link
into ``raw-native_gb300/librn_ao.so``. Device code builds with ``-fmad=false`` so no
multiply-add is contracted unless the source asks for it, and host code with
``-ffp-contract=off``: the reference's answers are defined by unfused float32 operations.
The C++23 drop-in shim (``host/``) builds into ``librn_ao_shim.so`` on top of it.

    python raw-native_gb300/rn_build.py         # library + shim
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librn_ao.so")
SHIM = os.path.join(HERE, "librn_ao_shim.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librn_ao.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _stale(target: str, sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_library(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "rn_ao.h"))
    jobs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f[:-3] + ".o")
        if _stale(obj, [src] + headers):
            jobs.append([nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    objs = [os.path.join(OBJ, f[:-3] + ".o") for f in cu]
    if _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_shim(verbose: bool = False) -> str:
    """The reference-facing C++23 shim (computeRTAO & co. over the C ABI), built stand-alone
    against host/mirror's headers with a C test API (librn_ao_shim.so). Inside a raw-native
    build the same ao_shim.cpp compiles against the reference's headers instead."""
    mirror = os.path.join(HOST, "mirror")
    srcs = [os.path.join(HOST, "ao_shim.cpp"), os.path.join(HOST, "gpu_shim.cpp")] + sorted(
        os.path.join(mirror, f) for f in os.listdir(mirror) if f.endswith(".cpp"))
    hdrs = [os.path.join(dp, f) for dp, _, fs in os.walk(HOST) for f in fs if f.endswith(".hpp")]
    if _stale(SHIM, srcs + hdrs + [LIB]):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-std=c++23", "-O2", "-fPIC", "-ffp-contract=off", "-shared", "-I" + mirror,
              "-I" + os.path.join(ROOT, "include"), "-I" + HOST, "-o", SHIM] + srcs +
             ["-L" + HERE, "-lrn_ao", "-Wl,-rpath,$ORIGIN"])
    return SHIM


def build(verbose: bool = False) -> None:
    build_library(verbose)
    if os.path.isdir(HOST):
        build_shim(verbose)


if __name__ == "__main__":
    build(verbose=True)
    print(LIB)
