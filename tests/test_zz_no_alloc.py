"""rn_reconcile_noalloc: the reconcile for callers that cannot let the library allocate GPU
memory (a host that budgets all device memory up front, as raw-native's fail-closed frame
arena does; a frame loop that must not stall on cudaMalloc). Its scratch is a fixed device
array inside the library. Called through the C ABI twice in a row on different data, it
must give what rn_reconcile gives: the same error map and the same counts, max and RMSE
(the tests' tolerance for RMSE is 1e-6; the reduction is the same kernel, so they agree
exactly). Also covered: no error map (err NULL), pointers that are not 16-byte aligned
(the scalar kernel and its tail), the legacy default stream (stream NULL), and, in a fresh
process, that the calls leave the device's free memory unchanged while rn_reconcile's first
call (its context and workspace) does not. This file is collected last."""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _noalloc(rn, a, t, m, w, h, tol, err, stream="current"):
    import torch
    r = rn.ReconcileOut()
    st = rn.Status()
    s = torch.cuda.current_stream().cuda_stream if stream == "current" else None
    rc = rn.lib().rn_reconcile_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(t.data_ptr()), C.c_void_p(m.data_ptr()),
                                       w, h, C.c_float(tol), C.c_void_p(s) if s else None,
                                       C.c_void_p(err.data_ptr()) if err is not None else None, C.byref(r),
                                       C.byref(st))
    assert rc == 0, st.message
    return r


def _inputs(rng, h, w):
    import torch
    a = torch.from_numpy(rng.random((h, w), dtype=np.float32)).cuda()
    t = torch.from_numpy((np.floor(rng.random((h, w)) * 256) / 256).astype(np.float32)).cuda()
    m = torch.from_numpy((rng.random((h, w)) < 0.55).astype(np.uint8)).cuda()
    return a, t, m


def _same(got, ref):
    assert got.pixels == ref.pixels and got.max_error == ref.max_error
    assert abs(got.rmse - ref.rmse) <= 1e-6 and got.sum_sq == ref.sum_sq
    assert bool(got.within_tolerance) == ref.within_tolerance


def test_noalloc_reconcile_matches_rn_reconcile_twice(rn):
    import torch
    rng = np.random.default_rng(2024)
    cases = [(2160, 3840, 0.12), (333, 517, 0.3)]        # two calls in a row, different sizes and data
    for h, w, tol in cases:
        a, t, m = _inputs(rng, h, w)
        err = torch.full((h, w), -1.0, device="cuda")
        got = _noalloc(rn, a, t, m, w, h, tol, err)
        ref = rn.reconcile(a, t, m, tol)
        torch.cuda.synchronize()
        assert torch.equal(err, ref.error_map)
        _same(got, ref)


def test_noalloc_without_error_map_unaligned_and_default_stream(rn):
    """err NULL; inputs offset by one element (no 16-byte alignment: the scalar kernel, whose
    tail covers the last pixels); the legacy default stream (stream NULL)."""
    import torch
    rng = np.random.default_rng(77)
    h, w = 611, 1033
    a, t, m = _inputs(rng, h, w)
    ref = rn.reconcile(a, t, m, 0.2)
    _same(_noalloc(rn, a, t, m, w, h, 0.2, None), ref)
    _same(_noalloc(rn, a, t, m, w, h, 0.2, None, stream=None), ref)
    # flat views one element in: 4-byte aligned floats, odd mask address, odd pixel count
    n = h * w - 1
    a1, t1, m1 = a.reshape(-1)[1:], t.reshape(-1)[1:], m.reshape(-1)[1:]
    e1 = torch.full((n + 1,), -1.0, device="cuda")[1:]
    got = _noalloc(rn, a1, t1, m1, n, 1, 0.2, e1, stream=None)
    ref1 = rn.reconcile(a1.contiguous().reshape(1, n), t1.contiguous().reshape(1, n), m1.contiguous().reshape(1, n), 0.2)
    torch.cuda.synchronize()
    assert torch.equal(e1.reshape(1, n), ref1.error_map)
    _same(got, ref1)


def test_noalloc_rejects_oversize_and_empty(rn):
    r = rn.ReconcileOut()
    st = rn.Status()
    one = C.c_void_p(1)
    assert rn.lib().rn_reconcile_noalloc(one, one, one, 65536, 65536, C.c_float(0.1), None, None, C.byref(r),
                                         C.byref(st)) == 1
    assert b"at most" in st.message
    assert rn.lib().rn_reconcile_noalloc(one, one, one, 0, 7, C.c_float(0.1), None, None, C.byref(r),
                                         C.byref(st)) == 0
    assert r.pixels == 0 and r.rmse == 0.0


_FRESH = textwrap.dedent(r"""
    import ctypes as C, sys
    import numpy as np, torch
    sys.path[:0] = [sys.argv[1], sys.argv[1] + "/raw-native_gb300"]
    import rn_ao as rn
    L = rn.lib()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(5)
    def inputs(h, w):
        a = torch.from_numpy(rng.random((h, w), dtype=np.float32)).cuda()
        t = torch.from_numpy(rng.random((h, w), dtype=np.float32)).cuda()
        m = torch.from_numpy((rng.random((h, w)) < 0.5).astype(np.uint8)).cuda()
        return a, t, m, torch.empty(h, w, device="cuda")
    def call(a, t, m, e, w, h, stream):
        r, st = rn.ReconcileOut(), rn.Status()
        rc = L.rn_reconcile_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(t.data_ptr()), C.c_void_p(m.data_ptr()),
                                    w, h, C.c_float(0.1), stream, C.c_void_p(e.data_ptr()) if e is not None else None,
                                    C.byref(r), C.byref(st))
        assert rc == 0, st.message
        return r
    small, big = inputs(64, 64), inputs(2160, 3840)
    flat = [x.reshape(-1)[1:] for x in big]
    torch.cuda.synchronize()
    # the first calls load the library's kernels and its scratch array (module loading, not a
    # cudaMalloc): one aligned and one unaligned call on a small image
    call(*small, 64, 64, None)
    call(*[x.reshape(-1)[1:] for x in small], 64 * 64 - 1, 1, None)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    r1 = call(*big, 3840, 2160, None)
    r2 = call(*flat, 3840 * 2160 - 1, 1, None)
    r3 = call(*big[:3], None, 3840, 2160, None)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert r1.pixels > 0 and r2.pixels > 0 and r3.pixels == r1.pixels
    ref = rn.reconcile(*big[:3], 0.1)           # the library's context and workspace: allocates
    torch.cuda.synchronize()
    free2 = torch.cuda.mem_get_info()[0]
    assert abs(ref.rmse - r1.rmse) <= 1e-6 and ref.pixels == r1.pixels
    print("FREE", free0, free1, free2)
""")


def test_noalloc_allocates_nothing_in_a_fresh_process():
    """A fresh process: after the first small calls (which load the kernels and the scratch
    array), three 4K calls leave cudaMemGetInfo's free bytes exactly unchanged; the control,
    rn_reconcile's first call, lowers them (it opens the context and its workspace)."""
    r = subprocess.run([sys.executable, "-c", _FRESH, ROOT], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-3000:]
    line = [x for x in r.stdout.splitlines() if x.startswith("FREE")][-1]
    free0, free1, free2 = (int(v) for v in line.split()[1:])
    assert free1 == free0, "rn_reconcile_noalloc changed free device memory by %d bytes" % (free0 - free1)
    assert free2 < free1, "the control (rn_reconcile's first call) allocated nothing visible"
