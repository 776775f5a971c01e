"""rn_reconcile_noalloc: the reconcile for callers that cannot let the library allocate GPU
memory (a host that budgets all device memory up front, as raw-native's fail-closed frame
arena does; a frame loop that must not stall on cudaMalloc). Its scratch is a fixed device
array inside the library. Called through the C ABI twice in a row on different data, it
must give what rn_reconcile gives: the same error map and the same counts, max and RMSE
(the tests' tolerance for RMSE is 1e-6; the reduction is the same kernel, so they agree
exactly). This file is collected last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(rn, a, t, m, tol, err):
    import torch
    r = rn.ReconcileOut()
    st = rn.Status()
    h, w = m.shape
    stream = torch.cuda.current_stream().cuda_stream
    rc = rn.lib().rn_reconcile_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(t.data_ptr()), C.c_void_p(m.data_ptr()),
                                       w, h, C.c_float(tol), C.c_void_p(stream),
                                       C.c_void_p(err.data_ptr()) if err is not None else None, C.byref(r),
                                       C.byref(st))
    assert rc == 0, st.message
    return r


def test_noalloc_reconcile_matches_rn_reconcile_twice(rn):
    import torch
    rng = np.random.default_rng(2024)
    cases = [(2160, 3840, 0.12), (333, 517, 0.3)]        # two calls in a row, different sizes and data
    for h, w, tol in cases:
        a = torch.from_numpy(rng.random((h, w), dtype=np.float32)).cuda()
        t = torch.from_numpy((np.floor(rng.random((h, w)) * 256) / 256).astype(np.float32)).cuda()
        m = torch.from_numpy((rng.random((h, w)) < 0.55).astype(np.uint8)).cuda()
        err = torch.full((h, w), -1.0, device="cuda")
        got = _noalloc(rn, a, t, m, tol, err)
        ref = rn.reconcile(a, t, m, tol)
        torch.cuda.synchronize()
        assert torch.equal(err, ref.error_map)
        assert got.pixels == ref.pixels and got.max_error == ref.max_error
        assert abs(got.rmse - ref.rmse) <= 1e-6 and got.sum_sq == ref.sum_sq
        assert bool(got.within_tolerance) == ref.within_tolerance


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
