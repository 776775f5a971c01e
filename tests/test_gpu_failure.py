"""Failure detection on the GPU without a fault: a bounded device-side wait is made to run
out (a tensor-core GEMM whose only stage is never filled); the kernel records the error,
frees its TMEM and returns, the call reports RN_ERR_BUDGET, and the next calls on the same
context work."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wait_budget_reports_and_the_context_survives(rn):
    import time
    import torch
    t0 = time.time()
    with pytest.raises(rn.RnError) as e:
        rn.selftest_wait_budget(1 << 14)
    assert e.value.code == 6, e.value                  # RN_ERR_BUDGET
    assert "iteration budget" in str(e.value)
    assert time.time() - t0 < 30
    # the same context keeps working: a GEMM and an AO pass
    P = torch.randn(256, 128, device="cuda").to(torch.bfloat16)
    Q = torch.randn(64, 128, device="cuda").to(torch.bfloat16)
    C = rn.tc_gemm(P, Q)
    torch.cuda.synchronize()
    assert torch.allclose(C, P.float() @ Q.float().T, rtol=1e-2, atol=1e-2)
    a = np.random.default_rng(0).random((64, 64), dtype=np.float32)
    r = rn.reconcile(a, a, np.ones((64, 64), np.uint8))
    assert r.rmse == 0.0 and r.pixels == 64 * 64
    with pytest.raises(rn.RnError):
        rn.selftest_wait_budget(0)                     # refused before any device work
