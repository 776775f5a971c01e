"""The benchmark's command-line contract, checked on a CPU host: the reference arm prints one
JSON line with every key the contract names (once, from rank 0, under torchrun), and the
GPU arm fails loudly without a GPU instead of falling back to the CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BENCH = os.path.join(ROOT, "bench.py")
KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config")


def _cuda_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def _json_lines(out: str):
    return [json.loads(ln) for ln in out.splitlines() if ln.startswith("{")]


def _check_reference_line(d, n_gpus):
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference" and d["n_gpus"] == n_gpus and d["value"] > 0
    assert d["higher_is_better"] is True and d["scaling"] == "weak" and d["vs_baseline"] is None
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_prints_the_contract_line(oracle):
    r = subprocess.run([sys.executable, BENCH, "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--cpu-row-stride", "64"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_reference_line(lines[0], 1)


def test_reference_arm_under_torchrun_prints_once(oracle):
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), BENCH, "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-row-stride", "64"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_reference_line(lines[0], 2)


@pytest.mark.skipif(_cuda_present(), reason="checks the behaviour without a GPU")
def test_gpu_arm_fails_without_a_gpu():
    r = subprocess.run([sys.executable, BENCH, "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode != 0
    assert not _json_lines(r.stdout)


def test_equal_rmse_spp_is_the_smallest_passing_integer():
    """The head-to-head's spp rule: the smallest integer spp meeting the RMSE bar on every
    view, found by powers of two and bisection, on monotone curves whose answer is known."""
    sys.path.insert(0, ROOT)
    import bench
    for c in (0.08, 0.25, 0.2368, 0.3, 0.64, 0.02, 0.0199):
        def worst(s, c=c):
            return c / s ** 0.5
        got, seen = bench.equal_rmse_spp(worst, 0.02, 16, 1024)
        want = next(k for k in range(1, 5000) if worst(k) <= 0.02)
        assert got == max(16, want), (c, got, want)
        assert worst(got) <= 0.02 and len(seen) <= 20
    got, _ = bench.equal_rmse_spp(lambda s: 1.0, 0.02, 16, 1024)     # never meets the bar: the cap
    assert got == 1024


def test_reference_arm_config_is_the_gpu_arms(oracle):
    """Both arms print the same config dict (covered pixels of the 4K default view included)."""
    sys.path.insert(0, ROOT)
    import bench
    cfg = bench.frame_config(1, bench.covered_pixels_cpu())
    assert cfg["covered_px"] == 3992795 and cfg["ao_rays_per_step"] == 3992795 * 256
