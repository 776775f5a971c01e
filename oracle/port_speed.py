"""Speed of the oracle port against the reference's own compiled path (test infrastructure).

Times, on this host's cores, the reference's computeRTVisibility + computeSSAO + reconcile
(oracle/_ref/libref_ao.so: src/renderer/ray_ao.cpp:53-63, src/renderer/ssao.cpp:11-39,
src/cert/reconcile.cpp:4-21 compiled where they lie) against the port's rno_trace + rno_ssao +
rno_reconcile (oracle/rn_oracle.c) on the same G-buffer: the built-in scene from the CLI's
camera, lighting model 2 (AO + sky + sun), SSAO 24 taps, tolerance 0.12. Each pass is timed
separately, median of `reps` alternating runs, the same thread count on both sides; the outputs are
checked equal first. Prints one JSON object. Needs oracle/_ref (a host with the raw-native
tree); the GPU host has none.

    python oracle/port_speed.py [--w 3840 --h 2160 --spp 256 --threads N --reps 5]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import sys
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:] = [q for q in sys.path if os.path.abspath(q or ".") != _HERE]
sys.path.insert(0, os.path.dirname(_HERE))
from oracle import oracle as O  # noqa: E402


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--w", type=int, default=3840)
    p.add_argument("--h", type=int, default=2160)
    p.add_argument("--spp", type=int, default=256)
    p.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    p.add_argument("--reps", type=int, default=5)
    a = p.parse_args()
    try:
        R = O.ref()
    except OSError:
        R = None
    if R is None:
        sys.exit("oracle/_ref is not built on this host (no raw-native tree)")
    L = O.lib()
    w, h, spp, T = a.w, a.h, a.spp, a.threads
    tris, nrm9, light = O.test_scene()
    _, pos, nrm, mask = O.rasterize(tris, nrm9, O.DEFAULT_CAMERA, w, h)
    tl = np.ascontiguousarray(-light, np.float32)
    covered = int(mask.sum())

    def port_trace():
        ao, sky, sun = (np.zeros((h, w), np.float32) for _ in range(3))
        acc = L.rno_accel_build(np.ascontiguousarray(tris), len(tris))
        L.rno_trace(w, h, pos, nrm, mask, acc, tris, len(tris), spp, 2.0, C.cast(tl.ctypes.data, C.c_void_p), 0, ao,
                    sky.ctypes.data_as(C.c_void_p), sun.ctypes.data_as(C.c_void_p), T, 0, 1)
        L.rno_accel_free(acc)
        return ao, sky, sun

    def ref_trace():
        ao, sky, sun = (np.zeros((h, w), np.float32) for _ in range(3))
        R.ref_trace(w, h, pos, nrm, mask, tris, len(tris), spp, 2.0, C.c_void_p(tl.ctypes.data), ao,
                    C.c_void_p(sky.ctypes.data), C.c_void_p(sun.ctypes.data), T)
        return ao, sky, sun

    def port_ssao():
        return O.ssao(pos, nrm, mask, O.SS_SAMPLES, 2.0, T)

    def ref_ssao():
        out = np.zeros((h, w), np.float32)
        R.ref_ssao(w, h, pos, nrm, mask, O.SS_SAMPLES, 2.0, out, T)
        return out

    ao_p, sky_p, sun_p = port_trace()
    ao_r, sky_r, sun_r = ref_trace()
    assert np.array_equal(ao_p, ao_r) and np.array_equal(sky_p, sky_r) and np.array_equal(sun_p, sun_r)
    ss_p, ss_r = port_ssao(), ref_ssao()
    assert np.array_equal(ss_p, ss_r)

    def port_rec():
        return O.reconcile(ss_p, ao_p, mask, O.TOLERANCE)

    def ref_rec():
        err = np.zeros((h, w), np.float32)
        st = np.zeros(4, np.float32)
        R.ref_reconcile(w, h, ss_r, ao_r, mask, O.TOLERANCE, err, st)
        return err

    assert np.array_equal(port_rec()[0], ref_rec())

    def med2(fp, fr):
        """Medians of alternating runs (port, reference, port, ...): drift of the host's clock or
        load falls on both sides alike."""
        tp, tr = [], []
        for _ in range(a.reps):
            for fn, ts in ((fp, tp), (fr, tr)):
                t0 = time.perf_counter()
                fn()
                ts.append(time.perf_counter() - t0)
        return statistics.median(tp), statistics.median(tr)

    res = {"host": os.uname().machine, "threads": T, "w": w, "h": h, "spp": spp, "covered_px": covered,
           "reps": a.reps, "outputs_equal": True, "passes": {}}
    for name, fp, fr in (("visibility (AO + sky + sun)", port_trace, ref_trace), ("ssao", port_ssao, ref_ssao),
                         ("reconcile", port_rec, ref_rec)):
        tp, tr = med2(fp, fr)
        res["passes"][name] = {"port_s": tp, "reference_s": tr, "port_over_reference": tp / tr}
    tp = sum(v["port_s"] for v in res["passes"].values())
    tr = sum(v["reference_s"] for v in res["passes"].values())
    res["frame"] = {"port_s": tp, "reference_s": tr, "port_over_reference": tp / tr,
                    "port_grays_per_s": covered * spp / tp / 1e9, "reference_grays_per_s": covered * spp / tr / 1e9}
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
