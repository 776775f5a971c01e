"""Generate tests/golden/*.json from the reference (run in a container that has the
raw-native tree; the committed JSON is what the tests read).

  - identity.json: the reference's committed SHA-256 goldens of the AO outputs for each
    CLI case (evidence/identity-golden.json), with the camera each case renders, and the
    exact reconcile numbers of each case from the reference's own code (oracle/_ref).
  - ploc.json: PLOC tree hashes and round counts: the soup scene from the reference's GPU
    evidence (evidence/rt-r2-bvh-gpu-d3d12-rtx4090.json) and the built-in test scene from
    the reference's rt::buildPloc.
  - gtao.json: raw::post::gtao (FP64) of the built-in scene at 256 x 256 from the two test
    cameras of evidence/m3-post-bounds.json, by the reference's own code: SHA-256 of the
    float64 output, its mean over covered pixels and the covered count.

    python tests/golden/make_golden.py [/path/to/raw-native]
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

FILES = ("ao_rt.pfm", "ao_ss.pfm", "mask.pgm", "ao_error.pgm")
# evidence/m3-post-bounds.json "scenes": the built-in scene from the CLI camera and from the
# near camera (eye 1.8, 3.2, 2.4 toward 0.8, 0.2, 1.0)
GTAO_CAMERAS = {"test_scene": tuple(O.DEFAULT_CAMERA), "near": (1.8, 3.2, 2.4, 0.8, 0.2, 1.0, 0.0, 1.0, 0.0, 0.9)}


def camera_of(args):
    w = h = 256
    cam = list(O.DEFAULT_CAMERA)
    it = iter(args)
    for a in it:
        if a == "--width":
            w = int(next(it))
        elif a == "--height":
            h = int(next(it))
        elif a == "--eye":
            cam[0:3] = [float(v) for v in next(it).split(",")]
        elif a == "--target":
            cam[3:6] = [float(v) for v in next(it).split(",")]
        elif a == "--fovy":
            cam[9] = float(next(it))
        elif a in ("--prev-eye", "--threads"):
            next(it)
    return w, h, cam


def main(ref_dir):
    O.build(with_ref=True)
    R = O.ref()
    gold = json.load(open(os.path.join(ref_dir, "evidence", "identity-golden.json")))["cases"]
    cases = {}
    for name, case in sorted(gold.items()):
        files = {f: case["files"][f] for f in FILES if f in case["files"]}
        if "ao_rt.pfm" not in files:
            continue
        w, h, cam = camera_of(case["args"])
        n = w * h
        bufs = dict(pos=np.zeros(n * 3, np.float32), nrm=np.zeros(n * 3, np.float32), mask=np.zeros(n, np.uint8),
                    ao=np.zeros(n, np.float32), sky=np.zeros(n, np.float32), sun=np.zeros(n, np.float32),
                    ss=np.zeros(n, np.float32), err=np.zeros(n, np.float32))
        stats = np.zeros(4, np.float32)
        R.ref_render_default(w, h, np.array(cam, np.float32), O.RT_SAMPLES, O.AO_RADIUS, O.SS_SAMPLES, O.TOLERANCE,
                             os.cpu_count() or 1, bufs["pos"], bufs["nrm"], bufs["mask"], bufs["ao"], bufs["sky"],
                             bufs["sun"], bufs["ss"], bufs["err"], stats)
        got = {"ao_rt.pfm": O.sha256(O.pfm1_bytes(bufs["ao"].reshape(h, w))),
               "ao_ss.pfm": O.sha256(O.pfm1_bytes(bufs["ss"].reshape(h, w))),
               "mask.pgm": O.sha256(O.mask_pgm_bytes(bufs["mask"].reshape(h, w))),
               "ao_error.pgm": O.sha256(O.pgm_bytes(bufs["err"].reshape(h, w)))}
        assert got == files, (name, got, files)
        cases[name] = dict(args=case["args"], width=w, height=h, camera=cam, files=files,
                           frame_files={f: case["files"][f] for f in ("frame.ppm", "frame_hdr.pfm")},
                           exact=dict(rmse=float(stats[0]), maxError=float(stats[1]), pixels=int(stats[2]),
                                      within=bool(stats[3])),
                           sky_sha256=O.sha256(O.pfm1_bytes(bufs["sky"].reshape(h, w))),
                           sun_sha256=O.sha256(O.pfm1_bytes(bufs["sun"].reshape(h, w))))
    json.dump(dict(source="evidence/identity-golden.json of raw-native (AO outputs) + reference build stats",
                   samples=dict(rt=O.RT_SAMPLES, ss=O.SS_SAMPLES), radius=O.AO_RADIUS, tolerance=O.TOLERANCE,
                   cases=cases), open(os.path.join(HERE, "identity.json"), "w"), indent=1, sort_keys=True)
    ev = json.load(open(os.path.join(ref_dir, "evidence", "rt-r2-bvh-gpu-d3d12-rtx4090.json")))
    soup = [s for s in ev["scenes"] if s["scene"] == "soup"][0]
    ts, _, _ = O.test_scene()
    n = len(ts)
    out = np.zeros((2 * n - 1, 9), np.int32)
    rounds = C.c_uint32()
    root = R.ref_ploc(ts, n, 16, out, C.byref(rounds))
    json.dump(dict(source="evidence/rt-r2-bvh-gpu-d3d12-rtx4090.json (soup) and rt::buildPloc (test scene)",
                   scenes=dict(soup=dict(count=20000, seed=7, triangles=soup["triangles"], rounds=soup["rounds"],
                                         tree_hash=soup["cpu_tree_hash"]),
                               test_scene=dict(triangles=n, rounds=rounds.value, root=root,
                                               tree_hash=O.tree_hash(out)))),
              open(os.path.join(HERE, "ploc.json"), "w"), indent=1, sort_keys=True)
    gt = {}
    tris, nrm9, _ = O.test_scene()
    for name, cam in GTAO_CAMERAS.items():
        _, pos, nrm, mask = O.rasterize(tris, nrm9, cam, 256, 256)
        vp, vn, vd = O.view_gbuffer(pos, nrm, mask, cam, use_ref=True)
        a = O.gtao(vp, vn, vd, cam[9], use_ref=True)
        gt[name] = dict(camera=list(cam), width=256, height=256, radius=0.5, slices=16, steps=16,
                        sha256=O.sha256(np.ascontiguousarray(a).tobytes()), covered=int(mask.sum()),
                        mean_covered=float(a[mask > 0].mean()))
    json.dump(dict(source="raw::post::gtao (src/renderer/post_gtao.cpp) built from the reference's sources",
                   cases=gt), open(os.path.join(HERE, "gtao.json"), "w"), indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "identity.json"), os.path.join(HERE, "ploc.json"),
          os.path.join(HERE, "gtao.json"))


if __name__ == "__main__":
    _ref = sys.argv[1] if len(sys.argv) > 1 else O.reference_dir()
    if not _ref:
        sys.exit("usage: make_golden.py RAW_NATIVE_TREE (or set RN_REFERENCE_DIR)")
    main(_ref)
