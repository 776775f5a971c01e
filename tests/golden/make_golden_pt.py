"""Generate the path tracer's golden fixtures from the reference's own build (run in a
container that has the raw-native tree; the committed files are what the tests read).

  - pt_scenes.npz: the reference's lit scenes as plain arrays, made by its own builders
    (src/renderer/rt_pt_scene.cpp: ptRetroRoom, ptIsoStreet, ptFurnace, ptWhitePlane) with
    their cameras: vertices, uvs, indices, per-triangle texture, the texture set, the
    materials (baseFactor, roughness, metallic, specular, emission), sun and sky.
  - pt.json: raw::rt::pathTraceCpu's outputs on those scenes for a set of render
    descriptions (seed, spp, size, controls): the SHA-256 of every AOV's float32 / int32
    bytes, plus the SHA-256 of the lobe's energy table (src/renderer/rt_pt_energy.cpp).

    python tests/golden/make_golden_pt.py [/path/to/raw-native]
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

SCENES = {
    "retro_room": dict(name="retro_room"),
    "iso_street": dict(name="iso_street"),
    "furnace": dict(name="furnace", emission=1.0, albedo=0.5),
    "white_plane_metal": dict(name="white_plane", material=(1.0, 0.2, 1.0, 1.0, 0, 0, 0), sky=(1.0, 1.0, 1.0)),
    "white_plane_dielectric": dict(name="white_plane", material=(1.0, 0.5, 0.0, 0.5, 0, 0, 0), sky=(1.0, 1.0, 1.0)),
}

# (case name, scene, render description); the camera is the scene's unless given
CASES = [
    ("retro_room_16spp", "retro_room", dict(seed=1, spp=16, width=96, height=64)),
    ("retro_room_legacy_lobe", "retro_room", dict(seed=3, spp=8, width=64, height=48, controls=["legacy_lobe_v2"])),
    ("retro_room_motion_nojitter", "retro_room", dict(seed=2, spp=4, spp_begin=5, width=80, height=60, jitter=False,
                                                      previous_shift=(0.3, 0.0, -0.2))),
    ("retro_room_mis_one_split_controls", "retro_room",
     dict(seed=9, spp=8, width=48, height=32, controls=["mis_weight_one", "aov_drop_specular_indirect"])),
    ("iso_street_16spp", "iso_street", dict(seed=1, spp=16, width=96, height=64)),
    ("furnace_no_rr", "furnace", dict(seed=101, spp=16, width=64, height=48, russian_roulette=False)),
    ("white_plane_metal", "white_plane_metal", dict(seed=1, spp=16, width=64, height=48)),
    ("white_plane_dielectric", "white_plane_dielectric", dict(seed=4, spp=16, width=64, height=48, max_bounces=8)),
]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def desc_for(case: dict, cam):
    d = {k: v for k, v in case.items() if k != "previous_shift"}
    d["camera"] = [float(v) for v in cam]
    prev = list(d["camera"])
    if "previous_shift" in case:
        for k in range(3):
            prev[k] = float(np.float32(prev[k] + case["previous_shift"][k]))
    d["previous"] = prev
    return d


def main(ref_dir):
    os.environ["RN_REFERENCE_DIR"] = ref_dir
    O.build(with_ref=True)
    table = O.pt_energy_table(use_ref=True)
    arrays, scenes = {}, {}
    for key, spec in SCENES.items():
        sc, cam = O.pt_reference_scene(spec["name"], spec.get("emission", 1.0), spec.get("albedo", 0.5),
                                       spec.get("material"), spec.get("sky", (1.0, 1.0, 1.0)))
        for k, v in sc.items():
            arrays["%s/%s" % (key, k)] = np.asarray(v)
        arrays["%s/camera" % key] = cam
        scenes[key] = dict(triangles=int(len(sc["idx"])), vertices=int(len(sc["pos"])), textures=int(len(sc["tex_entries"])))
    np.savez_compressed(os.path.join(HERE, "pt_scenes.npz"), **arrays)
    cases = {}
    for name, key, case in CASES:
        sc = {k.split("/", 1)[1]: v for k, v in arrays.items() if k.startswith(key + "/") and not k.endswith("/camera")}
        d = desc_for(case, arrays[key + "/camera"])
        out = O.pathtrace(sc, d, use_ref=True)
        cases[name] = dict(scene=key, desc=d, emitters=int(out["emitters"]),
                           sha256={k: sha(out[k]) for k, _, _ in O.PT_AOVS},
                           radiance_mean=float(out["radiance"].astype(np.float64).mean()))
    json.dump(dict(source="raw::rt::pathTraceCpu (src/renderer/rt_pt_cpu.cpp) of the reference's own build on its "
                          "lit scenes (src/renderer/rt_pt_scene.cpp)",
                   energy_table_sha256=sha(table), scenes=scenes, cases=cases),
              open(os.path.join(HERE, "pt.json"), "w"), indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "pt_scenes.npz"), os.path.join(HERE, "pt.json"))


if __name__ == "__main__":
    _ref = sys.argv[1] if len(sys.argv) > 1 else O.reference_dir()
    if not _ref:
        sys.exit("usage: make_golden_pt.py RAW_NATIVE_TREE (or set RN_REFERENCE_DIR)")
    main(_ref)
