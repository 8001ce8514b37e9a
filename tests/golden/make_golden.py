"""Generates tests/golden/oracle_frames.json: hashes and sample values of the
oracle's frames on seeded scenes, each scene and camera built by the oracle
itself. They pin the oracle (its load-time scene build and its frame)
against regressions; the reference itself cannot be run here, so these are
not reference outputs.

Run: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "swraster-viewer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
import scenes  # noqa: E402

CASES = [
    {"name": "small_default", "scene": ("small", 3), "size": (320, 200), "rsqrt": 1, "dt": 0.0},
    {"name": "small_ieee", "scene": ("small", 3), "size": (160, 96), "rsqrt": 0, "dt": 0.0},
    {"name": "small_odd", "scene": ("small", 7), "size": (97, 61), "rsqrt": 1, "dt": 0.5},
    {"name": "stress_reduced", "scene": ("stress", 4), "size": (480, 270), "rsqrt": 1, "dt": 0.0},
]


def build(spec, w, h):
    kind, seed = spec
    if kind == "small":
        s = oracle.Scene(scenes.small_scene(seed=seed))
        _, _, c, diag = s.bounds
        cam = oracle.camera(*scenes.default_camera_params(scenes.Bounds(c, diag), w, h))
    else:
        sd, cp = scenes.stress_scene(seed=seed, triangles=20_000, width=w, height=h, n_textures=2, tex_size=64,
                                     cube_size=16, voxel=16, specular_samples=8, brdf_lut_size=16)
        s = oracle.Scene(sd)
        cam = oracle.camera(*cp)
    return s, cam


def render_case(c):
    w, h = c["size"]
    s, cam = build(tuple(c["scene"]), w, h)
    rgba, vis, tl, res = oracle.render(s, cam, w, h, rsqrt_mode=c["rsqrt"], threads=1, dt=c["dt"])
    s.close()
    return {"rgba_sha256": hashlib.sha256(rgba.tobytes()).hexdigest(),
            "vis_sha256": hashlib.sha256(vis.tobytes()).hexdigest(),
            "tile_lum_sha256": hashlib.sha256(tl.tobytes()).hexdigest(),
            "covered": int((vis != np.uint64(2 ** 64 - 1)).sum()), "packets": int(res.packets),
            "exposure": float(res.exposure), "center_pixel": int(rgba[h // 2 & ~1, w // 2])}


def main():
    out = {"note": "oracle frames on seeded synthetic scenes (regression pins, not reference outputs)",
           "cases": []}
    for c in CASES:
        d = dict(c)
        d.update(render_case(c))
        out["cases"].append(d)
        print(c["name"], d["covered"], d["packets"])
    with open(os.path.join(HERE, "oracle_frames.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
