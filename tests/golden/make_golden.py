"""Generates tests/golden/dev_scene.json: regression fixtures of the oracle's render of the
reference's dev-test scene (Scene::new_dev_test, scene.rs:158-192).

The reference cannot run here (Rust + wgpu, no graphics stack), so these images come from the oracle
(the CPU restatement) — they pin the restatement against accidental change and give the GPU tests a
committed known answer; they are not reference outputs.  Run: python tests/golden/make_golden.py
"""
import hashlib
import json
import math
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from splatter_gb300 import camera, synthetic  # noqa: E402


def scene():
    s60 = synthetic.dev_test_splats60()
    return {"center": s60[:, 4:7].copy(), "rotation": s60[:, 0:4].copy(), "scale": s60[:, 8:11].copy(),
            "alpha": s60[:, 11].copy(), "sh": s60[:, 12:60].copy()}


def main():
    cases = []
    cams = {
        "front": camera.look_at([0.3, 0.4, -3.0], [0.3, 0.3, 0.3]),
        "oblique": camera.look_at([1.5, 1.2, -3.0], [0.3, 0.3, 0.3]),
        "close": camera.look_at([0.2, 0.1, -0.8], [0.6, 0.3, 0.4]),
    }
    sc = scene()
    for cname, cam in cams.items():
        for rect in (True, False):
            for cov in (True, False):
                for fovy in (math.pi / 2, math.radians(60)):
                    name = f"{cname}_rect{int(rect)}_cov{int(cov)}_fov{round(math.degrees(fovy))}"
                    u = oracle.uniforms(cam, 160, 120, fovy=fovy)
                    cfg = oracle.config_struct(depth_sorting=2, sh_order=0, use_covariance_for_scale=cov,
                                               use_unaligned_rectangles=rect)
                    img, st = oracle.render(u, cfg, sc)
                    cases.append({"name": name, "camera": [float(x) for x in cam], "width": 160, "height": 120,
                                  "fovy": fovy, "depth_sorting": 2, "covariance": cov, "rect": rect,
                                  "sha256": hashlib.sha256(img.tobytes()).hexdigest(), "stats": list(st),
                                  "nonblack_pixels": int(np.count_nonzero(img[..., :3].sum(-1)))})
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dev_scene.json")
    with open(out, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py (oracle render, unorm8 blend)", "cases": cases}, f,
                  indent=1)
    print(out, len(cases))


if __name__ == "__main__":
    main()
