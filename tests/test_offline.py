"""Headless offline renderer (the viewer loop without a window): the PNG writer on the CPU, and on
the GPU a camera path rendered to files that equal the frames render_frame gives, with and without
progressive loading."""
import numpy as np
import pytest

from splatter_gb300 import offline


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    for h, w in ((1, 1), (7, 13), (64, 48)):
        img = rng.integers(0, 256, size=(h, w, 3), dtype=np.uint8)
        p = tmp_path / f"x{h}_{w}.png"
        offline.write_png(p, img)
        assert p.read_bytes()[:8] == b"\x89PNG\r\n\x1a\n"
        assert np.array_equal(offline.read_png(p), img)


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [0, 10000])
def test_offline_sequence_equals_render_frame(cuda, tmp_path, chunk):
    from splatter_gb300 import Configuration, Renderer, Scene, camera, synthetic
    n, W, H, poses = 30000, 160, 120, 4
    rec = synthetic.clustered(n, seed=3, sh_order=3)
    ply = tmp_path / "s.ply"
    synthetic.write_ply(ply, rec)
    out = tmp_path / "frames"
    args = [str(ply), "--out", str(out), "--width", str(W), "--height", str(H), "--poses", str(poses),
            "--radius", "30", "40", "--seed", "5", "--fovy", "60"]
    if chunk:
        args += ["--chunk", str(chunk)]
    assert offline.main(args) == 0
    rows = (out / "timing.csv").read_text().strip().splitlines()
    assert rows[0] == "frame,device_ms,wall_ms,chunks_left" and len(rows) == 1 + poses
    assert all(float(r.split(",")[1]) > 0 for r in rows[1:])
    import math
    r = Renderer(Configuration(max_splat_count=n, spherical_harmonics_order=3, field_of_view_y=math.radians(60)))
    s = Scene(r, n)
    s.load_chunk(rec)
    cams = camera.orbit_poses(poses, 6, radius=(30.0, 40.0))
    first_full = 0 if not chunk else (n + chunk - 1) // chunk - 1  # the frame after the last chunk's step
    for k in range(first_full, poses):
        want = r.render_frame(s, cams[k], W, H).cpu().numpy()[..., :3]
        assert np.array_equal(offline.read_png(out / f"frame_{k:05d}.png"), want)
