"""Known-answer tests that pin the oracle (the CPU restatement) to closed forms.

The reference ships no tests or golden vectors and cannot be run here, so these closed-form checks
(and the committed golden fixtures of tests/golden/) are what pins the restatement.  CPU only.
"""
import json
import math
import os

import numpy as np
import pytest

import oracle
from splatter_gb300 import camera, synthetic
from tests.helpers import scene_from_splats60

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_expf_accuracy_and_specials():
    xs = np.concatenate([np.linspace(-103.0, 88.0, 20001), np.linspace(-6.0, 0.0, 20001)]).astype(np.float32)
    got = np.array([oracle.expf(float(x)) for x in xs[::7]], np.float64)
    ref = np.exp(xs[::7].astype(np.float64))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(got - ref) / ulp) <= 2.0
    assert oracle.expf(0.0) == 1.0
    assert oracle.expf(-200.0) == 0.0
    assert math.isinf(oracle.expf(100.0))
    assert math.isnan(oracle.expf(float("nan")))


def test_uniforms_closed_form():
    cam = camera.look_at([0.0, 0.0, -5.0], [0.0, 0.0, 0.0])
    u = oracle.uniforms(cam, 200, 100, fovy=math.pi / 2)
    vp = u["vp"][0].reshape(4, 4)  # [col][row]
    # camera looks along +z from z=-5: view z = world z + 5; P: x/(vw), y/(vh), z: 1000/999 (1 - 1/z)
    assert u["view_size"][0][1] == np.float32(1.0)  # tan(pi/4) rounds to 1 in f32
    assert u["view_size"][0][0] == np.float32(2.0)  # aspect * 1
    p = np.array([1.0, 0.5, 0.0, 1.0], np.float32)
    h = vp.T @ p
    assert abs(h[3] - 5.0) < 1e-6
    assert abs(h[0] / h[3] - 1.0 / 2.0 / 5.0) < 1e-6
    assert abs(h[1] / h[3] - 0.5 / 5.0) < 1e-6
    assert abs(h[2] / h[3] - (1000.0 / 999.0) * (1.0 - 1.0 / 5.0)) < 1e-6
    assert abs(float(u["bias"][0]) - 0.2 * 2.0 / 200) < 1e-9


def _single(center, rot, scale, sh=None):
    s60 = np.zeros((1, 60), np.float32)
    s60[0, 0:4] = rot
    s60[0, 4:7] = center
    s60[0, 8:11] = scale
    s60[0, 11] = 1.0
    if sh is not None:
        s60[0, 12:12 + len(sh)] = sh
    return scene_from_splats60(s60)


@pytest.mark.parametrize("d", [4.0, 9.0])
def test_on_axis_ellipsoid_contour_closed_form(d):
    # ellipsoid x^2/a^2 + y^2/b^2 + (z-d)^2/c^2 = 1 seen from the origin along +z: silhouette in the view
    # plane z = 1 is u^2/a^2 + v^2/b^2 = 1/(d^2 - c^2) centred at 0 (derived from the tangent condition).
    # The ellipsoid is turned by 20 degrees about the view axis, which turns the silhouette likewise.
    a, b, c = 0.5, 0.2, 0.3
    th = math.radians(20.0)
    q = [math.cos(th / 2), 0.0, 0.0, math.sin(th / 2)]
    cam = camera.look_at([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    u = oracle.uniforms(cam, 640, 480)
    sc = _single([0.0, 0.0, d], q, [a, b, c])
    cfg = oracle.config_struct(use_covariance_for_scale=False, sh_order=0)
    _, dbg, nv = oracle.preprocess(u, cfg, sc, np.array([0], np.uint32), fp64=True)
    t, rot, axes = dbg[0, 9:11], dbg[0, 11:13], dbg[0, 13:15]
    k = 1.0 / math.sqrt(d * d - c * c)
    assert np.allclose(t, 0.0, atol=1e-12)
    assert sorted(np.abs(axes)) == pytest.approx(sorted([a * k, b * k]), rel=1e-6)  # f32 inputs
    assert abs(np.hypot(*rot) - 1.0) < 1e-9
    # the semi-axis along (k, -j) is the first one; it lies along the ellipsoid's turned x or y axis
    ang = math.atan2(-rot[0], rot[1])
    assert min(abs(math.sin(ang - th)), abs(math.cos(ang - th))) < 1e-6
    # covariance mode: Jacobian-projected covariance at the centre gives a/d, b/d
    cfg = oracle.config_struct(use_covariance_for_scale=True, sh_order=0)
    _, dbg, _ = oracle.preprocess(u, cfg, sc, np.array([0], np.uint32), fp64=True)
    assert sorted(dbg[0, 13:15]) == pytest.approx(sorted([b / d, a / d]), rel=1e-6)


def test_axis_aligned_conic_collapses_like_the_reference():
    # extractRotationOfEllipse multiplies by sign(M.x.y) (shaders.wgsl:204): an ellipse whose conic has
    # M.x.y == 0 exactly gets rotation (0, 0), a zero-size rectangle, and is never drawn.
    cam = camera.look_at([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    u = oracle.uniforms(cam, 640, 480)
    sc = _single([0.0, 0.0, 4.0], [1.0, 0.0, 0.0, 0.0], [0.5, 0.2, 0.3])
    for fp64 in (False, True):
        rec, dbg, nv = oracle.preprocess(u, oracle.config_struct(sh_order=0), sc, np.array([0], np.uint32),
                                         fp64=fp64)
        assert nv == 0
        assert list(dbg[0, 11:13]) == [0.0, 0.0]


def test_off_axis_sphere_silhouette_is_tangent_cone():
    # A (slightly anisotropic, to keep the rotation defined) sphere off the optical axis: every point of
    # the extracted ellipse must lie on the tangent cone from the camera (angle asin(r/D) to the centre).
    r = 0.3
    center = np.array([1.5, -0.7, 6.0])
    cam = camera.look_at([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    u = oracle.uniforms(cam, 640, 480)
    sc = _single(center, [1.0, 0.0, 0.0, 0.0], [r, r * (1 + 1e-6), r])
    cfg = oracle.config_struct(use_covariance_for_scale=False, sh_order=0)
    _, dbg, _ = oracle.preprocess(u, cfg, sc, np.array([0], np.uint32), fp64=True)
    t, (j, kk), (sa, sb) = dbg[0, 9:11], dbg[0, 11:13], dbg[0, 13:15]
    major = np.array([kk, -j])
    minor = np.array([j, kk])
    D = np.linalg.norm(center)
    alpha = math.asin(r / D)
    for th in np.linspace(0, 2 * math.pi, 64, endpoint=False):
        p2 = t + math.cos(th) * sa * major + math.sin(th) * sb * minor
        p = np.array([p2[0], p2[1], 1.0])
        ang = math.acos(np.dot(p, center) / (np.linalg.norm(p) * D))
        assert abs(ang - alpha) < 1e-6


def test_sh_band0_and_direction_terms():
    sh = np.zeros(48, np.float32)
    sh[0:3] = (1.0, -0.5, 0.25)
    sh[3:6] = (0.5, 0.0, 0.0)  # band 1, coefficient 1 (times y)
    cam = camera.look_at([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    u = oracle.uniforms(cam, 64, 64)
    center = np.array([0.0, 3.0, 4.0])
    sc = _single(center, [1.0, 0.0, 0.0, 0.0], [0.1, 0.2, 0.3], sh)
    cfg = oracle.config_struct(sh_order=1)
    _, dbg, _ = oracle.preprocess(u, cfg, sc, np.array([0], np.uint32), fp64=True)
    dy = 3.0 / 5.0
    c0 = 0.28209479177387814
    assert dbg[0, 15] == pytest.approx(0.5 + c0 * 1.0 - 0.4886025119029199 * 0.5 * dy, abs=1e-12)
    assert dbg[0, 16] == pytest.approx(0.5 - c0 * 0.5, abs=1e-12)
    assert dbg[0, 17] == pytest.approx(0.5 + c0 * 0.25, abs=1e-12)


def test_depth_key_layout():
    cam = camera.look_at([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    u = oracle.uniforms(cam, 100, 100)
    pts = np.array([[0.0, 0.0, 10.0], [0.0, 0.0, 0.5], [50.0, 0.0, 10.0], [1.09 * 10, 0, 10]], np.float32)
    keys, vis = oracle.cull_keys(u, 2, pts)
    z = (1000.0 / 999.0) * (1.0 - 1.0 / 10.0)
    assert vis.tolist() == [True, False, False, True]
    assert keys[0] >> 16 == int(np.float32(z) * np.float32(65535.0))
    assert (keys[0] >> 8) & 0xFF == 127 and keys[0] & 0xFF == 127
    assert keys[1] == 0xFFFFFFFF and keys[2] == 0xFFFFFFFF
    # x beyond 1.0 (tolerance 1.1) overflows its byte into bit 16 (shaders.wgsl:323)
    xb = int(np.float32((np.float32(1.09) * np.float32(0.5) + np.float32(0.5)) * np.float32(255.0)))
    assert xb > 255 and (keys[3] >> 8) & 0x1FF == (xb & 0x1FF) | ((keys[3] >> 8) & 0x100)


def test_cpu_rule_and_fallback_sort_stable():
    rng = np.random.default_rng(5)
    pts = rng.normal(0, 2, (5000, 3)).astype(np.float32)
    pts[100] = pts[7]  # exact duplicate -> equal keys, stable order by index
    cam = camera.look_at([0.0, 0.0, -8.0], [0.0, 0.0, 0.0])
    u = oracle.uniforms(cam, 640, 480)
    ent = oracle.cpu_sort_fallback(u, pts)
    keys, vis = oracle.cull_keys(u, 1, pts)
    order = np.argsort(keys[vis], kind="stable")
    assert np.array_equal(ent[:, 1], np.nonzero(vis)[0][order])
    assert np.all(np.diff(ent[:, 0].astype(np.int64)) >= 0)
    i7 = np.where(ent[:, 1] == 7)[0]
    i100 = np.where(ent[:, 1] == 100)[0]
    if len(i7) and len(i100):
        assert i7[0] < i100[0]


def test_load_transform_known_values():
    rec = np.zeros((2, 62), np.float32)
    rec[0, 0:3] = (1, 2, 3)
    rec[0, 6:54] = np.arange(48)
    rec[0, 54] = 0.0
    rec[0, 55:58] = (0.0, np.log(2.0), -20.0)  # avg = (0 + 0.693 - 20)/3; clamp -20 to avg-5
    rec[0, 58:62] = (2.0, 0.0, 0.0, 0.0)
    rec[1, 54] = 3.0
    rec[1, 58:62] = (1.0, 1.0, 1.0, 1.0)
    s = oracle.load_transform(rec)
    assert s["rotation"][0].tolist() == [1.0, 0.0, 0.0, 0.0]
    assert np.allclose(s["rotation"][1], 0.5)
    assert s["alpha"][0] == np.float32(0.5)
    assert s["alpha"][1] == pytest.approx(1 / (1 + math.exp(-3.0)), rel=1e-6)
    avg = (0.0 + math.log(2.0) - 20.0) / 3.0
    # every log-scale is clamped into [avg - 5, avg + 5] (scene.rs:235-247)
    assert s["scale"][0] == pytest.approx([math.exp(avg + 5.0), math.exp(avg + 5.0), math.exp(avg - 5.0)], rel=1e-6)
    assert np.array_equal(s["sh"][0], np.arange(48, dtype=np.float32))


def test_blend_single_splat_unorm8():
    # one splat centred on the centre pixel (tc = 0 there): C = q(clamp(rgb * a)), T = q(1 - a)
    cam = camera.look_at([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    u = oracle.uniforms(cam, 33, 33)
    sh = np.zeros(48, np.float32)
    sh[0:3] = (0.0, 1.0, -5.0)
    th = math.radians(30.0)
    sc = _single([0.0, 0.0, 5.0], [math.cos(th / 2), 0.0, 0.0, math.sin(th / 2)], [1.0, 1.2, 0.5], sh)
    sc["alpha"][:] = 0.8
    img, st = oracle.render(u, oracle.config_struct(sh_order=0), sc)
    assert st == (1, 1, 1)
    px = img[16, 16]
    c0 = np.float32(0.28209479177387814)
    g = np.float32(0.5) + c0 * np.float32(1.0)
    assert px[0] == int(np.rint(np.float32(0.5) * np.float32(0.8) * np.float32(255.0)))
    assert px[1] == int(np.rint(g * np.float32(0.8) * np.float32(255.0)))
    assert px[2] == 0  # negative colour clamps to 0 in the blend unit
    assert px[3] == 51  # q(1 - 0.8)
    assert img[0, 0].tolist() == [0, 0, 0, 255]  # cleared to (0, 0, 0, 1), renderer.rs:441-442


def test_dev_scene_golden():
    """Pins the restatement against the committed golden image of the reference's dev-test scene
    (Scene::new_dev_test, scene.rs:158-192), produced by tests/golden/make_golden.py."""
    path = os.path.join(GOLDEN, "dev_scene.json")
    g = json.load(open(path))
    s60 = synthetic.dev_test_splats60()
    sc = scene_from_splats60(s60)
    for case in g["cases"]:
        cam = np.array(case["camera"], np.float32)
        u = oracle.uniforms(cam, case["width"], case["height"], fovy=case["fovy"])
        cfg = oracle.config_struct(depth_sorting=case["depth_sorting"], sh_order=0,
                                   use_covariance_for_scale=case["covariance"],
                                   use_unaligned_rectangles=case["rect"])
        img, st = oracle.render(u, cfg, sc)
        import hashlib
        assert hashlib.sha256(img.tobytes()).hexdigest() == case["sha256"], case["name"]
        assert list(st) == case["stats"]


@pytest.mark.parametrize("blend", [0, 1])
def test_raster_work_counts(blend):
    """oracle.raster_work (the raster's algorithmic unit) against a per-record sweep over all pixels
    in numpy: pairs inside the pixel boxes, pairs passing the coverage test, and blend steps before
    each pixel finishes (T == 0 in unorm8, T < 1e-4 in fp32)."""
    W, H = 72, 40
    rec = synthetic.plain_small(400, seed=9, sh_order=0)
    rec[:, 55:58] += 1.5  # splats a few pixels wide
    sc = oracle.load_transform(rec)
    cam = camera.look_at([0.4, 0.3, -9.0], [0.0, 0.0, 0.0])
    u = oracle.uniforms(cam, W, H, fovy=math.radians(60))
    cfg = oracle.config_struct(sh_order=0, blend_mode=blend)
    _, idx, _, nd = oracle.draw_list(u, 2, sc["center"])
    recs, _, _ = oracle.preprocess(u, cfg, sc, idx[:nd], threads=2)
    work = oracle.raster_work(u, cfg, recs, threads=3)
    f32, m = np.float32, np.float32(u["margin"][0])
    X = np.arange(W, dtype=f32)[None, :] + f32(0.5)
    Y = np.arange(H, dtype=f32)[:, None] + f32(0.5)
    px, py = np.arange(W)[None, :], np.arange(H)[:, None]
    fma = lambda a, b, c: (np.float64(a) * np.float64(b) + np.float64(c)).astype(f32)
    box = cov = blended = 0
    ta = np.full((H, W), 255, np.int64)
    ft = np.ones((H, W), f32)
    done = np.zeros((H, W), bool)
    lut = np.arange(256, dtype=f32) / f32(255.0)
    for rc in recs.astype(f32):
        lo, hi = int(rc[7:8].view(np.uint32)[0]), int(rc[11:12].view(np.uint32)[0])
        x0, y0, x1, y1 = lo & 0xFFFF, lo >> 16, hi & 0xFFFF, hi >> 16
        inb = (px >= x0) & (px <= x1) & (py >= y0) & (py <= y1)
        tcx = fma(rc[1], Y, fma(rc[0], X, rc[2]))
        tcy = fma(rc[4], Y, fma(rc[3], X, rc[5]))
        c = inb & (np.abs(tcx) <= m) & (np.abs(tcy) <= m)
        box += int(inb.sum())
        cov += int(c.sum())
        live = c & ~done
        for yy, xx in zip(*np.nonzero(live)):
            power = fma(tcx[yy, xx], tcx[yy, xx], tcy[yy, xx] * tcy[yy, xx])
            alpha = f32(rc[6] * f32(oracle.expf(f32(-0.5) * power)))
            if alpha < f32(1.0) / f32(255.0):
                continue
            blended += 1
            sa = np.clip(alpha, f32(0.0), f32(1.0))
            if blend == 0:
                ta[yy, xx] = int(np.rint(np.clip(lut[ta[yy, xx]] * (f32(1.0) - sa), 0, 1) * f32(255.0)))
                done[yy, xx] = ta[yy, xx] == 0
            else:
                ft[yy, xx] = ft[yy, xx] * (f32(1.0) - sa)
                done[yy, xx] = ft[yy, xx] < f32(1e-4)
    assert box > cov > blended > 0
    assert work == {"box": box, "covered": cov, "blended": blended}
