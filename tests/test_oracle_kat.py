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


def _quat_matrix(q):
    # the rotation matrix of the unit quaternion q = (scalar, i, j, k), textbook form
    w, x, y, z = (float(c) for c in q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


KAT_CAMERAS = [([0.0, 0.0, 0.0], [0.0, 0.0, 1.0]), ([1.0, 2.0, -3.0], [0.0, 0.5, 4.0]),
               ([-4.0, 1.5, 2.0], [3.0, -1.0, 1.0])]


def _random_ellipsoids(u, count, seed):
    """Unit-quaternion ellipsoids (scales 0.05-0.6, up to 12:1) in front of the camera, inside the view,
    with their centres, rotations and scales as f32 (what the oracle reads)."""
    rng = np.random.default_rng(seed)
    cam = np.asarray(u["camera"][0], np.float64).reshape(4, 4)  # column-major: rows are the columns
    C, eye = cam[:3, :3].T, cam[3, :3]
    zc = rng.uniform(4.0, 12.0, count)
    local = np.stack([rng.uniform(-0.5, 0.5, count) * zc, rng.uniform(-0.35, 0.35, count) * zc, zc], 1)
    centers = (eye[None, :] + local @ C.T).astype(np.float32)
    q = rng.normal(size=(count, 4))
    q = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    scales = np.exp(rng.uniform(math.log(0.05), math.log(0.6), (count, 3))).astype(np.float32)
    return centers, q, scales, C, eye


def _outline(dbg, theta):
    """Points of the oracle's outline ellipse (view plane z = 1): centre t, semi-axis a0 along
    (k, -j) and a1 along (j, k), rotation (j, k)."""
    t, (j, k), (a0, a1) = dbg[9:11], dbg[11:13], dbg[13:15]
    U, V = np.array([k, -j]), np.array([j, k])
    return t[None, :] + np.cos(theta)[:, None] * a0 * U[None, :] + np.sin(theta)[:, None] * a1 * V[None, :]


@pytest.mark.parametrize("cam_i", range(len(KAT_CAMERAS)))
def test_rotated_ellipsoid_outlines_lie_on_the_tangent_cone(cam_i):
    # General rotated, off-axis ellipsoids seen from three cameras: every point of the extracted outline
    # (extractTranslationOfEllipse, extractRotationOfEllipse with its sign fix-ups, extractScaleOfEllipse;
    # shaders.wgsl:179-237) must lie on the cone of rays from the camera tangent to the ellipsoid.  A ray
    # x = eye + s d meets (x - m)^T Q (x - m) = 1 (Q = R S^-2 R^T) in one point iff
    # (d.Q w)^2 = (d.Q d)(w.Q w - 1), w = eye - m; the view-plane point p is the ray d = C (p, 1).
    # An axis swapped between the two directions, a wrong sign fix-up or a wrong centre puts the sampled
    # points off the cone.
    cam = camera.look_at(*KAT_CAMERAS[cam_i])
    u = oracle.uniforms(cam, 640, 480)
    centers, q, scales, C, eye = _random_ellipsoids(u, 60, seed=100 + cam_i)
    s60 = np.zeros((len(centers), 60), np.float32)
    s60[:, 0:4], s60[:, 4:7], s60[:, 8:11], s60[:, 11] = q, centers, scales, 1.0
    sc = scene_from_splats60(s60)
    cfg = oracle.config_struct(use_covariance_for_scale=False, sh_order=0)
    _, dbg, nv = oracle.preprocess(u, cfg, sc, np.arange(len(centers), dtype=np.uint32), fp64=True)
    assert nv == len(centers)
    theta = np.linspace(0.0, 2.0 * math.pi, 48, endpoint=False)
    worst = 0.0
    for i in range(len(centers)):
        R = _quat_matrix(q[i].astype(np.float64))
        Q = R @ np.diag(1.0 / scales[i].astype(np.float64) ** 2) @ R.T
        w = eye - centers[i].astype(np.float64)
        wqw = w @ Q @ w - 1.0
        assert wqw > 0.0  # the camera is outside the ellipsoid
        p = _outline(dbg[i], theta)
        d = np.concatenate([p, np.ones((len(theta), 1))], 1) @ C.T
        dqd = np.einsum("ni,ij,nj->n", d, Q, d)
        dqw = d @ Q @ w
        worst = max(worst, float(np.max(np.abs(dqw * dqw - dqd * wqw) / (dqd * wqw))))
    assert worst < 1e-9


@pytest.mark.parametrize("rect", [True, False], ids=["rect", "square"])
def test_texture_coordinates_of_the_outline_closed_form(rect):
    # The record's affine map tc = A (X, Y) + B at pixel position (X, Y) is the inverse of the quad basis
    # [X Y] = [(k, -j)(bias + a0), (j, k)(bias + a1)] applied to the view-plane offset from the centre
    # (shaders.wgsl:543-571: the rectangle maps its corners, the axis-aligned square applies `inverse` to
    # its corner offsets; both interpolate affinely).  So a point of the outline at angle theta has
    # tc = (a0 cos theta / (bias + a0), a1 sin theta / (bias + a1)), with the pixel position
    # X = (p_x + vw) W / (2 vw), Y = (vh - p_y) H / (2 vh).  The square's half-size is
    # margin * max(bias + a0, bias + a1) and its offsets (bx, by) = (-vw - t_x, vh - t_y)
    # (shaders.wgsl:567-570); the rectangle's pixel box spans margin * (|X_x| + |Y_x|) horizontally.
    cam = camera.look_at(*KAT_CAMERAS[1])
    W, H = 640, 480
    u = oracle.uniforms(cam, W, H)
    centers, q, scales, C, eye = _random_ellipsoids(u, 40, seed=7)
    s60 = np.zeros((len(centers), 60), np.float32)
    s60[:, 0:4], s60[:, 4:7], s60[:, 8:11], s60[:, 11] = q, centers, scales * 4.0, 1.0
    sc = scene_from_splats60(s60)
    cfg = oracle.config_struct(use_covariance_for_scale=False, use_unaligned_rectangles=rect, sh_order=0)
    rec, dbg, nv = oracle.preprocess(u, cfg, sc, np.arange(len(centers), dtype=np.uint32), fp64=True)
    vw, vh = (float(x) for x in u["view_size"][0])
    bias, margin = float(u["bias"][0]), float(u["margin"][0])
    theta = np.linspace(0.0, 2.0 * math.pi, 36, endpoint=False)
    checked = 0
    for i in range(len(centers)):
        t, (j, k), (a0, a1) = dbg[i, 9:11], dbg[i, 11:13], dbg[i, 13:15]
        p = _outline(dbg[i], theta)
        X = (p[:, 0] + vw) * W / (2.0 * vw)
        Y = (vh - p[:, 1]) * H / (2.0 * vh)
        r = rec[i].astype(np.float64)
        tc = np.stack([r[0] * X + r[1] * Y + r[2], r[3] * X + r[4] * Y + r[5]], 1)
        want = np.stack([a0 * np.cos(theta) / (bias + a0), a1 * np.sin(theta) / (bias + a1)], 1)
        assert np.max(np.abs(tc - want)) < 1e-4
        if rect:
            assert r[12] == 0.0 and r[13] == 0.0 and r[14] == 0.0
            ex = margin * (abs(k * (bias + a0)) + abs(j * (bias + a1)))
        else:
            assert r[14] == pytest.approx(margin * max(bias + a0, bias + a1), rel=1e-6)
            assert r[12] == pytest.approx(-vw - t[0], rel=1e-6, abs=1e-7)
            assert r[13] == pytest.approx(vh - t[1], rel=1e-6, abs=1e-7)
            ex = float(r[14])
        lo, hi = rec[i, 7:8].view(np.uint32)[0], rec[i, 11:12].view(np.uint32)[0]
        if lo == 0xFFFFFFFF:
            continue  # entirely outside the image
        checked += 1
        x0, x1 = int(lo & 0xFFFF), int(hi & 0xFFFF)
        cxp, exp_ = (t[0] + vw) * W / (2.0 * vw), ex * W / (2.0 * vw)
        # pixel centres x + 0.5 in [cxp - exp_, cxp + exp_] (to 1/64 px), clamped to the image
        assert x0 == max(0, math.ceil(cxp - exp_ - 0.5 - 1.0 / 64)) or x0 == max(0, math.ceil(cxp - exp_ - 0.5))
        assert x1 == min(W - 1, math.floor(cxp + exp_ - 0.5 + 1.0 / 64)) or x1 == min(W - 1, math.floor(cxp + exp_ - 0.5))
        # the outline (margin 2 > 1) lies inside the box
        inside = (X >= x0) & (X <= x1 + 1)
        assert inside[(X >= 0) & (X <= W)].all()
    assert checked >= 30


def test_covariance_semi_axes_closed_form():
    # use_covariance_for_scale: the semi-axes are the square roots of the eigenvalues of the 2x2 covariance
    # J (C^T Sigma C) J^T, Sigma = R S^2 R^T, J the perspective Jacobian at the centre's camera coordinates
    # v = view (m, 1) (with v_x / v_z and v_y / v_z clamped to [-1, 1]) (shaders.wgsl:99-118, 240-246).
    cam = camera.look_at(*KAT_CAMERAS[2])
    u = oracle.uniforms(cam, 640, 480)
    centers, q, scales, C, eye = _random_ellipsoids(u, 60, seed=11)
    s60 = np.zeros((len(centers), 60), np.float32)
    s60[:, 0:4], s60[:, 4:7], s60[:, 8:11], s60[:, 11] = q, centers, scales, 1.0
    sc = scene_from_splats60(s60)
    cfg = oracle.config_struct(use_covariance_for_scale=True, sh_order=0)
    _, dbg, _ = oracle.preprocess(u, cfg, sc, np.arange(len(centers), dtype=np.uint32), fp64=True)
    view = np.asarray(u["view"][0], np.float64).reshape(4, 4).T  # the f32 view matrix, row-major
    assert np.allclose(view[:3, :3], C.T, atol=1e-6)  # the camera's inverse
    for i in range(len(centers)):
        R = _quat_matrix(q[i].astype(np.float64))
        sigma = R @ np.diag(scales[i].astype(np.float64) ** 2) @ R.T
        v = view[:3, :3] @ centers[i].astype(np.float64) + view[:3, 3]
        vx, vy = np.clip(v[0] / v[2], -1, 1) * v[2], np.clip(v[1] / v[2], -1, 1) * v[2]
        J = np.array([[1 / v[2], 0.0, -vx / v[2] ** 2], [0.0, 1 / v[2], -vy / v[2] ** 2]])
        P = J @ (C.T @ sigma @ C) @ J.T
        want = np.sqrt(np.sort(np.linalg.eigvalsh(P))[::-1])
        assert dbg[i, 13:15] == pytest.approx(want, rel=1e-9)


def test_sh_basis_is_orthonormal_on_the_sphere():
    # sphericalHarmonicsLookup (shaders.wgsl:249-294): rgb = 0.5 + sum_k B_k(d) sh[3k + c] with B_k the
    # real spherical harmonics of degree <= 3 scaled by the 16 constants of the `shc` table.  With the
    # standard normalisation they are orthonormal on the unit sphere: the Gram matrix of the oracle's
    # B_k (read from its FP64 colour with one coefficient set at a time, for splats in every direction
    # around the camera) over a Fibonacci sphere of 20,000 directions is the identity to quadrature
    # error.  This pins every constant and polynomial of the table (not their signs, which the
    # direction-term test below pins for band 1).
    m = 20000
    i = np.arange(m) + 0.5
    z = 1.0 - 2.0 * i / m
    phi = math.pi * (1.0 + math.sqrt(5.0)) * i
    d = np.stack([np.sqrt(1.0 - z * z) * np.cos(phi), np.sqrt(1.0 - z * z) * np.sin(phi), z], 1)
    cam = camera.look_at([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    u = oracle.uniforms(cam, 64, 64)
    cfg = oracle.config_struct(sh_order=3)
    s60 = np.zeros((m, 60), np.float32)
    s60[:, 0] = 1.0
    s60[:, 4:7] = (5.0 * d).astype(np.float32)
    s60[:, 8:11] = 0.1
    s60[:, 11] = 1.0
    B = np.zeros((m, 16))
    for k in range(16):
        s60[:, 12:60] = 0.0
        s60[:, 12 + 3 * k] = 1.0
        _, dbg, _ = oracle.preprocess(u, cfg, scene_from_splats60(s60), np.arange(m, dtype=np.uint32), fp64=True)
        B[:, k] = dbg[:, 15] - 0.5
    gram = (B.T @ B) * (4.0 * math.pi / m)
    assert np.max(np.abs(gram - np.eye(16))) < 1e-4  # measured 3.8e-6; a constant off by 0.01% gives 2e-4
    assert abs(B[0, 0] - 0.28209479177387814) < 1e-9  # band 0 is the constant 1 / (2 sqrt(pi))


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


@pytest.mark.parametrize("mode", [1, 2], ids=["cpu-rule", "gpu-rule"])
def test_frustum_boundaries(mode):
    # isInFrustum (shaders.wgsl:54-61; renderer.rs:381-387 for the CPU rule): visible iff |x| < tol,
    # |y| < tol and |z - 0.5| < 0.5 in normalised device coordinates.  A 90-degree square view from the
    # origin along +z maps (x, y, z) to (x / z, y / z) and depth (1000/999)(1 - 1/z): the near plane is
    # view z = 1 and the far plane z = 1000.  Points 1e-4 (relative) inside and outside every bound.
    cam = camera.look_at([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    u = oracle.uniforms(cam, 100, 100, tol=1.1)
    e = 1e-4
    cases = [((11 * (1 - e), 0, 10), True), ((11 * (1 + e), 0, 10), False),
             ((-11 * (1 - e), 0, 10), True), ((-11 * (1 + e), 0, 10), False),
             ((0, 11 * (1 - e), 10), True), ((0, 11 * (1 + e), 10), False),
             ((0, -11 * (1 - e), 10), True), ((0, -11 * (1 + e), 10), False),
             ((0, 0, 1 + 1e-3), True), ((0, 0, 1 - 1e-3), False),
             ((0, 0, 999), True), ((0, 0, 1001), False), ((0, 0, -5), False), ((0, 0, 0), False)]
    pts = np.array([c[0] for c in cases], np.float32)
    _, vis = oracle.cull_keys(u, mode, pts)
    assert vis.tolist() == [c[1] for c in cases]


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


@pytest.mark.parametrize("depth_sorting", [0, 1, 2, 3], ids=["none", "cpu", "gpu", "gpu-indirect"])
@pytest.mark.parametrize("blend_mode", [0, 1], ids=["unorm8", "fp32"])
def test_blend_two_splats_order_and_equation(depth_sorting, blend_mode):
    # Two splats centred on the centre pixel (tc = 0 there, so each contributes its full alpha): the far
    # one has index 0, the near one index 1.  The blend state (renderer.rs:260-270) is
    #   C' = src_rgb * dst_a + C,   A' = A * (1 - src_a),   cleared to (0, 0, 0, 1) (renderer.rs:442),
    # with the fragment's (rgb * alpha, alpha) clamped to [0, 1].  For the 8-bit target the blend runs
    # in f32 against the stored k / 255 and each result is rounded to the nearest k (ties to even: with
    # alpha 0.7f the transmittance (1 - 0.7f) * 255 is 76.5 in f32 and stores 76).  A sorted mode draws
    # near to far; DepthSorting::None draws in index order (renderer.rs:14-22), here far first.
    cam = camera.look_at([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    u = oracle.uniforms(cam, 33, 33)
    th = math.radians(30.0)
    q = [math.cos(th / 2), 0.0, 0.0, math.sin(th / 2)]
    s60 = np.zeros((2, 60), np.float32)
    s60[:, 0:4] = q
    s60[0, 4:7], s60[1, 4:7] = [0.0, 0.0, 7.0], [0.0, 0.0, 4.0]
    s60[:, 8:11] = [1.0, 1.2, 0.5]
    s60[0, 11], s60[1, 11] = 0.7, 0.6
    s60[0, 12:15], s60[1, 12:15] = [0.3, 0.8, -1.0], [1.0, -0.5, 0.2]
    sc = scene_from_splats60(s60)
    img, st = oracle.render(u, oracle.config_struct(depth_sorting=depth_sorting, sh_order=0,
                                                    blend_mode=blend_mode), sc)
    c0 = np.float32(0.28209479177387814)
    rgb = [np.float32(0.5) + c0 * s60[i, 12:15] for i in range(2)]
    order = [0, 1] if depth_sorting == 0 else [1, 0]
    f, one, k255 = np.float32, np.float32(1.0), np.float32(255.0)
    C, A = np.zeros(3, np.float32), one
    for i in order:
        a = s60[i, 11]
        src = np.clip(rgb[i] * a, f(0), one)
        if blend_mode == 0:  # stored as k / 255
            C = np.rint(np.clip(src * A + C, f(0), one) * k255) / k255
            A = np.rint(np.clip(A * (one - a), f(0), one) * k255) / k255
        else:
            C, A = src * A + C, A * (one - a)
    px = img[16, 16]
    if blend_mode == 0:
        assert px.tolist() == [int(x) for x in np.rint(np.append(C, A) * k255)]
    else:
        assert np.allclose(px, list(C) + [A], rtol=0, atol=1e-6)
    assert st[2] == 2  # both drawn


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
