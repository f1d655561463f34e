"""GPU parity tests: the CUDA path (through the C ABI) against the oracle on the same seeded inputs.

Bar: bit-exact depth keys, visible set, sorted permutation, per-splat records and images (FP32 math
with the WGSL operation order on both sides, and a shared exp method), in every depth-sorting mode,
both rectangle kinds, both semi-axis methods and both blend targets.
"""
import hashlib
import json
import math
import os

import numpy as np
import pytest

import oracle
from splatter_gb300 import BlendMode, Configuration, DepthSorting, Renderer, Scene, SplatterError, camera, synthetic
from splatter_gb300 import _lib
from tests.helpers import default_cam, image_psnr, oracle_cfg, oracle_uniforms

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 8
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def gpu_frame(cuda, config, records, cam, w, h, splats60=None):
    import torch
    r = Renderer(config)
    n = records.shape[0] if records is not None else splats60.shape[0]
    s = Scene(r, n)
    if records is not None:
        s.load_chunk(records)
    else:
        s.write_splats(splats60)
    img = r.render_frame(s, cam, w, h)
    torch.cuda.synchronize()
    keys, idx, info = r.sorted_entries()
    recs = r.records()
    torch.cuda.synchronize()
    out = (img.cpu().numpy(), keys.cpu().numpy().view(np.uint32), idx.cpu().numpy().view(np.uint32), info,
           recs.cpu().numpy(), s.read_splats())
    s.close()
    r.close()
    return out


def oracle_frame(config, sc, cam, w, h):
    u = oracle_uniforms(oracle, config, cam, w, h)
    cfg = oracle_cfg(oracle, config)
    keys, idx, v, nd = oracle.draw_list(u, int(config.depth_sorting), sc["center"])
    img, st = oracle.render(u, cfg, sc, threads=THREADS)
    vis_sorted = np.sort(idx)
    recs, _, _ = oracle.preprocess(u, cfg, sc, vis_sorted, threads=THREADS)
    return img, keys, idx, v, nd, recs


def assert_frame_parity(g, o, config):
    img, keys, idx, info, recs, _ = g
    oimg, okeys, oidx, v, nd, orecs = o
    assert info.visible_count == v
    assert info.draw_count == nd
    assert np.array_equal(keys, okeys)
    assert np.array_equal(idx, oidx)
    # bit-exact records; NaN only at the same places (IEEE arithmetic leaves NaN payloads to the
    # implementation: the GPU's default NaN is 0x7fffffff, the CPU's 0x7fc00000)
    gnan, onan = np.isnan(recs), np.isnan(orecs)
    assert np.array_equal(gnan, onan)
    assert np.array_equal(np.where(gnan, 0.0, recs).astype(np.float32).view(np.uint32),
                          np.where(onan, 0.0, orecs).astype(np.float32).view(np.uint32))
    if config.blend_mode == BlendMode.UNORM8:
        assert np.array_equal(img, oimg), f"max |diff| {np.abs(img.astype(int) - oimg.astype(int)).max()}"
    else:
        assert np.array_equal(img.view(np.uint32), oimg.view(np.uint32))


def test_loader_bit_exact(cuda):
    rec = synthetic.plain_small(5000, seed=11, sh_order=3)
    rec[17, 55:58] = (3.0, -30.0, 0.0)  # exercises the clamp around the mean log-scale
    rec[18, 54] = 120.0  # sigmoid saturates
    r = Renderer(Configuration(max_splat_count=5000))
    s = Scene(r, 5000)
    s.load_chunk(rec)
    got = s.read_splats()
    ref = oracle.load_transform(rec)
    exp60 = synthetic.records_to_splats60(ref["center"], ref["rotation"], ref["scale"], ref["alpha"], ref["sh"])
    assert np.array_equal(got.view(np.uint32), exp60.view(np.uint32))


def test_progressive_chunks_equal_single_load(cuda):
    rec = synthetic.plain_small(70000, seed=12, sh_order=1)
    r = Renderer(Configuration(max_splat_count=70000))
    a = Scene(r, 70000)
    a.load_chunk(rec)
    b = Scene(r, 70000)
    chunk = 16384
    for c in reversed(range((70000 + chunk - 1) // chunk)):  # showcase.rs:98-103 loads in reverse order
        b.load_chunk(rec[c * chunk:(c + 1) * chunk], start=c * chunk)
    assert np.array_equal(a.read_splats(), b.read_splats())


def test_load_chunk_file(cuda, tmp_path):
    rec = synthetic.plain_small(3000, seed=13, sh_order=2)
    header = ("ply\nformat binary_little_endian 1.0\nelement vertex 3000\n" +
              "".join(f"property float f{i}\n" for i in range(62)) + "end_header\n").encode()
    p = tmp_path / "scene.ply"
    p.write_bytes(header + rec.tobytes())
    hb, n = Scene.parse_file_header(p)
    r = Renderer(Configuration(max_splat_count=n))
    s = Scene(r, n)
    s.load_chunk_file(p, hb, 1000, 2000)
    s.load_chunk_file(p, hb, 0, 1000)
    t = Scene(r, n)
    t.load_chunk(rec)
    assert np.array_equal(s.read_splats(), t.read_splats())


def test_progressive_loading_frames(cuda, tmp_path):
    """The viewer's progressive loading (showcase.rs:54-59,98-103) from a validated file: after each
    step the frame equals the oracle's frame of the scene with only the loaded chunks set (the others
    zero, as in a fresh scene), and the last one equals the frame of the fully loaded scene."""
    from splatter_gb300 import ProgressiveLoader
    n, chunk, W, H = 60000, 16384, 320, 240
    rec = synthetic.clustered(n, seed=21, sh_order=3)
    p = tmp_path / "scene.ply"
    hb = synthetic.write_ply(p, rec)
    config = Configuration(max_splat_count=n, spherical_harmonics_order=3)
    r = Renderer(config)
    s, hb2 = Scene.open_file(r, p)
    assert hb2 == hb and s.splat_count == n
    loader = ProgressiveLoader(s, p, hb, chunk)
    assert loader.chunks_left == 4
    full = oracle.load_transform(rec)
    part = {k: np.zeros_like(v) for k, v in full.items()}
    cam = camera.look_at([4.0, 3.0, -34.0], [0.0, 0.0, 0.0])
    u = oracle_uniforms(oracle, config, cam, W, H)
    ocfg = oracle_cfg(oracle, config)
    drawn = []
    while loader.chunks_left:
        left = loader.step()
        lo, hi = left * chunk, min((left + 1) * chunk, n)  # the last chunk not yet loaded
        for k in part:
            part[k][lo:hi] = full[k][lo:hi]
        img = r.render_frame(s, cam, W, H).cpu().numpy()
        oimg, _ = oracle.render(u, ocfg, part, threads=THREADS)
        assert np.array_equal(img, oimg)
        drawn.append(int((img[..., 3] != 255).sum()))
    assert drawn[0] > 0 and drawn[-1] > drawn[0]  # the picture fills in
    assert loader.step() == 0  # nothing left: a no-op
    t = Scene(r, n)
    t.load_chunk(rec)
    assert np.array_equal(r.render_frame(t, cam, W, H).cpu().numpy(), img)
    loader.close()


@pytest.mark.parametrize("chunk", [0, 7000, 50000])
def test_progressive_loader_edge_cases(cuda, tmp_path, chunk):
    """chunk 0 (everything in the first step), a chunk that does not divide the count, a chunk above
    the count; and a file larger than max_splat_count (the scene clamps, scene.rs:46): every step
    count and the final scene equal a whole load of the same (clamped) range."""
    from splatter_gb300 import ProgressiveLoader
    n_file, n_max = 23000, 20000
    rec = synthetic.plain_small(n_file, seed=41, sh_order=3)
    p = tmp_path / "s.ply"
    hb = synthetic.write_ply(p, rec)
    r = Renderer(Configuration(max_splat_count=n_max, spherical_harmonics_order=3))
    s, hb2 = Scene.open_file(r, p)
    assert hb2 == hb and s.splat_count == n_max
    loader = ProgressiveLoader(s, p, hb, chunk)
    want_steps = 1 if chunk == 0 else -(-n_max // chunk)
    assert loader.chunks_left == want_steps
    steps = 0
    while loader.chunks_left:
        loader.step()
        steps += 1
    assert steps == want_steps and loader.step() == 0
    t = Scene(r, n_max)
    t.load_chunk(rec[:n_max])
    assert np.array_equal(s.read_splats(), t.read_splats())
    loader.close()


def test_render_frame_motor(cuda):
    """The reference's camera argument (a PGA motor, renderer.rs:355-364): the frame equals the frame
    of its motor3d_to_mat4 matrix and the oracle's frame of that camera."""
    from splatter_gb300.camera import Motor
    n, W, H = 20000, 256, 192
    rec = synthetic.clustered(n, seed=31, sh_order=3)
    config = Configuration(max_splat_count=n, spherical_harmonics_order=3)
    r = Renderer(config)
    s = Scene(r, n)
    s.load_chunk(rec)
    m = Motor.from_rotor_translation(Motor.rotate_around_axis(0.3, (0.0, 1.0, 0.0)), (-9.0, 1.0, -28.0))
    img = r.render_frame_motor(s, m, W, H).cpu().numpy()
    assert np.array_equal(img, r.render_frame(s, m.matrix(), W, H).cpu().numpy())
    oimg, _ = oracle.render(oracle_uniforms(oracle, config, m.matrix(), W, H), oracle_cfg(oracle, config),
                            oracle.load_transform(rec), threads=THREADS)
    assert np.array_equal(img, oimg)
    assert int((img[..., 3] != 255).sum()) > 100


def test_dev_scene_matches_golden(cuda):
    import torch
    g = json.load(open(os.path.join(GOLDEN, "dev_scene.json")))
    for case in g["cases"]:
        cfg = Configuration(depth_sorting=DepthSorting(case["depth_sorting"]), spherical_harmonics_order=0,
                            use_covariance_for_scale=case["covariance"], use_unaligned_rectangles=case["rect"],
                            field_of_view_y=case["fovy"], max_splat_count=16)
        r = Renderer(cfg)
        s = Scene.new_dev_test(r)
        img = r.render_frame(s, np.array(case["camera"], np.float32), case["width"], case["height"])
        torch.cuda.synchronize()
        assert hashlib.sha256(img.cpu().numpy().tobytes()).hexdigest() == case["sha256"], case["name"]


MODES = [
    dict(depth_sorting=DepthSorting.GPU),
    dict(depth_sorting=DepthSorting.GPU_INDIRECT_DRAW),
    dict(depth_sorting=DepthSorting.CPU),
    dict(depth_sorting=DepthSorting.NONE),
    dict(depth_sorting=DepthSorting.GPU, use_unaligned_rectangles=False),
    dict(depth_sorting=DepthSorting.GPU, use_covariance_for_scale=False),
    dict(depth_sorting=DepthSorting.GPU, blend_mode=BlendMode.FP32),
    dict(depth_sorting=DepthSorting.GPU, spherical_harmonics_order=1, splat_scale=1.7, ellipse_margin=3.0),
    dict(depth_sorting=DepthSorting.GPU, spherical_harmonics_order=2, frustum_culling_tolerance=1.3,
         field_of_view_y=math.radians(40)),
]


@pytest.mark.parametrize("mode", MODES, ids=lambda m: "-".join(f"{k}={v}" for k, v in m.items()))
def test_frame_parity_modes(cuda, mode):
    n = 30000
    kw = dict(spherical_harmonics_order=3, max_splat_count=n, field_of_view_y=math.radians(60))
    kw.update(mode)
    config = Configuration(**kw)
    rec = synthetic.plain_small(n, seed=21, sh_order=3)
    cam = default_cam(dist=7.0)
    w, h = 320, 240
    g = gpu_frame(cuda, config, rec, cam, w, h)
    sc = oracle.load_transform(rec)
    o = oracle_frame(config, sc, cam, w, h)
    assert g[3].visible_count > 1000
    assert_frame_parity(g, o, config)


def test_nonfinite_and_degenerate_inputs(cuda):
    """NaN and infinite positions, infinite log-scales, zero quaternions, extreme opacity logits and
    zero scales among ordinary splats: the same keys, visible set, records and image as the oracle
    (non-finite primitives are dropped, as the hardware drops NaN primitives), and no device error."""
    n = 20000
    config = Configuration(spherical_harmonics_order=3, max_splat_count=n, field_of_view_y=math.radians(60))
    rec = synthetic.plain_small(n, seed=41, sh_order=3)
    rec[:, 55:58] += 1.0
    rec[0::97, 0] = np.nan
    rec[1::97, 1] = np.inf
    rec[2::97, 2] = -np.inf
    rec[3::97, 55] = np.inf
    rec[4::97, 58:62] = 0.0
    rec[5::97, 54] = 1e30
    rec[6::97, 54] = -1e30
    rec[7::97, 55:58] = -1e30
    rec[8::97, 6:54] = np.nan
    cam = default_cam(dist=7.0)
    g = gpu_frame(cuda, config, rec, cam, 320, 240)
    o = oracle_frame(config, oracle.load_transform(rec), cam, 320, 240)
    assert g[3].device_error == 0
    assert g[3].visible_count > 1000
    assert_frame_parity(g, o, config)


@pytest.mark.parametrize("covariance", [True, False], ids=["covariance", "ellipse"])
def test_camera_inside_and_screen_filling_splats(cuda, covariance):
    """Splats whose ellipsoid contains the camera (the bounding cone of shaders.wgsl:125-169 has no
    real silhouette then), splats just beyond the near plane (view z = 1) that cover the whole
    viewport (boxes clamped to the image, every tile binned), and splats whose centre sits at the near
    plane, among ordinary ones: the same keys, visible set, records and image as the oracle, and no
    device error."""
    n = 20000
    config = Configuration(spherical_harmonics_order=3, max_splat_count=n, field_of_view_y=math.radians(60),
                           use_covariance_for_scale=covariance)
    rec = synthetic.plain_small(n, seed=43, sh_order=3)
    rec[:, 55:58] += 1.0
    eye = np.array([0.3, 0.5, -7.0], np.float32)
    cam = camera.look_at(eye, [0.0, 0.0, 0.0])
    fwd = -eye / np.linalg.norm(eye)
    rng = np.random.default_rng(44)
    k = np.arange(0, n, 211)  # ~95 special splats
    for j, i in enumerate(k):
        kind = j % 3
        if kind == 0:    # the camera inside: centre 1.2-1.5 ahead, radii ~e^1.5 = 4.5
            rec[i, 0:3] = eye + fwd * float(rng.uniform(1.2, 1.5)) + rng.normal(0.0, 0.05, 3).astype(np.float32)
            rec[i, 55:58] = 1.5 + rng.normal(0.0, 0.2, 3).astype(np.float32)
        elif kind == 1:  # just beyond the near plane, filling the view
            rec[i, 0:3] = eye + fwd * float(rng.uniform(1.1, 2.0)) + rng.normal(0.0, 0.05, 3).astype(np.float32)
            rec[i, 55:58] = rng.uniform(-1.0, 0.5, 3).astype(np.float32)
        else:            # centre at the near plane
            rec[i, 0:3] = eye + fwd * float(rng.uniform(0.95, 1.05)) + rng.normal(0.0, 0.2, 3).astype(np.float32)
            rec[i, 55:58] = rng.uniform(-1.0, 0.5, 3).astype(np.float32)
        rec[i, 54] = -2.0  # low opacity, so that the scene behind stays visible
    g = gpu_frame(cuda, config, rec, cam, 320, 240)
    o = oracle_frame(config, oracle.load_transform(rec), cam, 320, 240)
    assert g[3].device_error == 0
    assert g[3].visible_count > 1000
    assert_frame_parity(g, o, config)


@pytest.mark.parametrize("w,h", [(1, 1), (17, 9), (1000, 3), (3, 700), (257, 255), (4112, 4112)])
def test_viewports(cuda, w, h):
    """Viewports that are not multiples of the 16-pixel tile, degenerate strips, one pixel, and one
    with more than 65536 tiles (a 3-pass tile-id sort; up to 256 tiles take 1 pass)."""
    n = 20000
    config = Configuration(spherical_harmonics_order=3, max_splat_count=n, field_of_view_y=math.radians(60),
                           max_pair_count=1 << 23)
    rec = synthetic.plain_small(n, seed=31, sh_order=3)
    rec[:, 55:58] += 1.0
    cam = default_cam(dist=7.0)
    g = gpu_frame(cuda, config, rec, cam, w, h)
    o = oracle_frame(config, oracle.load_transform(rec), cam, w, h)
    assert_frame_parity(g, o, config)
    if w * h > 1000:
        assert g[3].pair_count > 0


@pytest.mark.parametrize("n", [0, 1, 2, 31, 1023, 1024, 1025, 4095, 4096, 4097, 8191, 12289])
def test_tile_boundaries(cuda, n):
    config = Configuration(spherical_harmonics_order=1, max_splat_count=max(n, 1), field_of_view_y=math.radians(60))
    rec = synthetic.plain_small(max(n, 1), seed=100 + n, sh_order=1)[:n]
    cam = default_cam(dist=6.0)
    g = gpu_frame(cuda, config, rec, cam, 200, 150)
    o = oracle_frame(config, oracle.load_transform(rec), cam, 200, 150)
    assert_frame_parity(g, o, config)


def test_everything_culled(cuda):
    config = Configuration(spherical_harmonics_order=0, max_splat_count=5000)
    rec = synthetic.plain_small(5000, seed=3)
    cam = camera.look_at([0.0, 0.0, -50.0], [0.0, 0.0, -100.0])  # looking away from the blob
    img, keys, idx, info, _, _ = gpu_frame(cuda, config, rec, cam, 64, 48)
    assert info.visible_count == 0 and info.draw_count == 0 and info.pair_count == 0
    assert (img == np.array([0, 0, 0, 255], np.uint8)).all()


def test_duplicate_positions_keep_index_order(cuda):
    # equal keys must come out in splat-index order (the stable order of the CPU fallback's sort_by)
    rec = synthetic.plain_small(20000, seed=31)
    rec[:, 0:3] = np.round(rec[:, 0:3] * 2) / 2  # many exact duplicates
    config = Configuration(max_splat_count=20000, spherical_harmonics_order=0)
    cam = default_cam(dist=9.0)
    g = gpu_frame(cuda, config, rec, cam, 256, 256)
    o = oracle_frame(config, oracle.load_transform(rec), cam, 256, 256)
    assert_frame_parity(g, o, config)
    keys = g[1]
    assert np.any(keys[1:] == keys[:-1])


@pytest.mark.parametrize("n,bits,distinct", [(1, 32, 1), (100, 8, 3), (4095, 16, 50), (4096, 32, 7),
                                             (4097, 24, 1000), (100000, 32, 10), (1 << 20, 32, 1 << 30),
                                             (777777, 16, 300)])
def test_sort_pairs_stable(cuda, n, bits, distinct):
    import torch
    rng = np.random.default_rng(n + bits)
    keys = (rng.integers(0, distinct, n, dtype=np.int64) * 2654435761 % (1 << 32)).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    r = Renderer(Configuration(max_splat_count=max(n, 1)))
    kd = torch.from_numpy(keys.view(np.int32)).cuda()
    vd = torch.from_numpy(vals.view(np.int32)).cuda()
    ko, vo = r.sort_pairs(kd, vd, key_bits=bits)
    torch.cuda.synchronize()
    mask = np.uint32((1 << bits) - 1) if bits < 32 else np.uint32(0xFFFFFFFF)
    order = np.argsort(keys & mask, kind="stable")
    assert np.array_equal(vo.cpu().numpy().view(np.uint32), vals[order])
    assert np.array_equal(ko.cpu().numpy().view(np.uint32), keys[order])


def test_small_frame_sorts_take_microseconds(cuda):
    """A 2k-splat frame: both cooperative sorts have grids sized for the renderer's capacity (the
    pair sort for >= 2^20 pairs) but read the live count on the device, and only the CTAs it needs
    take part in their grid barriers.  Median over 20 frames by CUDA events: each sort < 20 us; the
    frame stays bit-exact against the oracle."""
    import torch
    n = 2048
    config = Configuration(max_splat_count=n, spherical_harmonics_order=3, field_of_view_y=math.radians(60))
    rec = synthetic.plain_small(n, seed=4, sh_order=3)
    r = Renderer(config)
    s = Scene(r, n)
    s.load_chunk(rec)
    r.set_profiling(True)
    cam = camera.look_at([0.0, 1.0, -7.0], [0.0, 0.0, 0.0])
    times = {"depth_sort": [], "pair_sort": []}
    for _ in range(23):
        img = r.render_frame(s, cam, 640, 480)
        st = r.stage_times()
        for k in times:
            times[k].append(st[k])
    torch.cuda.synchronize()
    med = {k: float(np.median(v[3:])) * 1000.0 for k, v in times.items()}
    print(f"2k splats, 640x480: median depth sort {med['depth_sort']:.1f} us, pair sort {med['pair_sort']:.1f} us")
    o = oracle_frame(config, oracle.load_transform(rec), cam, 640, 480)
    assert np.array_equal(img.cpu().numpy(), o[0])
    assert med["depth_sort"] < 20.0 and med["pair_sort"] < 20.0


def test_lookback_timeout_reports_and_context_survives(cuda):
    import ctypes
    import torch
    lib = _lib.load()
    flag = ctypes.c_int(0)
    _lib.check(lib.spl_debug_lookback_timeout(2000, ctypes.byref(flag)))
    assert flag.value == 1
    # the context is still usable
    config = Configuration(max_splat_count=1000, spherical_harmonics_order=0)
    rec = synthetic.plain_small(1000, seed=5)
    g = gpu_frame(cuda, config, rec, default_cam(), 64, 64)
    o = oracle_frame(config, oracle.load_transform(rec), default_cam(), 64, 64)
    assert_frame_parity(g, o, config)
    torch.cuda.synchronize()


def test_pair_capacity_overflow_is_an_error_not_a_fault(cuda):
    import torch
    config = Configuration(max_splat_count=20000, max_pair_count=500, spherical_harmonics_order=0)
    rec = synthetic.plain_small(20000, seed=8)
    r = Renderer(config)
    s = Scene(r, 20000)
    s.load_chunk(rec)
    r.render_frame(s, default_cam(dist=6.0), 320, 240)
    torch.cuda.synchronize()
    with pytest.raises(SplatterError) as e:
        r.frame_info()
    assert e.value.code == _lib.SPL_ERR_CAPACITY
    info = r.frame_info(check_status=False)
    assert info.pair_count > 500


@pytest.mark.parametrize("sorting", [DepthSorting.CPU, DepthSorting.GPU], ids=["cpu-fallback-keys", "gpu-keys"])
def test_small_scene_640x480_parity(cuda, sorting):
    """Config 'plain path, small scene' (the reference's CPU-runnable case): 100k splats, positions ~
    N(0, 2^2), SH degree 0, 640x480, fovy 60, camera at distance 8 looking at the origin; with the CPU
    depth-sort fallback's keys (what the reference runs on the CPU) and with the GPU keys."""
    n = 100_000
    config = Configuration(depth_sorting=sorting, spherical_harmonics_order=0, max_splat_count=n,
                           field_of_view_y=math.radians(60))
    rec = synthetic.plain_small(n, seed=0, sh_order=0)
    cam = camera.look_at([0.0, 0.0, -8.0], [0.0, 0.0, 0.0])
    g = gpu_frame(cuda, config, rec, cam, 640, 480)
    o = oracle_frame(config, oracle.load_transform(rec), cam, 640, 480)
    assert g[3].visible_count > 50000
    assert_frame_parity(g, o, config)
    assert image_psnr(g[0], o[0]) == float("inf")


def gpu_frames(config, records, cams, w, h):
    """gpu_frame's outputs for several cameras of one scene, through one renderer."""
    import torch
    r = Renderer(config)
    s = Scene(r, records.shape[0])
    s.load_chunk(records)
    try:
        for cam in cams:
            img = r.render_frame(s, cam, w, h)
            torch.cuda.synchronize()
            keys, idx, info = r.sorted_entries()
            recs = r.records()
            torch.cuda.synchronize()
            yield (img.cpu().numpy(), keys.cpu().numpy().view(np.uint32), idx.cpu().numpy().view(np.uint32), info,
                   recs.cpu().numpy(), None)
    finally:
        s.close()
        r.close()


def test_clustered_1m_1080p_parity(cuda):
    """Config 'plain path 1M': 1M clustered splats, SH 3, 1920x1080, all 32 seeded orbit poses: keys,
    visible set, permutation, records and image bit-exact against the oracle."""
    n = 1_000_000
    config = Configuration(max_splat_count=n, spherical_harmonics_order=3, field_of_view_y=math.radians(60))
    rec = synthetic.clustered(n, seed=1)
    sc = oracle.load_transform(rec)
    poses = camera.orbit_poses(32, seed=7, radius=(6.0, 12.0))
    for k, g in enumerate(gpu_frames(config, rec, poses, 1920, 1080)):
        o = oracle_frame(config, sc, poses[k], 1920, 1080)
        assert_frame_parity(g, o, config)


def near_plane_cuts(centers, poses, w, h, fovy, stride=6):
    """Per pose, the splat centres (every stride-th) in the frustum's slab 0 < view z < 2 around the
    near plane (view z = 1), scaled back to the whole scene, over the count a uniform background of
    the clustered scene's density would put there: a ratio well above 1 means the near plane cuts a
    cluster."""
    c = np.asarray(centers[::stride], np.float64)
    vh = math.tan(fovy / 2.0)
    vw = vh * w / h
    density = 0.2 * len(centers) / 40.0 ** 3  # the uniform background: 20% of the splats in the 40^3 box
    slab = 4.0 * vw * vh * 8.0 / 3.0  # frustum volume between view z = 0 and 2
    out = []
    for cam in poses:
        m = np.asarray(cam, np.float64).reshape(4, 4)  # rows = the camera's columns
        v = (c - m[3, :3]) @ m[:3, :3].T
        z = v[:, 2]
        near = (z > 0.0) & (z < 2.0) & (np.abs(v[:, 0]) < vw * z) & (np.abs(v[:, 1]) < vh * z)
        out.append(stride * int(near.sum()) / (density * slab))
    return np.array(out)


def flythrough_parity_poses():
    """The fly-through poses the 6M parity test renders: every pose whose near plane cuts a cluster
    (near-slab count >= 3x the background's) and seeded others, 24 in all."""
    n = 6_000_000
    rec = synthetic.clustered(n, seed=2)
    poses = camera.flythrough_poses(128, seed=9)
    ratio = near_plane_cuts(rec[:, 0:3], poses, 1920, 1080, math.radians(60))
    cut = [int(i) for i in np.nonzero(ratio >= 3.0)[0]]
    rng = np.random.default_rng(2024)
    others = [int(i) for i in rng.permutation(128) if i not in cut]
    return rec, poses, cut, sorted(cut + others[:max(0, 24 - len(cut))])


@pytest.fixture(scope="module")
def flythrough_6m():
    rec, poses, cut, chosen = flythrough_parity_poses()
    return rec, oracle.load_transform(rec), poses, cut, chosen


@pytest.mark.parametrize("w,h", [(1920, 1080), (3840, 2160)], ids=["1080p", "2160p"])
def test_clustered_6m_flythrough_parity(cuda, flythrough_6m, w, h):
    """Config 'plain path at scale': 6M clustered splats, SH 3, ~40% culled, 24 of the 128 fly-through
    poses (every pose whose near plane cuts a cluster, the rest seeded) at 1920x1080 and 3840x2160:
    keys, visible set, permutation, records and image bit-exact against the oracle."""
    rec, sc, poses, cut, chosen = flythrough_6m
    n = rec.shape[0]
    assert len(cut) >= 4 and len(chosen) >= 16
    print(f"near plane cuts a cluster at poses {cut}; rendering {chosen}")
    config = Configuration(max_splat_count=n, spherical_harmonics_order=3, field_of_view_y=math.radians(60))
    culled = []
    for k, g in zip(chosen, gpu_frames(config, rec, [poses[i] for i in chosen], w, h)):
        o = oracle_frame(config, sc, poses[k], w, h)
        culled.append(1.0 - o[3] / n)
        assert_frame_parity(g, o, config)
    print(f"culled per view: mean {np.mean(culled):.2f}, min {np.min(culled):.2f}, max {np.max(culled):.2f}")
    assert 0.1 < np.mean(culled) < 0.8
