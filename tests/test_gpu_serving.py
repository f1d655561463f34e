"""Captured frame graphs, the onesweep sort mode and the serving runtime on the GPU.

The bar is bit-identity: a frame replayed from a graph, a frame sorted by the onesweep passes and a
request served among others (concurrent slots, graphs or direct launches, scenes evicted to host
memory and copied back) all give the same bytes as the same frame rendered alone by a plain
Renderer with the cooperative sort.
"""
import numpy as np
import pytest

from splatter_gb300 import (SORT_ONESWEEP, BlendMode, Configuration, DepthSorting, Renderer, Scene, SplatterError,
                             camera, synthetic)

pytestmark = pytest.mark.gpu

RES = [(256, 256), (320, 180), (480, 270)]
SIZES = [30000, 80000, 150000]


def _cfg(n):
    return Configuration(max_splat_count=n, spherical_harmonics_order=3)


def test_frame_graph_and_onesweep_match_direct(cuda):
    import torch
    n, W, H = 60000, 320, 240
    rec = synthetic.clustered(n, seed=3, sh_order=3)
    poses = camera.orbit_poses(6, seed=4, radius=(6.0, 14.0))
    r = Renderer(_cfg(n))
    s = Scene(r, n)
    s.load_chunk(rec)
    ref = [r.render_frame(s, p, W, H).cpu() for p in poses]
    assert sum(int((im[..., 3] != 255).sum()) for im in ref) > 1000  # something drawn
    r2 = Renderer(_cfg(n))
    r2.set_sort_mode(SORT_ONESWEEP)
    s2 = Scene(r2, n)
    s2.load_chunk(rec)
    for p, im in zip(poses, ref):
        assert torch.equal(r2.render_frame(s2, p, W, H).cpu(), im)
    g = r2.capture_frame(W, H)
    for p, im in zip(poses, ref):
        out = g.launch(s2, p)
        torch.cuda.synchronize()
        assert torch.equal(out.cpu(), im)
    # the renderer's frame state follows the replayed frame
    info = r2.frame_info()
    assert info.width == W and info.height == H and info.splat_count == n
    # one graph serves scenes of other sizes (grids sized for max_splat_count)
    small = synthetic.clustered(9000, seed=8, sh_order=3)
    s3 = _scene_on(r2, small)
    s3_alone = _scene_on(r, small)
    for p in poses[:3]:
        want = r.render_frame(s3_alone, p, W, H).cpu()
        out = g.launch(s3, p)
        torch.cuda.synchronize()
        assert torch.equal(out.cpu(), want)
    g.close()
    # a graph bounded to small scenes: same bytes, and larger scenes are refused
    gs = r2.capture_frame(W, H, max_splats=10000)
    for p in poses[:2]:
        want = r.render_frame(s3_alone, p, W, H).cpu()
        out = gs.launch(s3, p)
        torch.cuda.synchronize()
        assert torch.equal(out.cpu(), want)
    with pytest.raises(SplatterError):
        gs.launch(s2, poses[0])
    gs.close()


def test_render_frame_replays_its_own_graph(cuda):
    """render_frame captures the second frame in a row of a viewport and scene size into a graph and
    replays it for the frames that follow: every frame equals a direct launch bit for bit, with the
    output buffer alternating, another scene of the same size, a larger viewport in between (which
    reallocates the per-viewport scratch) and the viewport changing back; the frame state (counters,
    entries) follows the replayed frame."""
    import torch
    n = 60000
    recs = [synthetic.clustered(n, seed=3, sh_order=3), synthetic.clustered(n, seed=5, sh_order=3)]
    poses = camera.orbit_poses(10, seed=6, radius=(6.0, 14.0))
    direct = Renderer(_cfg(n))
    direct.set_frame_graphs(False)
    r = Renderer(_cfg(n))
    sd = [_scene_on(direct, x) for x in recs]
    sr = [_scene_on(r, x) for x in recs]
    bufs = {vp: [r.output_buffer(*vp) for _ in range(2)] for vp in ((320, 240), (640, 360))}
    plan = [(0, (320, 240)), (0, (320, 240)), (0, (320, 240)), (1, (320, 240)), (0, (640, 360)),
            (1, (640, 360)), (1, (640, 360)), (0, (320, 240)), (0, (320, 240)), (1, (320, 240))]
    for k, (si, vp) in enumerate(plan):
        want = direct.render_frame(sd[si], poses[k], *vp).cpu()
        got = r.render_frame(sr[si], poses[k], *vp, out=bufs[vp][k % 2])
        torch.cuda.synchronize()
        assert torch.equal(got.cpu(), want), f"frame {k}"
        a, b = r.frame_info(), direct.frame_info()
        assert (a.visible_count, a.draw_count, a.pair_count, a.width, a.height) == \
            (b.visible_count, b.draw_count, b.pair_count, b.width, b.height)
        ka, ia, _ = r.sorted_entries()
        kb, ib, _ = direct.sorted_entries()
        assert torch.equal(ka, kb) and torch.equal(ia, ib)
    assert int((want[..., 3] != 255).sum()) > 1000  # something drawn


GRAPH_MODES = [
    dict(depth_sorting=DepthSorting.NONE),
    dict(depth_sorting=DepthSorting.CPU),
    dict(depth_sorting=DepthSorting.GPU_INDIRECT_DRAW),
    dict(depth_sorting=DepthSorting.GPU, use_unaligned_rectangles=False, use_covariance_for_scale=False),
    dict(depth_sorting=DepthSorting.GPU, blend_mode=BlendMode.FP32, spherical_harmonics_order=1),
]


@pytest.mark.parametrize("mode", GRAPH_MODES, ids=lambda m: "-".join(f"{k}={int(v)}" for k, v in m.items()))
@pytest.mark.parametrize("sort_mode", ["cooperative", "onesweep"])
def test_own_graph_replay_in_every_mode(cuda, mode, sort_mode):
    """The renderer's own frame graph (captured on the second frame of a viewport and scene size,
    replayed after) in the other depth-sorting modes, rectangle kinds, semi-axis methods and blend
    targets, with either sort: every frame equals a renderer's direct launches bit for bit."""
    import torch
    n, W, H = 40000, 320, 240
    cfg = Configuration(max_splat_count=n, **{"spherical_harmonics_order": 3, **mode})
    rec = synthetic.clustered(n, seed=9, sh_order=3)
    poses = camera.orbit_poses(6, seed=10, radius=(6.0, 14.0))
    direct = Renderer(cfg)
    direct.set_frame_graphs(False)
    r = Renderer(cfg)
    if sort_mode == "onesweep":
        direct.set_sort_mode(SORT_ONESWEEP)
        r.set_sort_mode(SORT_ONESWEEP)
    sd, sr = _scene_on(direct, rec), _scene_on(r, rec)
    drawn = 0
    for k, pose in enumerate(poses):
        want = direct.render_frame(sd, pose, W, H).cpu()
        got = r.render_frame(sr, pose, W, H).cpu()
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"frame {k}"
        a, b = r.frame_info(), direct.frame_info()
        assert (a.visible_count, a.draw_count, a.pair_count) == (b.visible_count, b.draw_count, b.pair_count)
        drawn = max(drawn, a.pair_count)
    assert drawn > 1000


def _scene_on(renderer, rec):
    sc = Scene(renderer, rec.shape[0])
    sc.load_chunk(rec)
    return sc


def _requests(count, seed):
    rng = np.random.default_rng(seed)
    poses = camera.orbit_poses(count, seed=seed + 1, radius=(6.0, 14.0))
    return [(int(rng.integers(len(SIZES))), poses[i], RES[int(rng.integers(len(RES)))]) for i in range(count)]


@pytest.fixture(scope="module")
def alone():
    """The requests rendered one by one by a plain Renderer (cooperative sort, direct launches)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    scenes = [synthetic.clustered(n, seed=10 + i, sh_order=3) for i, n in enumerate(SIZES)]
    reqs = _requests(48, seed=21)
    r = Renderer(_cfg(max(SIZES)))
    objs = []
    for rec in scenes:
        sc = Scene(r, rec.shape[0])
        sc.load_chunk(rec)
        objs.append(sc)
    imgs = [r.render_frame(objs[sid], pose, w, h).cpu() for sid, pose, (w, h) in reqs]
    torch.cuda.synchronize()
    return scenes, reqs, imgs


@pytest.mark.parametrize("graphs,budget_mb", [(True, 0), (False, 0), (True, 40)],
                         ids=["graphs", "direct", "graphs-evicting"])
def test_served_results_equal_alone(cuda, alone, graphs, budget_mb):
    import torch
    from splatter_gb300.serving import Server
    scenes, reqs, imgs = alone
    srv = Server(_cfg(max(SIZES)), slots=4, use_graphs=graphs, scene_memory_budget=budget_mb << 20, max_width=480,
                 max_height=270)
    ids = [srv.add_scene(rec) for rec in scenes]
    assert ids == [0, 1, 2]
    outs = [srv.output_buffer(w, h) for _, _, (w, h) in reqs]
    tags = [srv.submit(sid, pose, w, h, out) for (sid, pose, (w, h)), out in zip(reqs, outs)]
    done = srv.wait_all(len(reqs))
    assert sorted(c.tag for c in done) == sorted(tags)
    assert all(c.status == 0 for c in done)
    assert all(c.t_submit_ns <= c.t_start_ns <= c.t_done_ns for c in done)
    for out, im in zip(outs, imgs):
        assert torch.equal(out, im)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["max_in_flight"] >= 2
    if graphs:
        assert st["graph_launches"] == len(reqs) and st["graphs_captured"] >= 1
    else:
        assert st["direct_launches"] == len(reqs)
    if budget_mb:
        assert st["evictions"] > 0 and st["restores"] > 0 and any(c.restored for c in done)
        assert st["resident_bytes"] <= budget_mb << 20
    srv.close()


def test_server_one_slot_is_the_plain_loop(cuda, alone):
    """slots=1: one request at a time with the cooperative sort (the plain per-request loop)."""
    import torch
    from splatter_gb300.serving import Server
    scenes, reqs, imgs = alone
    srv = Server(_cfg(max(SIZES)), slots=1, use_graphs=False, max_width=480, max_height=270)
    for rec in scenes:
        srv.add_scene(rec)
    outs = [srv.output_buffer(w, h) for _, _, (w, h) in reqs[:12]]
    for (sid, pose, (w, h)), out in zip(reqs[:12], outs):
        srv.submit(sid, pose, w, h, out)
    done = srv.wait_all(12)
    assert all(c.status == 0 for c in done) and srv.stats()["max_in_flight"] == 1
    for out, im in zip(outs, imgs[:12]):
        assert torch.equal(out, im)
    srv.close()


@pytest.mark.parametrize("graphs", [True, False], ids=["graphs", "direct"])
def test_served_fp32_square_frames_equal_alone(cuda, graphs):
    """The FP32 blend target (float4 pixels) with axis-aligned squares and ellipse-equation semi-axes:
    served frames (four slots, a budget that forces evictions) equal the same frames rendered alone,
    bit for bit."""
    import torch
    from splatter_gb300.serving import Server
    cfg = Configuration(max_splat_count=max(SIZES), spherical_harmonics_order=2, blend_mode=BlendMode.FP32,
                        use_unaligned_rectangles=False, use_covariance_for_scale=False)
    scenes = [synthetic.clustered(n, seed=30 + i, sh_order=3) for i, n in enumerate(SIZES)]
    reqs = _requests(20, seed=31)
    r = Renderer(cfg)
    objs = [_scene_on(r, rec) for rec in scenes]
    want = [r.render_frame(objs[sid], pose, w, h).cpu() for sid, pose, (w, h) in reqs]
    torch.cuda.synchronize()
    srv = Server(cfg, slots=4, use_graphs=graphs, scene_memory_budget=40 << 20, max_width=480, max_height=270)
    for rec in scenes:
        srv.add_scene(rec)
    outs = [srv.output_buffer(w, h) for _, _, (w, h) in reqs]
    assert all(o.dtype == torch.float32 for o in outs)
    for (sid, pose, (w, h)), out in zip(reqs, outs):
        srv.submit(sid, pose, w, h, out)
    done = srv.wait_all(len(reqs))
    assert all(c.status == 0 for c in done)
    for out, im in zip(outs, want):
        assert torch.equal(out.view(torch.int32), im.view(torch.int32))
    assert srv.stats()["restores"] > 0
    srv.close()


def test_server_rejects_bad_requests(cuda):
    from splatter_gb300.serving import Server
    srv = Server(_cfg(50000), slots=2, max_width=128, max_height=128)
    sid = srv.add_scene(synthetic.clustered(20000, seed=1, sh_order=3))
    out = srv.output_buffer(128, 128)
    pose = camera.look_at([0, 0, -10], [0, 0, 0])
    with pytest.raises(SplatterError):
        srv.submit(sid + 5, pose, 64, 64, out)
    with pytest.raises(SplatterError):
        srv.submit(sid, pose, 256, 64, srv.output_buffer(256, 64))
    # a scene larger than the whole budget is refused when it is added
    small = Server(_cfg(50000), slots=1, scene_memory_budget=1 << 20, max_width=64, max_height=64)
    with pytest.raises(SplatterError):
        small.add_scene(synthetic.clustered(20000, seed=2, sh_order=3))
    small.close()
    srv.submit(sid, pose, 128, 128, out)
    assert [c.status for c in srv.wait_all(1)] == [0]
    srv.close()
