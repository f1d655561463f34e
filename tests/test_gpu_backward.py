"""Backward pass on the GPU against the FP64 reference gradient and FP64 central finite differences.

The differentiable frame is the fp32 blend mode; loss L = sum over pixels and RGB of (C - target)^2.
Target images come from the unperturbed seed scene, the forward from a copy with positions perturbed
by N(0, 0.01^2), log-scales by N(0, 0.05^2) and opacity logits by N(0, 0.2^2) (the differentiation
configuration).  Tolerance: |g_gpu - g_ref| <= 1e-3 * max(|g_ref|, floor) per parameter, with floor =
1e-2 x the RMS of the compared reference values (gradients of parameters that barely move the loss
are compared absolutely at that scale).  Splats touching a pixel where the FP32 frame and the FP64
frame take a decision differently (a coverage edge, the 1/255 discard, the early stop or a
saturation boundary crossed within rounding) have different gradients by construction; the oracle
finds them exactly (its FP32 raster is the GPU's bit for bit) and they are excluded and counted.

With use_covariance_for_scale = false the semi-axes come from the ellipse equation, which the
reference's FP32 vertex stage carries to only ~1e-4 (median) of FP64 at this view: an FP32 frame
then differs from the FP64 frame before any gradient is taken.  In that mode the oracle composites
in FP64 on the renderer's own FP32 records (pin_records: the compositing backward is checked
exactly), and parameter gradients are compared for the splats whose FP32 ellipse agrees with FP64
to 1e-4.

The parameter gradients that miss 1e-3 are sums whose terms cancel: the record gradient times the
vertex-stage Jacobian, summed over the record's 10 entries, where |sum| is far below the sum of the
|terms|; the record gradients themselves carry ~1e-4 of FP32 accumulation error, which the
cancellation magnifies.  The Jacobian is not the cause: the outline ellipse's derivatives come from
the dual conic (spl_vertex.cuh, vertex_vjp_t), which FP32 carries to ~1e-7.
"""
import math

import numpy as np
import pytest

import oracle
from splatter_gb300 import BlendMode, Configuration, Renderer, Scene, camera, synthetic
from splatter_gb300.autograd import render_raw, render_splats

pytestmark = pytest.mark.gpu

REL_TOL = 1e-3
PARAM_NAMES = ["cx", "cy", "cz", "q0", "q1", "q2", "q3", "sx", "sy", "sz", "alpha"] + [f"sh{i}" for i in range(48)]


def _perturbed(rec, seed):
    rng = np.random.default_rng(seed)
    p = rec.copy()
    p[:, 0:3] += rng.normal(0.0, 0.01, (p.shape[0], 3)).astype(np.float32)
    p[:, 55:58] += rng.normal(0.0, 0.05, (p.shape[0], 3)).astype(np.float32)
    p[:, 54] += rng.normal(0.0, 0.2, p.shape[0]).astype(np.float32)
    return p


def _gpu_grads(renderer, sc, cam, W, H, target):
    import torch
    dev = "cuda"
    xyz = torch.tensor(np.ascontiguousarray(sc["center"].T), device=dev, requires_grad=True)
    rot = torch.tensor(sc["rotation"], device=dev, requires_grad=True)
    sa = torch.tensor(np.concatenate([sc["scale"], sc["alpha"][:, None]], 1), device=dev, requires_grad=True)
    sh = torch.tensor(sc["sh"], device=dev, requires_grad=True)
    img = render_splats(xyz, rot, sa, sh, renderer, cam, W, H)
    tgt = torch.tensor(target, device=dev, dtype=torch.float32)
    loss = ((img[..., :3] - tgt) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    g = np.zeros((sc["center"].shape[0], 59), np.float64)
    g[:, 0:3] = xyz.grad.t().cpu().numpy()
    g[:, 3:7] = rot.grad.cpu().numpy()
    g[:, 7:11] = sa.grad.cpu().numpy()
    g[:, 11:] = sh.grad.cpu().numpy()
    return float(loss.item()), g, img.detach().cpu().numpy()


def _compare(g, ref, idx):
    a = np.array([g[k, p] for k, p in idx])
    b = np.array([ref[k, p] for k, p in idx])
    floor = 1e-2 * math.sqrt(float(np.mean(b * b))) if len(b) else 0.0
    rel = np.abs(a - b) / np.maximum(np.abs(b), floor)
    return rel, floor


def _setup(n, W, H, seed, sh_order=3, scale_boost=0.0, dist=7.0, cov=True, rect=True):
    rec = synthetic.plain_small(n, seed=seed, sh_order=sh_order)
    rec[:, 55:58] += scale_boost
    cam = camera.look_at([0.3, 0.5, -dist], [0.0, 0.0, 0.0])
    cfg = Configuration(max_splat_count=n, spherical_harmonics_order=sh_order, blend_mode=BlendMode.FP32,
                        field_of_view_y=math.radians(60), use_covariance_for_scale=cov,
                        use_unaligned_rectangles=rect)
    return rec, cam, cfg


MODES = [(True, True), (False, True), (True, False)]


@pytest.fixture(scope="module", params=MODES, ids=["cov-rect", "ellipse-rect", "cov-square"])
def frame(request):
    """One differentiated frame: 20000 splats, 256x192, SH3, and its FP64 reference, per
    (use_covariance_for_scale, use_unaligned_rectangles)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    cov, rect = request.param
    n, W, H = 20000, 256, 192
    rec, cam, cfg = _setup(n, W, H, seed=41, scale_boost=1.0, cov=cov, rect=rect)
    r = Renderer(cfg)
    seed_sc = oracle.load_transform(rec)
    # target: the seed scene rendered by the same path
    xyz = torch.tensor(np.ascontiguousarray(seed_sc["center"].T), device="cuda")
    rot = torch.tensor(seed_sc["rotation"], device="cuda")
    sa = torch.tensor(np.concatenate([seed_sc["scale"], seed_sc["alpha"][:, None]], 1), device="cuda")
    sh = torch.tensor(seed_sc["sh"], device="cuda")
    target = render_splats(xyz, rot, sa, sh, r, cam, W, H)[..., :3].cpu().numpy().astype(np.float64)
    sc = oracle.load_transform(_perturbed(rec, seed=42))
    loss, g, img = _gpu_grads(r, sc, cam, W, H, target)
    u = oracle.uniforms(cam, W, H, fovy=cfg.field_of_view_y)
    ocfg = oracle.config_struct(depth_sorting=2, sh_order=3, blend_mode=1, use_covariance_for_scale=cov,
                                use_unaligned_rectangles=rect)
    ctx = oracle.GradContext(u, ocfg, {k: v.astype(np.float64) for k, v in sc.items()}, target)
    keys, idx, info = r.sorted_entries()
    vis = np.sort(idx.cpu().numpy().astype(np.int64))  # compaction order = ascending splat index
    well = np.ones(n, bool)
    if not cov:
        # The ellipse-equation semi-axes are ill-conditioned in FP32 (the reference's own forward):
        # composite in FP64 on the renderer's FP32 records, and compare parameter gradients only
        # where the FP32 ellipse (centre, axes, rotation) agrees with FP64 to 1e-4.
        ctx.pin_records(r.records().cpu().numpy(), vis)
        _, d32, _ = oracle.preprocess(u, ocfg, sc, vis)
        _, d64, _ = oracle.preprocess(u, ocfg, sc, vis, fp64=True)
        err = np.abs(d32[:, 9:15] - d64[:, 9:15]) / np.maximum(np.abs(d64[:, 9:15]), 1e-2)
        well[:] = False
        well[vis] = err.max(1) <= 1e-4
    loss64, ref, img64 = ctx.loss_and_grad(threads=16)
    amb, npix = ctx.ambiguous(threads=16)
    drawn_all = np.nonzero(np.abs(ref).sum(1) > 0)[0]
    drawn = drawn_all[~amb[drawn_all]]
    print(f"{len(drawn_all)} drawn splats, {npix} pixels decide differently in FP32 and FP64, "
          f"{len(drawn_all) - len(drawn)} splats excluded"
          + ("" if cov else f"; FP32 ellipse within 1e-4 of FP64 for {int(well[drawn].sum())}"))
    nparam = 11 + 3 * (cfg.spherical_harmonics_order + 1) ** 2
    yield dict(r=r, ctx=ctx, loss=loss, loss64=loss64, g=g, ref=ref, amb=amb, drawn=drawn, drawn_all=drawn_all,
               nparam=nparam, well=drawn[well[drawn]], cov=cov, rect=rect, img=img, img64=img64, npix=npix)
    ctx.close()


def test_fp32_frame_against_fp64_frame(frame):
    """The renderer's FP32 frame against the FP64 frame of the same scene (the oracle's FP64 vertex
    stage and compositing): PSNR >= 60 dB over RGB — the brief's image bar, with FP64 math standing in
    for the reference's wgpu render, which cannot run here.  (With use_covariance_for_scale = false
    the FP32 frame is compared on its own records, see the fixture: FP32 ellipses differ from FP64.)"""
    a = np.asarray(frame["img"], np.float64)[..., :3]
    b = np.asarray(frame["img64"], np.float64)[..., :3]
    mse = float(np.mean((a - b) ** 2))
    psnr = float("inf") if mse == 0 else 10.0 * math.log10(1.0 / mse)
    err = np.abs(a - b).max(axis=2)
    print(f"PSNR {psnr:.1f} dB, max |diff| {err.max():.2e}, {int((err > 2 / 255).sum())} pixels above 2/255 "
          f"({frame['npix']} pixels decide a coverage edge, discard or stop differently)")
    assert psnr >= 60.0
    assert int((err > 2 / 255).sum()) <= max(frame["npix"], 0)


def test_loss_and_drawn_set(frame):
    assert abs(frame["loss"] - frame["loss64"]) <= 1e-3 * frame["loss64"]
    drawn, drawn_all = frame["drawn"], frame["drawn_all"]
    assert len(drawn) > 1000 and len(drawn) >= 0.95 * len(drawn_all)
    if frame["cov"]:
        assert len(frame["well"]) == len(drawn)


def test_record_gradients_match_fp64(frame):
    """The raster backward alone: per visible splat the 10 gradients of its screen-space record
    (spl_renderer_copy_record_gradients) against the FP64 oracle's.  The GPU takes A against pixel
    offsets from the centre of the record's pixel box; the oracle's absolute-coordinate values are
    moved to that centre in FP64.  Each is a sum over the splat's pixels whose terms can cancel; at
    1e-3 of max(|ref|, 1e-2 x the component's RMS) >= 99.5% agree per component, and none is off by
    more than 0.25 of that scale (the few strongly cancelling sums)."""
    import ctypes
    import torch
    r, ctx = frame["r"], frame["ctx"]
    keys, idx, info = r.sorted_entries()
    V = int(info.visible_count)
    vis = np.sort(idx.cpu().numpy().astype(np.int64))  # compaction order = ascending splat index
    grec = torch.empty((V, 10), dtype=torch.float32, device="cuda")
    check_rc = r._lib.spl_renderer_copy_record_gradients(r.handle, ctypes.c_void_p(grec.data_ptr()), V, None)
    assert check_rc == 0
    torch.cuda.synchronize()
    grec = grec.cpu().numpy().astype(np.float64)
    recs = r.records().cpu().numpy()
    lo, hi = recs[:, 7].view(np.uint32), recs[:, 11].view(np.uint32)
    cx = 0.5 * ((lo & 0xFFFF).astype(np.float64) + (hi & 0xFFFF) + 1)
    cy = 0.5 * ((lo >> 16).astype(np.float64) + (hi >> 16) + 1)
    orr, order = ctx.record_gradients(threads=16)
    slot = np.searchsorted(vis, order.astype(np.int64))
    assert np.all(vis[slot] == order)
    ref = orr.copy()
    ref[:, 0] -= cx[slot] * ref[:, 2]
    ref[:, 1] -= cy[slot] * ref[:, 2]
    ref[:, 3] -= cx[slot] * ref[:, 5]
    ref[:, 4] -= cy[slot] * ref[:, 5]
    keep = (np.abs(ref).sum(1) > 0) & ~frame["amb"][order]
    a, b = grec[slot[keep]], ref[keep]
    names = ["A00", "A01", "B0", "A10", "A11", "B1", "opacity", "r", "g", "b"]
    for j in range(10):
        scale = np.maximum(np.abs(b[:, j]), 1e-2 * math.sqrt(float(np.mean(b[:, j] ** 2))))
        rel = np.abs(a[:, j] - b[:, j]) / scale
        print(f"record d/d{names[j]}: {100 * np.mean(rel <= REL_TOL):.3f}% within {REL_TOL}, max {rel.max():.2e}")
        assert np.mean(rel <= REL_TOL) >= 0.995
        assert rel.max() <= 0.25


def test_parameter_gradients_match_fp64_reference(frame):
    """Every parameter of every drawn splat against the FP64 reference gradient: >= 99.9% within
    1e-3 of max(|ref|, floor)."""
    g, ref, drawn, nparam = frame["g"], frame["ref"], frame["well"], frame["nparam"]
    assert len(drawn) > 1000
    idx = [(k, p) for k in drawn for p in range(nparam)]
    rel, floor = _compare(g, ref, idx)
    frac_ok = float(np.mean(rel <= REL_TOL))
    worst = sorted(zip(rel, idx), reverse=True)[:5]
    print(f"vs FP64 reference: {len(idx)} params, {100 * frac_ok:.3f}% within {REL_TOL}, floor {floor:.3e}, "
          f"p99 {np.percentile(rel, 99):.2e}, worst {[(f'{e:.2e}', PARAM_NAMES[p]) for e, (k, p) in worst]}")
    assert frac_ok >= 0.999


def test_parameter_gradients_match_finite_differences(frame):
    """256 seeded parameters against FP64 central differences (h = 1e-4) of the FP64 loss."""
    g, ref, drawn, nparam, ctx = frame["g"], frame["ref"], frame["well"], frame["nparam"], frame["ctx"]
    rng = np.random.default_rng(7)
    fd_idx, fd_val, excluded = [], [], 0
    while len(fd_idx) < 256:
        k = int(rng.choice(drawn))
        p = int(rng.integers(0, nparam))
        ok, v = ctx.fd(k, p, 1e-4)
        if not ok:
            excluded += 1
            continue
        fd_idx.append((k, p))
        fd_val.append(v)
    fd = np.zeros_like(ref)
    for (k, p), v in zip(fd_idx, fd_val):
        fd[k, p] = v
    rel_fd, floor_fd = _compare(g, fd, fd_idx)
    rel_ref_fd, _ = _compare(ref, fd, fd_idx)
    print(f"vs FP64 FD: 256 params ({excluded} excluded: discrete change under +-h), "
          f"{100 * np.mean(rel_fd <= REL_TOL):.1f}% within {REL_TOL}, max {rel_fd.max():.2e}; "
          f"FP64 reference vs FD max {rel_ref_fd.max():.2e}")
    if frame["cov"] and frame["rect"]:
        # the default configuration: every parameter
        assert np.all(rel_ref_fd <= REL_TOL)
        assert np.all(rel_fd <= REL_TOL)
    elif frame["cov"]:
        # axis-aligned squares: a square's side is the larger rotated semi-axis, max(|a|, |b|), whose
        # derivative switches where the two meet; 255 of 256 within 1e-3 (max 1.25e-3) measured
        assert np.mean(rel_ref_fd <= REL_TOL) >= 0.99
        assert np.mean(rel_fd <= REL_TOL) >= 0.99
    else:
        # pinned records: the differences move the perturbed splat's FP64 record while the others
        # stay pinned, so they test the same function only where the FP64 reference agrees with them
        agree = rel_ref_fd <= REL_TOL
        assert np.mean(agree) >= 0.9
        assert np.mean(rel_fd[agree] <= REL_TOL) >= 0.99


def _small_frame_against_fp64(mode, sh_order, contrast):
    """5000 splats at 160x120 in a depth-sorting mode and SH degree: the GPU's parameter gradients and
    their agreement with the FP64 reference gradient of the same mode (and, with `contrast`, of
    another mode's draw order)."""
    import torch
    from splatter_gb300 import DepthSorting
    n, W, H = 5000, 160, 120
    rec = synthetic.plain_small(n, seed=83, sh_order=sh_order)
    rec[:, 55:58] += 1.0
    cam = camera.look_at([0.3, 0.5, -7.0], [0.0, 0.0, 0.0])
    cfg = Configuration(max_splat_count=n, spherical_harmonics_order=sh_order, blend_mode=BlendMode.FP32,
                        field_of_view_y=math.radians(60), depth_sorting=DepthSorting(mode))
    r = Renderer(cfg)
    seed_sc = oracle.load_transform(rec)
    t = [torch.tensor(a, device="cuda") for a in (np.ascontiguousarray(seed_sc["center"].T), seed_sc["rotation"],
                                                 np.concatenate([seed_sc["scale"], seed_sc["alpha"][:, None]], 1),
                                                 seed_sc["sh"])]
    target = render_splats(*t, r, cam, W, H)[..., :3].cpu().numpy().astype(np.float64)
    sc = oracle.load_transform(_perturbed(rec, seed=84))
    loss, g, img = _gpu_grads(r, sc, cam, W, H, target)
    u = oracle.uniforms(cam, W, H, fovy=cfg.field_of_view_y)
    refs = {}
    for m in ((mode, 0 if mode != 0 else 2) if contrast else (mode,)):
        ctx = oracle.GradContext(u, oracle.config_struct(depth_sorting=m, sh_order=sh_order, blend_mode=1),
                                 {k: v.astype(np.float64) for k, v in sc.items()}, target)
        try:
            loss64, ref, _ = ctx.loss_and_grad(threads=16)
            amb, _ = ctx.ambiguous(threads=16)
        finally:
            ctx.close()
        refs[m] = (loss64, ref, amb)
    loss64, ref, amb = refs[mode]
    assert abs(loss - loss64) <= 1e-3 * loss64
    drawn_all = np.nonzero(np.abs(ref).sum(1) > 0)[0]
    drawn = drawn_all[~amb[drawn_all]]
    assert len(drawn) > 500 and len(drawn) >= 0.9 * len(drawn_all)
    nparam = 11 + 3 * (sh_order + 1) ** 2
    idx = [(k, p) for k in drawn for p in range(nparam)]
    rel, _ = _compare(g, ref, idx)
    geo = np.array([p < 11 for k, p in idx])
    frac_geo, frac_sh = float(np.mean(rel[geo] <= REL_TOL)), float(np.mean(rel[~geo] <= REL_TOL))
    frac_other = None
    if contrast:
        other = [m for m in refs if m != mode][0]
        rel_other, _ = _compare(g, refs[other][1], idx)
        frac_other = float(np.mean(rel_other <= REL_TOL))
    print(f"mode {mode}, SH {sh_order}: {len(drawn)} drawn splats within {REL_TOL} of the FP64 reference: "
          f"centre/rotation/scale/opacity {100 * frac_geo:.3f}%, SH {100 * frac_sh:.3f}%"
          + ("" if frac_other is None else f"; {100 * frac_other:.3f}% of all against another mode's order"))
    return frac_geo, frac_sh, frac_other


@pytest.mark.parametrize("mode", [0, 1, 2, 3], ids=["none", "cpu-keys", "gpu", "gpu-indirect"])
def test_backward_in_every_depth_sorting_mode(cuda, mode):
    """The backward re-walks each tile in the frame's draw order: index order without sorting, the
    reference's CPU keys, the GPU keys or the indirect draw's order.  Every parameter of every drawn
    splat against the FP64 reference gradient of the same mode (the oracle's draw list for it), within
    1e-3 of max(|ref|, floor), splats at FP32/FP64 decision boundaries excluded: >= 99% of the centre,
    rotation, scale and opacity gradients (99.16-99.28% measured on this scene of large splats, where
    the sums over a splat's pixels cancel more than at 20k splats) and >= 99.95% of the SH gradients;
    against another mode's draw order ~5% of all (the order decides the gradients)."""
    frac_geo, frac_sh, frac_other = _small_frame_against_fp64(mode, 3, contrast=True)
    assert frac_geo >= 0.99 and frac_sh >= 0.9995
    assert frac_other < 0.5


@pytest.mark.parametrize("sh_order", [0, 1, 2])
def test_backward_at_lower_sh_degrees(cuda, sh_order):
    """The vertex-stage backward is compiled per SH degree: degrees 0-2 against the FP64 reference
    gradient of the same degree, with the bars of the depth-sorting test (99.29-99.40% and >= 99.99%
    measured)."""
    frac_geo, frac_sh, _ = _small_frame_against_fp64(2, sh_order, contrast=False)
    assert frac_geo >= 0.99 and frac_sh >= 0.9995


def test_raw_parameter_gradients_through_autograd(cuda):
    """render_raw: the loader's activations and their backward on the GPU around the hand-written
    backward.  The frame equals the frame of a scene loaded from the same file records, and the raw
    gradients equal torch autograd's vector-Jacobian product through the torch restatement of the
    activations (`activate`) applied to the activated-parameter gradients of the same frame.  Some
    splats have a log-scale beyond mean + 5, so the clamp (whose gradient goes through the mean of
    all three) is exercised."""
    import torch
    from splatter_gb300.autograd import activate, activate_native
    n, W, H = 5000, 128, 96
    rec, cam, cfg = _setup(n, W, H, seed=51, scale_boost=1.0)
    rec[::250, 57] = rec[::250, 55] + 8.0  # clamped to mean + 5
    r = Renderer(cfg)
    leaves = [torch.tensor(rec[:, a:b], device="cuda").squeeze(1).contiguous().requires_grad_(True)
              for a, b in ((0, 3), (58, 62), (55, 58), (54, 55), (6, 54))]
    means, quats, logs, logits, sh = leaves
    img = render_raw(means, quats, logs, logits, sh, r, cam, W, H)
    (img[..., :3] ** 2).sum().backward()
    # the same frame from records through the loader
    sc = Scene(r, n)
    sc.load_chunk(rec)
    assert torch.equal(img, r.render_frame(sc, cam, W, H))
    # activated gradients of the same frame (same activated values, bit for bit)
    xyz, rot, sa = activate_native(means, quats, logs, logits)
    act = [t.clone().requires_grad_(True) for t in (xyz, rot, sa)]
    sh_ = sh.detach().clone().requires_grad_(True)
    img2 = render_splats(act[0], act[1], act[2], sh_, r, cam, W, H)
    assert torch.equal(img, img2)
    (img2[..., :3] ** 2).sum().backward()
    # chain through the torch restatement of the activations
    raw = [t.detach().clone().requires_grad_(True) for t in (means, quats, logs, logits)]
    ref = torch.autograd.grad(activate(*raw), raw, grad_outputs=[a.grad for a in act])
    torch.cuda.synchronize()
    # float atomics make the gradient sums order-dependent: compare at 1e-4 of each array's scale
    def close(a, b):
        return torch.allclose(a, b, rtol=1e-4, atol=1e-4 * float(b.abs().max()))
    assert close(sh.grad, sh_.grad)
    for got, want in zip((means.grad, quats.grad, logs.grad, logits.grad), ref):
        assert close(got, want)


@pytest.mark.parametrize("gap", [4.0, 6.0, 8.0])
def test_needle_gradients_are_repeatable(cuda, gap):
    """Needles (one log-scale `gap` above another: scale ratios 55 to 3000).  The exact gradient of a
    rotation about a needle's long axis is a sum of terms of order s_max^2 that cancel to order
    s_min^2, so a float reverse sweep leaves an error of ~eps (s_max / s_min)^2 that follows the last
    bits of the float-atomic record gradients (measured: 2.4e-5 of the frame's largest gradient at
    ratio 55, 7e-2 at 3000).  Beyond ratio 32 the vertex-stage backward sweeps in double: two
    backward passes of the same frame agree to 5e-6 of each array's largest gradient, the order
    of the atomics' own noise (~1e-6)."""
    import torch
    n, W, H = 5000, 128, 96
    rec, cam, cfg = _setup(n, W, H, seed=51, scale_boost=1.0)
    rec[::250, 57] = rec[::250, 55] + gap
    r = Renderer(cfg)

    def grads():
        leaves = [torch.tensor(rec[:, a:b], device="cuda").squeeze(1).contiguous().requires_grad_(True)
                  for a, b in ((0, 3), (58, 62), (55, 58), (54, 55), (6, 54))]
        img = render_raw(*leaves, r, cam, W, H)
        (img[..., :3] ** 2).sum().backward()
        return [t.grad.clone() for t in leaves]

    runs = [grads() for _ in range(3)]
    needles = torch.arange(0, n, 250, device="cuda")
    assert float(runs[0][1][needles].abs().sum()) > 0.0  # the needles are drawn and have gradients
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            assert float((a - b).abs().max()) <= 5e-6 * float(a.abs().max())


def test_backward_rejects_unaligned_gradient_arrays(cuda):
    """spl_render_backward writes rotation, scale/opacity and SH gradients with 16-byte stores: an output
    array that is not 16-byte aligned is refused with SPL_ERR_INVALID before anything is launched, and
    aligned arrays of the same frame are accepted."""
    import ctypes
    import torch
    from splatter_gb300 import SplatterError
    from splatter_gb300._lib import check
    n, W, H = 2000, 64, 48
    rec, cam, cfg = _setup(n, W, H, seed=71, scale_boost=1.0)
    r = Renderer(cfg)
    sc = Scene(r, n)
    sc.load_chunk(rec)
    img = r.render_frame(sc, cam, W, H).contiguous()
    g = torch.ones_like(img)
    xyz = torch.zeros((3, n), device="cuda")
    # one buffer per array, a float longer than it: element 0 is aligned, element 1 is 4 bytes off
    bufs = [torch.zeros(k * n + 4, device="cuda") for k in (4, 4, 48)]
    aligned = [b[:k * n] for b, k in zip(bufs, (4, 4, 48))]
    shifted = [b[1:k * n + 1] for b, k in zip(bufs, (4, 4, 48))]
    assert all(t.data_ptr() % 16 == 0 for t in aligned) and all(t.data_ptr() % 16 == 4 for t in shifted)

    def call(arrays):
        p = [ctypes.c_void_p(t.data_ptr()) for t in (img, g, xyz[0], xyz[1], xyz[2], *arrays)]
        check(r._lib.spl_render_backward(r.handle, sc.handle, *p, None))

    for k in range(3):
        with pytest.raises(SplatterError):
            call([shifted[i] if i == k else aligned[i] for i in range(3)])
    call(aligned)
    torch.cuda.synchronize()
    assert float(aligned[2].abs().sum()) > 0.0  # SH gradients were written


def test_l2_image_loss_equals_torch(cuda):
    """l2_image_loss against the torch expression it replaces, ((images[..., :3] - targets) ** 2).sum():
    the same loss to summation rounding and the same gradient bit for bit, with a non-unit upstream
    gradient and a pixel count that is not a multiple of the block size."""
    import torch
    from splatter_gb300.autograd import l2_image_loss
    g = torch.Generator(device="cuda").manual_seed(5)
    images = torch.rand((3, 37, 53, 4), device="cuda", generator=g)
    targets = torch.rand((3, 37, 53, 3), device="cuda", generator=g)
    a = images.clone().requires_grad_(True)
    b = images.clone().requires_grad_(True)
    la = l2_image_loss(a, targets)
    lb = ((b[..., :3] - targets) ** 2).sum()
    (la * 0.37).backward()
    (lb * 0.37).backward()
    assert torch.allclose(la, lb, rtol=1e-6, atol=0.0)
    assert torch.equal(a.grad, b.grad)
    with pytest.raises(ValueError):
        l2_image_loss(images[..., :3], targets)


def test_render_raw_views_equals_per_view_sum(cuda):
    """render_raw_views: the stacked frames equal render_raw's frame of each view bit for bit, and
    the in-place accumulated gradients equal the per-view render_raw gradients that autograd sums
    over the views (to the rounding of the float atomics and of the activations' chain rule applied
    to the sum).  Two renderers for three views, so the backward renders one view again."""
    import torch
    from splatter_gb300.autograd import render_raw_views
    n, W, H = 5000, 128, 96
    rec, cam, cfg = _setup(n, W, H, seed=61, scale_boost=0.5)
    cams = [cam] + [camera.look_at(np.array([math.sin(a) * 7.0, 0.8, math.cos(a) * 7.0], np.float32),
                                   np.zeros(3, np.float32)) for a in (0.4, -0.7)]
    rs = [Renderer(cfg), Renderer(cfg)]

    def leaves():
        return [torch.tensor(rec[:, a:b], device="cuda").squeeze(1).contiguous().requires_grad_(True)
                for a, b in ((0, 3), (58, 62), (55, 58), (54, 55), (6, 54))]
    weights = torch.rand((len(cams), H, W, 3), device="cuda", generator=torch.Generator("cuda").manual_seed(5))
    batched = leaves()
    imgs = render_raw_views(*batched, rs, cams, W, H)
    (imgs[..., :3] ** 2 * weights).sum().backward()
    single = leaves()
    for v, c in enumerate(cams):
        img = render_raw(*single, rs[0], c, W, H)
        assert torch.equal(img, imgs[v])
        (img[..., :3] ** 2 * weights[v]).sum().backward()
    torch.cuda.synchronize()
    for got, want in zip((t.grad for t in batched), (t.grad for t in single)):
        assert float(want.abs().max()) > 0.0
        assert torch.allclose(got, want, rtol=1e-4, atol=1e-4 * float(want.abs().max()))


def test_backward_requires_fp32_blend(cuda):
    import torch
    from splatter_gb300 import SplatterError
    r = Renderer(Configuration(max_splat_count=10, blend_mode=BlendMode.UNORM8))
    x = torch.zeros((3, 10), device="cuda")
    with pytest.raises(ValueError):
        render_splats(x, torch.zeros((10, 4), device="cuda"), torch.zeros((10, 4), device="cuda"),
                      torch.zeros((10, 48), device="cuda"), r, camera.look_at([0, 0, -5], [0, 0, 0]), 8, 8)
    del SplatterError
