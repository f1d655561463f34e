"""The backward pass at the differentiation configuration's own size, in the raw parameters.

Workload: 1M clustered splats, SH degree 3, 1024x1024, 8 orbit views; the targets are the seed
scene's frames, the forward runs on a copy with positions perturbed by N(0, 0.01^2), log-scales by
N(0, 0.05^2) and opacity logits by N(0, 0.2^2); the loss is the L2 image loss summed over the 8
views.  The GPU side is render_raw_views (the loader's activations and their backward on the GPU
around the hand-written raster and vertex-stage backward), giving gradients of the RAW parameters:
means, quaternions, log-scales, opacity logits and SH.

The FP64 side is the oracle: the raw parameters activated in FP64 (activate64, the loader's
transform), one FP64 gradient context per view (the analytic FP64 gradient of the view's loss, the
splats whose pixels decide a threshold differently in FP32 and FP64, and central differences of the
FP64 loss that re-render only the tiles the perturbed splat touches), summed over the views, and the
chain rule of the activations in FP64 (raw_gradients64).

Comparisons, per value |g_gpu - g_ref| <= tol * max(|g_ref|, floor), floor = 1e-2 x the RMS of the
compared reference values:
  * central differences of the FP64 loss, 256 seeded raw parameters: every one within 1e-3;
  * the compositing backward alone, view 0: the renderer's per-record gradients against the FP64
    compositing backward on the renderer's own FP32 records (pin_records) from the FP32 frame's own
    upstream gradient dL/dC = 2 (C32 - target) (set_image_gradient): >= 99.9% within 1e-3 per record
    component;
  * raw parameters against the FP64 backward from the same dL/dC on FP64 records: >= 99.5% within
    1e-3 and >= 99.99% within 1e-2.  The remaining gap is the FP32 forward's own precision: a small
    splat's texture coordinate is tc = A X + B with |A X| up to ~1e4 |tc| at 1024 pixels, so the FP32
    records (fixed bit for bit by the parity bar) carry ~1e-4 of relative rounding into the position
    gradients, which sum such terms over a few pixels with cancellation;
  * raw parameters against the FP64 gradient of the FP64 loss: >= 99.5% within 1e-2.  At this size
    the residual C - target is small (the perturbations move each pixel a little), so dL/dC is
    sensitive to the FP32 frame's own rounding (the FP32 and FP64 frames differ by ~1e-6): a few
    percent of the parameters differ by more than 1e-3 from the FP64 loss's gradient before the
    backward runs.
Excluded and counted: splats touching, in any view, a pixel where the FP32 and FP64 frames take a
decision differently (coverage edge, 1/255 discard, early stop, saturation), and differences under
which something discrete changes (depth key, tile set, a pixel's list of contributors).
"""
import ctypes
import math
import os

import numpy as np
import pytest

import oracle
from splatter_gb300 import BlendMode, Configuration, Renderer, camera, synthetic
from splatter_gb300.autograd import render_raw, render_raw_views

pytestmark = pytest.mark.gpu

REL_TOL = 1e-3
N, W, H, VIEWS = 1_000_000, 1024, 1024, 8
H_FD = 1e-4
THREADS = os.cpu_count() or 8
SLOT_NAMES = (["mx", "my", "mz", "q0", "q1", "q2", "q3", "log_sx", "log_sy", "log_sz", "logit"]
              + [f"sh{i}" for i in range(48)])


def _rel(a, b):
    floor = 1e-2 * math.sqrt(float(np.mean(b * b))) if len(b) else 0.0
    return np.abs(a - b) / np.maximum(np.abs(b), floor), floor


@pytest.fixture(scope="module")
def diff_config(cuda):
    import torch
    rec = synthetic.clustered(N, seed=111, sh_order=3)
    poses = camera.orbit_poses(VIEWS, seed=113)
    cfg = Configuration(max_splat_count=N, spherical_harmonics_order=3, blend_mode=BlendMode.FP32,
                        field_of_view_y=math.radians(60.0))
    renderers = [Renderer(cfg) for _ in range(VIEWS)]

    def leaves(a, grad):
        t = torch.tensor(a, device="cuda")
        out = [t[:, 0:3].contiguous(), t[:, 58:62].contiguous(), t[:, 55:58].contiguous(), t[:, 54].contiguous(),
               t[:, 6:54].contiguous()]
        return [x.requires_grad_(grad) for x in out]

    with torch.no_grad():
        seed_p = leaves(rec, False)
        targets = torch.stack([render_raw(*seed_p, renderers[0], poses[v], W, H)[..., :3].clone()
                               for v in range(VIEWS)])
    rng = np.random.default_rng(117)
    pert = rec.copy()
    pert[:, 0:3] += rng.normal(0.0, 0.01, (N, 3)).astype(np.float32)
    pert[:, 55:58] += rng.normal(0.0, 0.05, (N, 3)).astype(np.float32)
    pert[:, 54] += rng.normal(0.0, 0.2, N).astype(np.float32)
    lv = leaves(pert, True)
    imgs = render_raw_views(*lv, renderers, poses, W, H)
    loss = ((imgs[..., :3] - targets) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    g = np.zeros((N, 59), np.float64)
    g[:, 0:3] = lv[0].grad.cpu().numpy()
    g[:, 3:7] = lv[1].grad.cpu().numpy()
    g[:, 7:10] = lv[2].grad.cpu().numpy()
    g[:, 10] = lv[3].grad.cpu().numpy()
    g[:, 11:59] = lv[4].grad.cpu().numpy()
    gpu_loss = float(loss.item())
    target64 = targets.cpu().numpy().astype(np.float64)
    gimg64 = 2.0 * (imgs[..., :3].detach().cpu().numpy().astype(np.float64) - target64)
    # view 0's frame state: its records, visible set and per-record gradients (its renderer ran its backward)
    r0 = renderers[0]
    _, idx0, info0 = r0.sorted_entries()
    vis0 = np.sort(idx0.cpu().numpy().astype(np.int64))
    recs0 = r0.records().cpu().numpy()
    grec0 = torch.empty((int(info0.visible_count), 10), dtype=torch.float32, device="cuda")
    assert r0._lib.spl_renderer_copy_record_gradients(r0.handle, ctypes.c_void_p(grec0.data_ptr()),
                                                      int(info0.visible_count), None) == 0
    torch.cuda.synchronize()
    grec0 = grec0.cpu().numpy().astype(np.float64)
    del imgs, loss, lv, seed_p, targets, renderers, r0
    torch.cuda.empty_cache()

    # FP64: one gradient context per view, kept one at a time
    raw = oracle.raw_slots(pert)
    act = oracle.activate64(raw)
    sc = oracle.scene64(act)
    ocfg = oracle.config_struct(depth_sorting=2, sh_order=3, blend_mode=1)
    ref_act = np.zeros((N, 59), np.float64)
    drv_act = np.zeros((N, 59), np.float64)
    amb = np.zeros(N, bool)
    drawn = np.zeros(N, bool)
    loss64 = 0.0
    npix = 0
    cand, fd_sum, fd_ok = None, None, None
    crng = np.random.default_rng(119)
    for v in range(VIEWS):
        u = oracle.uniforms(poses[v], W, H, fovy=cfg.field_of_view_y)
        ctx = oracle.GradContext(u, ocfg, sc, target64[v])
        lv64, gv, _ = ctx.loss_and_grad(threads=THREADS)
        loss64 += lv64
        ref_act += gv
        ctx.set_image_gradient(gimg64[v])
        drv_act += ctx.loss_and_grad(threads=THREADS)[1]
        ctx.set_image_gradient(None)
        a_v, np_v = ctx.ambiguous(threads=THREADS)
        amb |= a_v
        npix += np_v
        dv = np.abs(gv).sum(1) > 0
        drawn |= dv
        if cand is None:
            # 512 seeded (splat, raw slot) candidates among the splats view 0 draws and decides alike
            pool = np.nonzero(dv & ~a_v)[0]
            cand = [(int(crng.choice(pool)), int(crng.integers(0, 59))) for _ in range(512)]
            fd_sum = np.zeros(len(cand))
            fd_ok = np.ones(len(cand), bool)
        for i, (k, j) in enumerate(cand):
            if not fd_ok[i]:
                continue
            pp, pm = raw[k].copy(), raw[k].copy()
            pp[j] += H_FD
            pm[j] -= H_FD
            ok, val = ctx.fd_params(k, oracle.activate64(pp)[0], oracle.activate64(pm)[0], 2.0 * H_FD)
            fd_ok[i] = ok
            fd_sum[i] += val
        if v == 0:
            # the compositing backward alone: FP64 on the renderer's FP32 records, same dL/dC
            ctx.pin_records(recs0, vis0)
            ctx.set_image_gradient(gimg64[0])
            orec0, order0 = ctx.record_gradients(threads=THREADS)
            amb0 = a_v.copy()
        ctx.close()
    ref = oracle.raw_gradients64(raw, ref_act)
    drv = oracle.raw_gradients64(raw, drv_act)
    keep = drawn & ~amb
    print(f"loss: GPU {gpu_loss:.6e}, FP64 {loss64:.6e}; {int(drawn.sum())} splats drawn over {VIEWS} views, "
          f"{npix} pixels decide differently in FP32 and FP64, {int((drawn & amb).sum())} splats excluded")
    # the oracle takes A against absolute pixel-centre coordinates, the renderer against offsets from
    # the record's box centre: move the FP64 values to the box centre
    slot0 = np.searchsorted(vis0, order0.astype(np.int64))
    lo, hi = recs0[:, 7].view(np.uint32), recs0[:, 11].view(np.uint32)
    bcx = 0.5 * ((lo & 0xFFFF).astype(np.float64) + (hi & 0xFFFF) + 1)
    bcy = 0.5 * ((lo >> 16).astype(np.float64) + (hi >> 16) + 1)
    orec0[:, 0] -= bcx[slot0] * orec0[:, 2]
    orec0[:, 1] -= bcy[slot0] * orec0[:, 2]
    orec0[:, 3] -= bcx[slot0] * orec0[:, 5]
    orec0[:, 4] -= bcy[slot0] * orec0[:, 5]
    rkeep = (np.abs(orec0).sum(1) > 0) & ~amb0[order0]
    yield dict(g=g, ref=ref, drv=drv, raw=raw, rec_gpu=grec0[slot0[rkeep]], rec_ref=orec0[rkeep], keep=keep, drawn=drawn, amb=amb, cand=cand, fd=fd_sum, fd_ok=fd_ok & ~amb[
        [k for k, _ in cand]], gpu_loss=gpu_loss, loss64=loss64)


def test_loss_matches_fp64(diff_config):
    d = diff_config
    assert abs(d["gpu_loss"] - d["loss64"]) <= 1e-3 * d["loss64"]
    assert int(d["keep"].sum()) >= 0.95 * int(d["drawn"].sum())


def _subset(d):
    pool = np.nonzero(d["keep"])[0]
    return np.random.default_rng(121).choice(pool, size=min(12_000, len(pool)), replace=False)


def _report(name, a, b, tol, nsplat):
    rel, floor = _rel(a.ravel(), b.ravel())
    per_slot = rel.reshape(nsplat, 59)
    worst = np.argsort(rel)[::-1][:5]
    print(f"{name}: {nsplat} splats x 59 = {len(rel)} raw parameters, {100 * np.mean(rel <= tol):.3f}% within {tol} "
          f"({100 * np.mean(rel <= 1e-3):.3f}% within 1e-3, {100 * np.mean(rel <= 1e-2):.3f}% within 1e-2), floor "
          f"{floor:.3e}, worst {[(f'{rel[i]:.2e}', SLOT_NAMES[i % 59]) for i in worst]}")
    for kind, sl in (("means", slice(0, 3)), ("quaternions", slice(3, 7)), ("log-scales", slice(7, 10)),
                     ("opacity logits", slice(10, 11)), ("SH", slice(11, 59))):
        print(f"  {kind}: {100 * np.mean(per_slot[:, sl] <= tol):.3f}% within {tol}")
    return float(np.mean(rel <= tol))


def test_compositing_backward_matches_fp64_on_the_same_records(diff_config):
    """View 0 (~130k drawn splats, lists hundreds deep): the raster backward's 10 gradients per record
    against the FP64 compositing backward on the same FP32 records and the same dL/dC: >= 99.9% within
    1e-3 per component."""
    d = diff_config
    a, b = d["rec_gpu"], d["rec_ref"]
    assert len(b) > 50_000
    for j, name in enumerate(["A00", "A01", "B0", "A10", "A11", "B1", "opacity", "r", "g", "b"]):
        rel, _ = _rel(a[:, j], b[:, j])
        print(f"record d/d{name}: {100 * np.mean(rel <= REL_TOL):.3f}% within {REL_TOL}, "
              f"{100 * np.mean(rel <= 1e-4):.3f}% within 1e-4, max {rel.max():.2e}")
        assert np.mean(rel <= REL_TOL) >= 0.999


def test_raw_gradients_match_fp64_backward(diff_config):
    """A seeded 12,000 of the drawn splats, every raw parameter, against the FP64 backward of the same
    8 views on FP64 records, started from the FP32 frames' own dL/dC: >= 99.5% within 1e-3 and
    >= 99.99% within 1e-2 of max(|ref|, floor) (the FP32 records' precision; module docstring)."""
    d = diff_config
    ks = _subset(d)
    assert len(ks) >= 10_000
    assert _report("vs FP64 backward (same dL/dC)", d["g"][ks], d["drv"][ks], REL_TOL, len(ks)) >= 0.995
    rel, _ = _rel(d["g"][ks].ravel(), d["drv"][ks].ravel())
    assert np.mean(rel <= 1e-2) >= 0.9999


def test_raw_gradients_match_fp64_reference(diff_config):
    """The same parameters against the FP64 gradient of the FP64 loss: >= 99.5% within 1e-2 (the FP32
    frame's rounding moves dL/dC; see the module docstring)."""
    d = diff_config
    ks = _subset(d)
    assert _report("vs FP64 reference gradient", d["g"][ks], d["ref"][ks], 1e-2, len(ks)) >= 0.995


def test_raw_gradients_match_finite_differences(diff_config):
    """256 seeded raw parameters (raw log-scales and opacity logits included) against FP64 central
    differences (h = 1e-4) of the 8-view FP64 loss: every one within 1e-3."""
    d = diff_config
    valid = [i for i in range(len(d["cand"])) if d["fd_ok"][i]]
    excluded = len(d["cand"]) - len(valid)
    use = valid[:256]
    ks = np.array([d["cand"][i][0] for i in use])
    js = np.array([d["cand"][i][1] for i in use])
    fd = d["fd"][use]
    rel_gpu, floor = _rel(d["g"][ks, js], fd)
    rel_ref, _ = _rel(d["ref"][ks, js], fd)
    kinds = {name: int(np.sum((js >= lo) & (js < hi))) for name, lo, hi in
             (("means", 0, 3), ("quaternions", 3, 7), ("log-scales", 7, 10), ("logits", 10, 11), ("SH", 11, 59))}
    worst = np.argsort(rel_gpu)[::-1][:5]
    print(f"vs FP64 central differences: {len(use)} raw parameters {kinds} ({excluded} of {len(d['cand'])} "
          f"candidates excluded: a discrete change under +-h or an FP32/FP64 decision), GPU max rel "
          f"{rel_gpu.max():.2e}, FP64 reference max rel {rel_ref.max():.2e}, floor {floor:.3e}, worst "
          f"{[(f'{rel_gpu[i]:.2e}', SLOT_NAMES[js[i]]) for i in worst]}")
    assert len(use) == 256
    assert kinds["log-scales"] > 0 and kinds["logits"] > 0
    assert np.all(rel_ref <= REL_TOL)
    assert np.all(rel_gpu <= REL_TOL)
