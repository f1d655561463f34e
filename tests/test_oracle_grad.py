"""The oracle's FP64 reference gradient against its own FP64 central finite differences (CPU).

This pins the checker of the backward pass: the analytic gradient (back-to-front compositing
backward + the vertex stage through FP64 dual numbers) must agree with differences of the FP64 loss
wherever the perturbation changes nothing discrete."""
import math

import numpy as np
import pytest

import oracle
from splatter_gb300 import camera, synthetic


@pytest.mark.parametrize("cov,rect", [(True, True), (False, True), (True, False)])
def test_fp64_gradient_matches_central_differences(cov, rect):
    rng = np.random.default_rng(3)
    n = 2500
    rec = synthetic.plain_small(n, seed=9, sh_order=3)
    rec[:, 55:58] += 1.0  # larger splats for a small image
    sc = {k: v.astype(np.float64) for k, v in oracle.load_transform(rec).items()}
    W, H = 96, 72
    cam = camera.look_at([0.4, 0.6, -7.0], [0.0, 0.0, 0.0])
    u = oracle.uniforms(cam, W, H, fovy=math.radians(60))
    cfg = oracle.config_struct(depth_sorting=2, sh_order=3, blend_mode=1, use_covariance_for_scale=cov,
                               use_unaligned_rectangles=rect)
    g = oracle.GradContext(u, cfg, sc, np.full((H, W, 3), 0.3))
    loss, grads, _ = g.loss_and_grad(threads=4)
    assert loss > 0
    drawn = np.nonzero(np.abs(grads).sum(1) > 0)[0]
    assert len(drawn) > 500
    ok = checked = 0
    for _ in range(160):
        k = int(rng.choice(drawn))
        p = int(rng.integers(0, 59))
        valid, fd = g.fd(k, p, 1e-4)
        if not valid:
            continue
        checked += 1
        ok += abs(grads[k, p] - fd) <= 1e-3 * max(abs(fd), 1e-6)
    g.close()
    assert checked >= 120
    assert ok >= 0.98 * checked


def test_record_gradients_chain_to_parameter_gradients():
    """record_gradients() x jacobian() reproduces loss_and_grad()'s centre/rotation/scale gradients,
    opacity gradient = the record's d/dopacity (the two diagnostic outputs the GPU record-gradient
    test relies on)."""
    n = 800
    rec = synthetic.plain_small(n, seed=5, sh_order=3)
    rec[:, 55:58] += 1.0
    sc = {k: v.astype(np.float64) for k, v in oracle.load_transform(rec).items()}
    W, H = 64, 48
    cam = camera.look_at([0.4, 0.6, -7.0], [0.0, 0.0, 0.0])
    u = oracle.uniforms(cam, W, H, fovy=math.radians(60))
    cfg = oracle.config_struct(depth_sorting=2, sh_order=3, blend_mode=1)
    g = oracle.GradContext(u, cfg, sc, np.full((H, W, 3), 0.3))
    _, grads, _ = g.loss_and_grad(threads=4)
    rg, order = g.record_gradients(threads=4)
    checked = 0
    for p in range(len(order)):
        k = int(order[p])
        if not np.any(rg[p]):
            continue
        J = g.jacobian(k)
        r9 = np.concatenate([rg[p, 0:6], rg[p, 7:10]])
        np.testing.assert_allclose(J @ r9, grads[k, :10], rtol=1e-9, atol=1e-12)
        assert grads[k, 10] == pytest.approx(rg[p, 6], rel=1e-12, abs=1e-15)  # atomic order varies
        checked += 1
    g.close()
    assert checked > 100


def test_pinned_records_reproduce_the_oracles_own():
    """pin_records with the oracle's own FP64 records rounded to FP32 changes the record gradients
    only at FP32 rounding level."""
    n = 800
    rec = synthetic.plain_small(n, seed=5, sh_order=3)
    rec[:, 55:58] += 1.0
    sc = {k: v.astype(np.float64) for k, v in oracle.load_transform(rec).items()}
    W, H = 64, 48
    cam = camera.look_at([0.4, 0.6, -7.0], [0.0, 0.0, 0.0])
    u = oracle.uniforms(cam, W, H, fovy=math.radians(60))
    cfg = oracle.config_struct(depth_sorting=2, sh_order=3, blend_mode=1)
    g = oracle.GradContext(u, cfg, sc, np.full((H, W, 3), 0.3))
    rg0, order = g.record_gradients(threads=4)
    sc32 = {k: v.astype(np.float32) for k, v in sc.items()}
    recs, _, _ = oracle.preprocess(u, cfg, sc32, order, fp64=True)
    g.pin_records(recs, order)
    rg1, order1 = g.record_gradients(threads=4)
    g.close()
    assert np.array_equal(order, order1)
    live = np.abs(rg0).sum(1) > 0
    assert live.sum() > 100
    scale = np.maximum(np.abs(rg0[live]), 1e-3 * np.abs(rg0[live]).max(0))
    assert np.mean(np.abs(rg1[live] - rg0[live]) / scale <= 1e-3) >= 0.99
