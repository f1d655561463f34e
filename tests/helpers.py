"""Shared helpers for the parity tests: seeded scenes, poses and the GPU/oracle pair runs."""
import math

import numpy as np

from splatter_gb300 import camera, synthetic


def scene_from_splats60(s60):
    return {"center": np.ascontiguousarray(s60[:, 4:7]), "rotation": np.ascontiguousarray(s60[:, 0:4]),
            "scale": np.ascontiguousarray(s60[:, 8:11]), "alpha": np.ascontiguousarray(s60[:, 11]),
            "sh": np.ascontiguousarray(s60[:, 12:60])}


def oracle_cfg(oracle, config):
    return oracle.config_struct(depth_sorting=int(config.depth_sorting),
                                use_covariance_for_scale=config.use_covariance_for_scale,
                                use_unaligned_rectangles=config.use_unaligned_rectangles,
                                sh_order=config.spherical_harmonics_order, blend_mode=int(config.blend_mode))


def oracle_uniforms(oracle, config, cam, w, h):
    return oracle.uniforms(cam, w, h, fovy=config.field_of_view_y, tol=config.frustum_culling_tolerance,
                           margin=config.ellipse_margin, splat_scale=config.splat_scale)


def small_scene_records(n, seed=0, sh_order=3):
    """Gaussian blob of n splats (config 'plain small' distribution, optional higher SH bands)."""
    return synthetic.plain_small(n, seed=seed, sh_order=sh_order)


def default_cam(dist=8.0, az=0.3, el=0.2):
    eye = [dist * math.cos(el) * math.sin(az), dist * math.sin(el), -dist * math.cos(el) * math.cos(az)]
    return camera.look_at(eye, [0.0, 0.0, 0.0])


def image_psnr(a, b):
    a = np.asarray(a, np.float64)[..., :3] / 255.0
    b = np.asarray(b, np.float64)[..., :3] / 255.0
    mse = float(np.mean((a - b) ** 2))
    return float("inf") if mse == 0 else 10.0 * math.log10(1.0 / mse)
