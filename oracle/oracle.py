"""ctypes wrapper around oracle/_build/liboracle.so (TEST INFRASTRUCTURE ONLY).

Each function cites the reference code it restates (Lichtso/splatter).  Arrays are numpy, SoA:
centers (N,3) f32, rotations (N,4) f32 (scalar first), scales (N,3) f32, alphas (N,) f32,
sh (N,48) f32 with coefficient k of channel c at column 3k+c (shaders.wgsl:268-294).
"""
import ctypes
import os

import numpy as np

from . import build_oracle

__all__ = [
    "lib", "uniforms", "cull_keys", "draw_list", "preprocess", "raster", "raster_work", "render", "load_transform",
    "cpu_sort_fallback", "cpu_frame_timed", "expf", "GradContext", "OCFG", "UNIFORM_DTYPE", "config_struct",
    "RAW_SLOT_COLUMNS", "raw_slots", "activate64", "scene64", "raw_gradients64",
]

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        u64 = ctypes.c_uint64
        L.oracle_expf.restype = ctypes.c_float
        L.oracle_expf.argtypes = [ctypes.c_float]
        L.oracle_uniforms.restype = None
        L.oracle_uniforms.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, ctypes.c_float, P]
        L.oracle_cull_keys.restype = None
        L.oracle_cull_keys.argtypes = [P, ctypes.c_int, P, u64, P, P]
        L.oracle_draw_list.restype = None
        L.oracle_draw_list.argtypes = [P, ctypes.c_int, P, u64, P, P, P, P]
        for name in ("oracle_preprocess_f32", "oracle_preprocess_f64"):
            f = getattr(L, name)
            f.restype = u64
            f.argtypes = [P, P, P, P, P, P, P, P, u64, P, P, ctypes.c_int]
        L.oracle_raster.restype = None
        L.oracle_raster.argtypes = [P, P, P, u64, P, ctypes.c_int]
        L.oracle_raster_work.restype = None
        L.oracle_raster_work.argtypes = [P, P, P, u64, ctypes.c_int, P]
        L.oracle_render.restype = u64
        L.oracle_render.argtypes = [P, P, P, P, P, P, P, u64, P, ctypes.c_int, P]
        L.oracle_load_transform.restype = None
        L.oracle_load_transform.argtypes = [P, u64, P, P, P, P, P]
        L.oracle_cpu_sort_fallback.restype = u64
        L.oracle_cpu_sort_fallback.argtypes = [P, P, u64, P]
        L.oracle_cpu_frame_timed.restype = u64
        L.oracle_cpu_frame_timed.argtypes = [P, P, P, P, P, P, P, u64, P, ctypes.c_int, ctypes.c_int, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# 224-byte uniform block (renderer.rs:49-61).
UNIFORM_DTYPE = np.dtype([
    ("camera", "<f4", 16), ("view", "<f4", 16), ("vp", "<f4", 16), ("view_size", "<f4", 2),
    ("image_size", "<u4", 2), ("tol", "<f4"), ("bias", "<f4"), ("margin", "<f4"), ("splat_scale", "<f4"),
])
assert UNIFORM_DTYPE.itemsize == 224

OCFG = np.dtype([("depth_sorting", "<i4"), ("use_covariance_for_scale", "<i4"),
                 ("use_unaligned_rectangles", "<i4"), ("sh_order", "<i4"), ("blend_mode", "<i4")])


def config_struct(depth_sorting=2, use_covariance_for_scale=True, use_unaligned_rectangles=True, sh_order=3,
                  blend_mode=0):
    c = np.zeros(1, OCFG)
    c["depth_sorting"] = int(depth_sorting)
    c["use_covariance_for_scale"] = int(bool(use_covariance_for_scale))
    c["use_unaligned_rectangles"] = int(bool(use_unaligned_rectangles))
    c["sh_order"] = int(sh_order)
    c["blend_mode"] = int(blend_mode)
    return c


def expf(x):
    return lib().oracle_expf(float(x))


def uniforms(cam_to_world, width, height, fovy=np.pi / 2, tol=1.1, margin=2.0, splat_scale=1.0):
    """Frame uniforms (renderer.rs:364-409, utils.rs:45-70); cam_to_world is (4,4) column-major
    flattened to 16 floats (columns: right, up, forward, position)."""
    cam = _c(np.asarray(cam_to_world, np.float32).reshape(16), np.float32)
    u = np.zeros(1, UNIFORM_DTYPE)
    lib().oracle_uniforms(_p(cam), int(width), int(height), float(fovy), float(tol), float(margin),
                          float(splat_scale), _p(u))
    return u


def cull_keys(u, mode, centers):
    """Per-splat key and visibility (shaders.wgsl:318-324 or renderer.rs:372-392 for mode 1)."""
    c = _c(centers, np.float32)
    n = c.shape[0]
    keys = np.empty(n, np.uint32)
    vis = np.empty(n, np.uint8)
    lib().oracle_cull_keys(_p(u), int(mode), _p(c), n, _p(keys), _p(vis))
    return keys, vis.astype(bool)


def draw_list(u, mode, centers):
    """Ordered visible entries (key, index), V and draw count for a depth-sorting mode."""
    c = _c(centers, np.float32)
    n = c.shape[0]
    keys = np.empty(max(n, 1), np.uint32)
    idx = np.empty(max(n, 1), np.uint32)
    nv = np.zeros(1, np.uint64)
    nd = np.zeros(1, np.uint64)
    lib().oracle_draw_list(_p(u), int(mode), _p(c), n, _p(keys), _p(idx), _p(nv), _p(nd))
    v = int(nv[0])
    return keys[:v].copy(), idx[:v].copy(), v, int(nd[0])


def preprocess(u, cfg, scene, idx, fp64=False, threads=8):
    """Vertex-stage restatement (shaders.wgsl:507-573) for splat indices idx.

    Returns (records (n,16) f32, dbg (n,18) = M[9] t[2] rot[2] axes[2] rgb[3], n_valid)."""
    centers, rots, scales, alphas, shs = (_c(scene[k], np.float32) for k in ("center", "rotation", "scale",
                                                                            "alpha", "sh"))
    idx = _c(idx, np.uint32)
    n = idx.shape[0]
    recs = np.empty((max(n, 1), 16), np.float32)
    dbg = np.empty((max(n, 1), 18), np.float64 if fp64 else np.float32)
    f = lib().oracle_preprocess_f64 if fp64 else lib().oracle_preprocess_f32
    nvalid = f(_p(u), _p(cfg), _p(centers), _p(rots), _p(scales), _p(alphas), _p(shs), _p(idx), n, _p(recs),
               _p(dbg), int(threads))
    return recs[:n], dbg[:n], int(nvalid)


def raster(u, cfg, records, threads=8):
    W, H = (int(x) for x in u["image_size"][0])
    recs = _c(records, np.float32).reshape(-1, 16)
    if int(cfg["blend_mode"][0]) == 0:
        out = np.zeros((H, W, 4), np.uint8)
    else:
        out = np.zeros((H, W, 4), np.float32)
    lib().oracle_raster(_p(u), _p(cfg), _p(recs), recs.shape[0], _p(out), int(threads))
    return out


def raster_work(u, cfg, records, threads=8):
    """The raster's work for a frame's records in draw order (not a reference function; the
    algorithmic unit of the raster's compute roofline): `box` (pixel, record) pairs with the pixel
    inside the record's pixel box, `covered` those whose pixel centre passes the coverage test of
    shaders.wgsl:580-583 (all of them, also after the pixel has finished), `blended` the blend steps
    the pixels perform (coverage, alpha >= 1/255, before the pixel finishes)."""
    recs = _c(records, np.float32).reshape(-1, 16)
    work = np.zeros(3, np.uint64)
    lib().oracle_raster_work(_p(u), _p(cfg), _p(recs), recs.shape[0], int(threads), _p(work))
    return {"box": int(work[0]), "covered": int(work[1]), "blended": int(work[2])}


def render(u, cfg, scene, threads=8):
    """Whole frame through the restated pipeline; returns (image, (V, n_draw, n_valid))."""
    centers, rots, scales, alphas, shs = (_c(scene[k], np.float32) for k in ("center", "rotation", "scale",
                                                                            "alpha", "sh"))
    W, H = (int(x) for x in u["image_size"][0])
    if int(cfg["blend_mode"][0]) == 0:
        out = np.zeros((H, W, 4), np.uint8)
    else:
        out = np.zeros((H, W, 4), np.float32)
    stats = np.zeros(3, np.uint64)
    lib().oracle_render(_p(u), _p(cfg), _p(centers), _p(rots), _p(scales), _p(alphas), _p(shs),
                        centers.shape[0], _p(out), int(threads), _p(stats))
    return out, tuple(int(s) for s in stats)


def load_transform(records):
    """Scene::load_chunk transform (scene.rs:225-250) of (N,62) f32 PLY records into SoA arrays."""
    r = _c(records, np.float32).reshape(-1, 62)
    n = r.shape[0]
    out = {
        "center": np.empty((n, 3), np.float32), "rotation": np.empty((n, 4), np.float32),
        "scale": np.empty((n, 3), np.float32), "alpha": np.empty(n, np.float32),
        "sh": np.empty((n, 48), np.float32),
    }
    lib().oracle_load_transform(_p(r), n, _p(out["center"]), _p(out["rotation"]), _p(out["scale"]),
                                _p(out["alpha"]), _p(out["sh"]))
    return out


# Raw parameters in the 59-slot order of the gradient context (centre 3, quaternion 4, log-scale 3,
# opacity logit, SH 48): their columns in the 62-float file record (scene.rs:15-24).
RAW_SLOT_COLUMNS = np.array([0, 1, 2, 58, 59, 60, 61, 55, 56, 57, 54] + list(range(6, 54)))


def raw_slots(records):
    """(N, 59) raw parameters of (N, 62) file records in slot order, as float64."""
    return np.asarray(records, np.float64).reshape(-1, 62)[:, RAW_SLOT_COLUMNS]


def activate64(raw):
    """The loader's transform (scene.rs:225-250) in FP64 on (N, 59) raw slots: the activated slots
    (centre, unit rotation, scale = exp(clamp(log-scale, mean -+ 5)), opacity = sigmoid(logit), SH)."""
    raw = np.asarray(raw, np.float64).reshape(-1, 59)
    out = raw.copy()
    q = raw[:, 3:7]
    out[:, 3:7] = q / np.sqrt((q * q).sum(1, keepdims=True))
    ls = raw[:, 7:10]
    avg = ls.sum(1, keepdims=True) / 3.0
    out[:, 7:10] = np.exp(np.clip(ls, avg - 5.0, avg + 5.0))
    out[:, 10] = 1.0 / (1.0 + np.exp(-raw[:, 10]))
    return out


def scene64(activated):
    """The gradient context's scene dict of (N, 59) activated slots."""
    a = np.asarray(activated, np.float64)
    return {"center": a[:, 0:3], "rotation": a[:, 3:7], "scale": a[:, 7:10], "alpha": a[:, 10], "sh": a[:, 11:59]}


def raw_gradients64(raw, grads):
    """Chain rule of activate64: gradients of the activated slots (N, 59) -> gradients of the raw slots."""
    raw = np.asarray(raw, np.float64).reshape(-1, 59)
    g = np.array(grads, np.float64).reshape(-1, 59)
    out = g.copy()
    q = raw[:, 3:7]
    nq = np.sqrt((q * q).sum(1, keepdims=True))
    r = q / nq
    gr = g[:, 3:7]
    out[:, 3:7] = (gr - (gr * r).sum(1, keepdims=True) * r) / nq
    ls = raw[:, 7:10]
    avg = ls.sum(1, keepdims=True) / 3.0
    clamped = (ls < avg - 5.0) | (ls > avg + 5.0)
    s = np.exp(np.clip(ls, avg - 5.0, avg + 5.0))
    gs = g[:, 7:10] * s
    out[:, 7:10] = np.where(clamped, 0.0, gs) + np.where(clamped, gs, 0.0).sum(1, keepdims=True) / 3.0
    a = 1.0 / (1.0 + np.exp(-raw[:, 10]))
    out[:, 10] = g[:, 10] * a * (1.0 - a)
    return out


def cpu_frame_timed(u, cfg, scene, threads=8, tile_stride=1):
    """The reference's CPU path for one frame (CPU depth-sort fallback + restated vertex/fragment/blend),
    timed per stage; returns (image, V, (t_sort, t_vertex, t_raster) seconds)."""
    centers, rots, scales, alphas, shs = (_c(scene[k], np.float32) for k in ("center", "rotation", "scale",
                                                                            "alpha", "sh"))
    W, H = (int(x) for x in u["image_size"][0])
    out = np.zeros((H, W, 4), np.uint8 if int(cfg["blend_mode"][0]) == 0 else np.float32)
    secs = np.zeros(3, np.float64)
    v = lib().oracle_cpu_frame_timed(_p(u), _p(cfg), _p(centers), _p(rots), _p(scales), _p(alphas), _p(shs),
                                     centers.shape[0], _p(out), int(threads), int(tile_stride), _p(secs))
    return out, int(v), tuple(float(x) for x in secs)


def cpu_sort_fallback(u, positions):
    """The reference's CPU depth-sort fallback (renderer.rs:372-395): (V,2) u32 entries (key, index)."""
    p = _c(positions, np.float32)
    n = p.shape[0]
    ent = np.empty((max(n, 1), 2), np.uint32)
    v = lib().oracle_cpu_sort_fallback(_p(u), _p(p), n, _p(ent))
    return ent[:v]


class GradContext:
    """FP64 reference gradients and finite differences of the fp32-blend frame (TEST INFRASTRUCTURE).

    Parameters per splat (59): centre 3, rotation 4 (as given), scale 3, opacity 1, SH 48.  The loss is
    sum over pixels and RGB of (C - target)^2; target is (H, W, 3) float64."""

    NPARAM = 59

    def __init__(self, u, cfg, scene64, target):
        L = lib()
        if not hasattr(L, "_grad_bound"):
            P = ctypes.c_void_p
            L.oracle_grad_create.restype = P
            L.oracle_grad_create.argtypes = [P, P, ctypes.c_uint64, P, P, P, P, P, P]
            L.oracle_grad_destroy.restype = None
            L.oracle_grad_destroy.argtypes = [P]
            L.oracle_grad_loss.restype = ctypes.c_double
            L.oracle_grad_loss.argtypes = [P, P, P, ctypes.c_int]
            L.oracle_grad_fd.restype = ctypes.c_int
            L.oracle_grad_fd.argtypes = [P, ctypes.c_uint64, ctypes.c_int, ctypes.c_double, P]
            L.oracle_grad_set_image_gradient.restype = None
            L.oracle_grad_set_image_gradient.argtypes = [P, P]
            L.oracle_grad_fd_params.restype = ctypes.c_int
            L.oracle_grad_fd_params.argtypes = [P, ctypes.c_uint64, P, P, ctypes.c_double, P]
            L.oracle_grad_pin_records.restype = None
            L.oracle_grad_pin_records.argtypes = [P, P, P, ctypes.c_uint64]
            L.oracle_grad_jacobian.restype = None
            L.oracle_grad_jacobian.argtypes = [P, ctypes.c_uint64, P]
            L.oracle_grad_loss_ex.restype = ctypes.c_double
            L.oracle_grad_loss_ex.argtypes = [P, P, P, ctypes.c_int, P, P]
            L.oracle_grad_ambiguous.restype = ctypes.c_uint64
            L.oracle_grad_ambiguous.argtypes = [P, P, ctypes.c_int]
            L._grad_bound = True
        self._keep = [np.ascontiguousarray(scene64[k], np.float64) for k in ("center", "rotation", "scale", "alpha",
                                                                             "sh")]
        self.n = self._keep[0].shape[0]
        self.W, self.H = (int(x) for x in u["image_size"][0])
        tgt = np.ascontiguousarray(target, np.float64).reshape(self.H, self.W, 3)
        self._h = L.oracle_grad_create(_p(u), _p(cfg), self.n, *(_p(a) for a in self._keep), _p(tgt))

    def loss_and_grad(self, threads=8):
        grads = np.zeros((self.n, self.NPARAM), np.float64)
        image = np.zeros((self.H, self.W, 4), np.float64)
        loss = lib().oracle_grad_loss(self._h, _p(grads), _p(image), int(threads))
        return loss, grads, image

    def record_gradients(self, threads=8):
        """(per draw position the 10 record gradients, A against pixel-centre coordinates; splat index
        of each draw position)."""
        nd = self.n
        rg = np.zeros((nd, 10), np.float64)
        order = np.zeros(nd, np.uint32)
        lib().oracle_grad_loss_ex(self._h, None, None, int(threads), _p(rg), _p(order))
        return rg, order

    def pin_records(self, records16, splat_idx):
        """Composite (and differentiate the compositing) in FP64 on these FP32 records (16 floats per
        splat, renderer layout) instead of the oracle's own FP64 records; the vertex-stage Jacobian
        stays the FP64 one."""
        rec = np.ascontiguousarray(records16, np.float32).reshape(-1, 16)
        idx = np.ascontiguousarray(splat_idx, np.uint32)
        assert rec.shape[0] == idx.shape[0]
        lib().oracle_grad_pin_records(self._h, _p(rec), _p(idx), rec.shape[0])

    def jacobian(self, k):
        """(10, 9) FP64 Jacobian of splat k's record (A00, A01, B0, A10, A11, B1, r, g, b; A against
        pixel-centre coordinates) in its centre, rotation and scale."""
        J = np.zeros((10, 9), np.float64)
        lib().oracle_grad_jacobian(self._h, int(k), _p(J))
        return J

    def ambiguous(self, threads=8):
        """(flags per splat, #pixels) where the FP32 frame and the FP64 frame differ in a decision."""
        flags = np.zeros(self.n, np.uint8)
        npix = lib().oracle_grad_ambiguous(self._h, _p(flags), int(threads))
        return flags.astype(bool), int(npix)

    def fd(self, k, param, h=1e-4):
        out = np.zeros(1, np.float64)
        ok = lib().oracle_grad_fd(self._h, int(k), int(param), float(h), _p(out))
        return bool(ok), float(out[0])

    def set_image_gradient(self, grad_image):
        """Use grad_image (H, W, 3) as dL/dC in the backward (None: 2 (C - target) of the FP64 frame)."""
        if grad_image is None:
            lib().oracle_grad_set_image_gradient(self._h, None)
            return
        self._gimg = np.ascontiguousarray(grad_image, np.float64).reshape(self.H, self.W, 3)
        lib().oracle_grad_set_image_gradient(self._h, _p(self._gimg))

    def fd_params(self, k, p_plus, p_minus, denom):
        """(loss(p_plus) - loss(p_minus)) / denom for splat k's 59 activated parameters; (ok, value)."""
        pp = np.ascontiguousarray(p_plus, np.float64).reshape(self.NPARAM)
        pm = np.ascontiguousarray(p_minus, np.float64).reshape(self.NPARAM)
        out = np.zeros(1, np.float64)
        ok = lib().oracle_grad_fd_params(self._h, int(k), _p(pp), _p(pm), float(denom), _p(out))
        return bool(ok), float(out[0])

    def close(self):
        if getattr(self, "_h", None):
            lib().oracle_grad_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
