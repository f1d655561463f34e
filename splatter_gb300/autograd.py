"""Differentiable rendering: torch.autograd.Function over the hand-written backward kernels.

`render_splats` takes the splat parameters the renderer uses (centres, rotations as given, scales,
opacities, SH) and returns the float4 image of an fp32-blend frame; its backward calls
spl_render_backward (raster backward + vertex-stage backward on the GPU).  `render_raw` applies the
file loader's activations first (Scene::load_chunk, scene.rs:225-250: rotor normalisation, exp of the
log-scales clamped to mean +- 5, sigmoid of the opacity logit) with the loader's own arithmetic on the
GPU (spl_activate_splats) and chains its backward there too (spl_activate_splats_backward), so
gradients reach the raw parameters a training loop optimises without torch elementwise kernels per
frame.  `render_raw_views` renders several views of the same raw parameters in one autograd node and
sums their gradients in place on the GPU (spl_render_backward_accumulate).  `l2_image_loss` is the
L2 loss of such frames against RGB targets, one pass each way (spl_l2_image_loss).  `activate` is
the same transform written in torch (a reference).  Depth order, culling and the 1/255 discard are
constants of the frame (no gradient), as in any splat rasteriser.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check
from .renderer import BlendMode, Renderer, _stream_ptr

__all__ = ["render_splats", "render_raw", "render_raw_views", "activate", "activate_native", "l2_image_loss"]


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class _WrappedScene:
    """A scene over caller-owned device tensors (spl_scene_wrap); keeps the tensors alive."""

    def __init__(self, renderer, xyz, rot, scale_alpha, sh):
        self._lib = _lib.load()
        self._keep = (xyz, rot, scale_alpha, sh)
        n = rot.shape[0]
        h = ctypes.c_void_p()
        check(self._lib.spl_scene_wrap(renderer.handle, n, _ptr(xyz[0]), _ptr(xyz[1]), _ptr(xyz[2]), _ptr(rot),
                                       _ptr(scale_alpha), _ptr(sh), ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.spl_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _import_torch():
    import torch
    return torch


class _RenderSplats:  # built lazily so that importing the package does not import torch
    fn = None

    @classmethod
    def get(cls):
        if cls.fn is None:
            torch = _import_torch()

            class RenderSplats(torch.autograd.Function):
                @staticmethod
                def forward(ctx, xyz, rot, scale_alpha, sh, renderer, camera_to_world, width, height):
                    xyz = xyz.contiguous()
                    rot = rot.contiguous()
                    scale_alpha = scale_alpha.contiguous()
                    sh = sh.contiguous()
                    scene = _WrappedScene(renderer, xyz, rot, scale_alpha, sh)
                    img = renderer.render_frame(scene, camera_to_world, width, height)
                    ctx.renderer = renderer
                    ctx.scene = scene
                    ctx.cam = np.ascontiguousarray(np.asarray(camera_to_world, np.float32).reshape(16))
                    ctx.size = (width, height)
                    ctx.save_for_backward(img)
                    renderer._last_frame_key = (id(scene), ctx.cam.tobytes(), width, height)
                    return img

                @staticmethod
                def backward(ctx, grad_img):
                    (img,) = ctx.saved_tensors
                    _frame_ready(ctx)
                    r = ctx.renderer
                    xyz, rot, sa, sh = ctx.scene._keep
                    gxyz = torch.zeros_like(xyz)
                    grot = torch.zeros_like(rot)
                    gsa = torch.zeros_like(sa)
                    gsh = torch.zeros_like(sh)
                    g = grad_img.contiguous().float()
                    check(r._lib.spl_render_backward(r.handle, ctx.scene.handle, _ptr(img), _ptr(g), _ptr(gxyz[0]),
                                                     _ptr(gxyz[1]), _ptr(gxyz[2]), _ptr(grot), _ptr(gsa), _ptr(gsh),
                                                     _stream_ptr(None)))
                    return gxyz, grot, gsa, gsh, None, None, None, None

            cls.fn = RenderSplats
        return cls.fn


def _ensure_frame(r, scene, cam, w, h):
    """Re-renders (scene, cam) on renderer r if r has rendered another frame since: the backward
    reuses the renderer's frame state (sorted pairs, records, tile ranges)."""
    key = (id(scene), cam.tobytes(), w, h)
    if getattr(r, "_last_frame_key", None) != key:
        r.render_frame(scene, cam, w, h)  # deterministic: the same frame again
        r._last_frame_key = key


def _frame_ready(ctx):
    """Re-renders the frame of this autograd node if the renderer has rendered another one since."""
    _ensure_frame(ctx.renderer, ctx.scene, ctx.cam, *ctx.size)


class _RenderRaw:  # built lazily, like _RenderSplats
    fn = None

    @classmethod
    def get(cls):
        if cls.fn is None:
            torch = _import_torch()

            class RenderRaw(torch.autograd.Function):
                @staticmethod
                def forward(ctx, means, quats, log_scales, logits, sh, renderer, camera_to_world, width, height):
                    means, quats, log_scales, logits, sh = (t.contiguous() for t in (means, quats, log_scales, logits,
                                                                                      sh))
                    n = quats.shape[0]
                    f32 = dict(device=quats.device, dtype=torch.float32)
                    xyz = torch.empty((3, n), **f32)
                    rot = torch.empty((n, 4), **f32)
                    sa = torch.empty((n, 4), **f32)
                    lib = _lib.load()
                    check(lib.spl_activate_splats(n, _ptr(means), _ptr(quats), _ptr(log_scales), _ptr(logits),
                                                  _ptr(xyz[0]), _ptr(xyz[1]), _ptr(xyz[2]), _ptr(rot), _ptr(sa),
                                                  _stream_ptr(None)))
                    scene = _WrappedScene(renderer, xyz, rot, sa, sh)
                    img = renderer.render_frame(scene, camera_to_world, width, height)
                    ctx.renderer = renderer
                    ctx.scene = scene
                    ctx.cam = np.ascontiguousarray(np.asarray(camera_to_world, np.float32).reshape(16))
                    ctx.size = (width, height)
                    ctx.save_for_backward(img, quats, log_scales)
                    renderer._last_frame_key = (id(scene), ctx.cam.tobytes(), width, height)
                    return img

                @staticmethod
                def backward(ctx, grad_img):
                    img, quats, log_scales = ctx.saved_tensors
                    _frame_ready(ctx)
                    r = ctx.renderer
                    xyz, rot, sa, sh = ctx.scene._keep
                    n = rot.shape[0]
                    gxyz = torch.zeros_like(xyz)
                    grot = torch.zeros_like(rot)
                    gsa = torch.zeros_like(sa)
                    gsh = torch.zeros_like(sh)
                    g = grad_img.contiguous().float()
                    st = _stream_ptr(None)
                    check(r._lib.spl_render_backward(r.handle, ctx.scene.handle, _ptr(img), _ptr(g), _ptr(gxyz[0]),
                                                     _ptr(gxyz[1]), _ptr(gxyz[2]), _ptr(grot), _ptr(gsa), _ptr(gsh),
                                                     st))
                    g_means = torch.empty((n, 3), device=rot.device, dtype=torch.float32)
                    g_quats = torch.empty((n, 4), device=rot.device, dtype=torch.float32)
                    g_logs = torch.empty((n, 3), device=rot.device, dtype=torch.float32)
                    g_logits = torch.empty((n,), device=rot.device, dtype=torch.float32)
                    check(r._lib.spl_activate_splats_backward(n, _ptr(quats), _ptr(log_scales), _ptr(rot), _ptr(sa),
                                                              _ptr(gxyz[0]), _ptr(gxyz[1]), _ptr(gxyz[2]),
                                                              _ptr(grot), _ptr(gsa), _ptr(g_means), _ptr(g_quats),
                                                              _ptr(g_logs), _ptr(g_logits), st))
                    return g_means, g_quats, g_logs, g_logits, gsh, None, None, None, None

            cls.fn = RenderRaw
        return cls.fn


class _RenderRawViews:  # built lazily, like _RenderSplats
    fn = None

    @classmethod
    def get(cls):
        if cls.fn is None:
            torch = _import_torch()

            class RenderRawViews(torch.autograd.Function):
                @staticmethod
                def forward(ctx, means, quats, log_scales, logits, sh, renderers, cameras, width, height):
                    means, quats, log_scales, logits, sh = (t.contiguous() for t in (means, quats, log_scales, logits,
                                                                                      sh))
                    n = quats.shape[0]
                    f32 = dict(device=quats.device, dtype=torch.float32)
                    xyz = torch.empty((3, n), **f32)
                    rot = torch.empty((n, 4), **f32)
                    sa = torch.empty((n, 4), **f32)
                    lib = _lib.load()
                    check(lib.spl_activate_splats(n, _ptr(means), _ptr(quats), _ptr(log_scales), _ptr(logits),
                                                  _ptr(xyz[0]), _ptr(xyz[1]), _ptr(xyz[2]), _ptr(rot), _ptr(sa),
                                                  _stream_ptr(None)))
                    out = torch.empty((len(cameras), height, width, 4), **f32)
                    scenes, views = {}, []
                    for v, cam in enumerate(cameras):
                        r = renderers[v % len(renderers)]
                        if id(r) not in scenes:
                            scenes[id(r)] = _WrappedScene(r, xyz, rot, sa, sh)
                        scene = scenes[id(r)]
                        c = np.ascontiguousarray(np.asarray(cam, np.float32).reshape(16))
                        r.render_frame(scene, c, width, height, out=out[v])
                        r._last_frame_key = (id(scene), c.tobytes(), width, height)
                        views.append((r, scene, c))
                    ctx.views = views
                    ctx.size = (width, height)
                    ctx.save_for_backward(out, quats, log_scales)
                    return out

                @staticmethod
                def backward(ctx, grad_out):
                    out, quats, log_scales = ctx.saved_tensors
                    w, h = ctx.size
                    xyz, rot, sa, sh = ctx.views[0][1]._keep
                    n = rot.shape[0]
                    gxyz = torch.zeros_like(xyz)
                    grot = torch.zeros_like(rot)
                    gsa = torch.zeros_like(sa)
                    gsh = torch.zeros_like(sh)
                    g = grad_out.contiguous().float()
                    st = _stream_ptr(None)
                    # the views in order, each adding its gradients in place
                    for v, (r, scene, c) in enumerate(ctx.views):
                        _ensure_frame(r, scene, c, w, h)
                        check(r._lib.spl_render_backward_accumulate(r.handle, scene.handle, _ptr(out[v]), _ptr(g[v]),
                                                                    _ptr(gxyz[0]), _ptr(gxyz[1]), _ptr(gxyz[2]),
                                                                    _ptr(grot), _ptr(gsa), _ptr(gsh), st))
                    g_means = torch.empty((n, 3), device=rot.device, dtype=torch.float32)
                    g_quats = torch.empty((n, 4), device=rot.device, dtype=torch.float32)
                    g_logs = torch.empty((n, 3), device=rot.device, dtype=torch.float32)
                    g_logits = torch.empty((n,), device=rot.device, dtype=torch.float32)
                    check(_lib.load().spl_activate_splats_backward(n, _ptr(quats), _ptr(log_scales), _ptr(rot),
                                                                   _ptr(sa), _ptr(gxyz[0]), _ptr(gxyz[1]),
                                                                   _ptr(gxyz[2]), _ptr(grot), _ptr(gsa),
                                                                   _ptr(g_means), _ptr(g_quats), _ptr(g_logs),
                                                                   _ptr(g_logits), st))
                    return g_means, g_quats, g_logs, g_logits, gsh, None, None, None, None

            cls.fn = RenderRawViews
        return cls.fn


def render_splats(xyz, rotation, scale_alpha, sh, renderer: Renderer, camera_to_world, width, height):
    """Differentiable frame.  xyz: (3, N) centre planes; rotation: (N, 4) scalar first; scale_alpha:
    (N, 4) scale xyz + opacity; sh: (N, 48).  Returns (H, W, 4) float32 (r, g, b, T)."""
    if renderer.config.blend_mode != BlendMode.FP32:
        raise ValueError("render_splats needs a renderer with blend_mode FP32")
    return _RenderSplats.get().apply(xyz, rotation, scale_alpha, sh, renderer, camera_to_world, width, height)


def activate_native(means, quats, log_scales, opacity_logits):
    """The loader's activations on the GPU (spl_activate_splats, no autograd): (xyz planes (3, N),
    rotation (N, 4), scale_alpha (N, 4)), bit for bit the arrays of a scene loaded from records."""
    torch = _import_torch()
    means, quats, log_scales, opacity_logits = (t.detach().contiguous() for t in (means, quats, log_scales,
                                                                                  opacity_logits))
    n = quats.shape[0]
    f32 = dict(device=quats.device, dtype=torch.float32)
    xyz, rot, sa = torch.empty((3, n), **f32), torch.empty((n, 4), **f32), torch.empty((n, 4), **f32)
    check(_lib.load().spl_activate_splats(n, _ptr(means), _ptr(quats), _ptr(log_scales), _ptr(opacity_logits),
                                          _ptr(xyz[0]), _ptr(xyz[1]), _ptr(xyz[2]), _ptr(rot), _ptr(sa),
                                          _stream_ptr(None)))
    return xyz, rot, sa


def activate(means, quats, log_scales, opacity_logits):
    """The loader's activations (scene.rs:225-250) in torch: (xyz planes, rotation, scale_alpha)."""
    torch = _import_torch()
    rot = quats * (1.0 / torch.sqrt((quats * quats).sum(-1, keepdim=True)))
    avg = log_scales.sum(-1, keepdim=True) / 3.0
    ls = torch.minimum(torch.maximum(log_scales, avg - 5.0), avg + 5.0)
    scale = torch.exp(ls)
    alpha = torch.sigmoid(opacity_logits)
    return means.t(), rot, torch.cat([scale, alpha[:, None]], 1)


def render_raw(means, quats, log_scales, opacity_logits, sh, renderer, camera_to_world, width, height):
    """Differentiable frame from raw parameters: means (N, 3), quaternions (N, 4, scalar first),
    log-scales (N, 3), opacity logits (N,), SH (N, 48), all float32 CUDA tensors.  The frame equals the
    frame of a scene loaded from the same file records; gradients reach every raw parameter."""
    if renderer.config.blend_mode != BlendMode.FP32:
        raise ValueError("render_raw needs a renderer with blend_mode FP32")
    for t, shape in ((means, 3), (quats, 4), (log_scales, 3), (sh, 48)):
        if t.dim() != 2 or t.shape[1] != shape or t.dtype.itemsize != 4 or not t.is_cuda:
            raise ValueError("render_raw: float32 CUDA tensors (N, 3), (N, 4), (N, 3), (N,), (N, 48) expected")
    return _RenderRaw.get().apply(means, quats, log_scales, opacity_logits, sh, renderer, camera_to_world, width,
                                  height)


def render_raw_views(means, quats, log_scales, opacity_logits, sh, renderers, cameras, width, height):
    """render_raw over several views of the same parameters in one autograd node: returns
    (len(cameras), H, W, 4) float32.  The backward adds every view's gradients into one set of arrays
    in place (spl_render_backward_accumulate), view after view, and chains the loader's activations
    once, instead of a gradient array per view that autograd zeroes and sums.  `renderers`: one
    Renderer, or a sequence used round robin over the views; a renderer keeps the frame state of the
    last view it rendered, so with fewer renderers than views the backward renders the other views
    again (same frames).  Gradients equal the per-view render_raw gradients summed over the views, to
    rounding: the raster backward sums with float atomics, and the activations' chain rule is
    applied to the sum instead of to each view."""
    if isinstance(renderers, Renderer):
        renderers = [renderers]
    renderers = list(renderers)
    cameras = list(cameras)
    if not renderers or not cameras:
        raise ValueError("render_raw_views: at least one renderer and one camera")
    if any(r.config.blend_mode != BlendMode.FP32 for r in renderers):
        raise ValueError("render_raw_views needs renderers with blend_mode FP32")
    for t, shape in ((means, 3), (quats, 4), (log_scales, 3), (sh, 48)):
        if t.dim() != 2 or t.shape[1] != shape or t.dtype.itemsize != 4 or not t.is_cuda:
            raise ValueError("render_raw_views: float32 CUDA tensors (N, 3), (N, 4), (N, 3), (N,), (N, 48) expected")
    return _RenderRawViews.get().apply(means, quats, log_scales, opacity_logits, sh, renderers, cameras, width,
                                       height)


class _L2ImageLoss:  # built lazily, like _RenderSplats
    fn = None

    @classmethod
    def get(cls):
        if cls.fn is None:
            torch = _import_torch()

            class L2ImageLoss(torch.autograd.Function):
                @staticmethod
                def forward(ctx, images, targets):
                    images, targets = images.contiguous(), targets.contiguous()
                    pixels = images.numel() // 4
                    lib = _lib.load()
                    partial = torch.empty(int(lib.spl_l2_image_loss_partials(pixels)), device=images.device,
                                          dtype=torch.float32)
                    check(lib.spl_l2_image_loss(_ptr(images), _ptr(targets), pixels, _ptr(partial), _stream_ptr(None)))
                    ctx.save_for_backward(images, targets)
                    return partial.sum()

                @staticmethod
                def backward(ctx, grad_loss):
                    images, targets = ctx.saved_tensors
                    grad = torch.empty_like(images)
                    scale = grad_loss.detach().to(torch.float32).contiguous()
                    check(_lib.load().spl_l2_image_loss_backward(_ptr(images), _ptr(targets), images.numel() // 4,
                                                                 _ptr(scale), _ptr(grad), _stream_ptr(None)))
                    return grad, None

            cls.fn = L2ImageLoss
        return cls.fn


def l2_image_loss(images, targets):
    """sum over pixels and RGB of (images[..., :3] - targets)^2 for float4 frames (..., 4) (r, g, b, T),
    such as render_raw_views returns, against float32 RGB targets (..., 3): the value of
    ((images[..., :3] - targets) ** 2).sum() (summed in another order) with the same gradient bit for
    bit, (2 (image - target) * upstream, 0), each way in one pass over the frames."""
    if images.dim() < 1 or images.shape[-1] != 4 or targets.shape[-1] != 3 or images.shape[:-1] != targets.shape[:-1]:
        raise ValueError("l2_image_loss: images (..., 4) and targets (..., 3) with the same leading shape expected")
    torch = _import_torch()
    if images.dtype != torch.float32 or targets.dtype != torch.float32 or not images.is_cuda or not targets.is_cuda:
        raise ValueError("l2_image_loss: float32 CUDA tensors expected")
    return _L2ImageLoss.get().apply(images, targets)
