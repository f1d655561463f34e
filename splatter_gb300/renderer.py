"""Python mirror of the reference's host API (Lichtso/splatter src/renderer.rs, src/scene.rs) over the
C ABI of libsplatter_cuda.so.  Names, argument meaning and error behaviour follow the Rust API:

    Configuration, DepthSorting            renderer.rs:14-47 (+ field_of_view_y, blend_mode, max_pair_count)
    Renderer(config)                       Renderer::new            renderer.rs:88
    renderer.render_frame(...)             Renderer::render_frame   renderer.rs:355
    Scene(renderer, splat_count)           Scene::new               scene.rs:45
    Scene.new_dev_test(renderer)           Scene::new_dev_test      scene.rs:158
    Scene.parse_file_header(path)          Scene::parse_file_header scene.rs:197
    scene.load_chunk(records | path, ...)  Scene::load_chunk        scene.rs:216

The reference panics on bad input; here a SplatterError (with the C status code) is raised.  Device
memory and streams come from PyTorch (plumbing only): outputs are CUDA tensors, the stream is the
current torch stream unless one is given.
"""
import enum
import math
from dataclasses import dataclass

import ctypes
import numpy as np

from . import _lib
from ._lib import SORT_COOPERATIVE, SORT_ONESWEEP, SplatterError, check

__all__ = ["DepthSorting", "BlendMode", "Configuration", "Renderer", "Scene", "SplatterError", "FrameInfo",
           "compute_uniforms"]


class DepthSorting(enum.IntEnum):
    """renderer.rs:14-23"""
    NONE = 0
    CPU = 1
    GPU = 2
    GPU_INDIRECT_DRAW = 3


class BlendMode(enum.IntEnum):
    UNORM8 = 0  # Bgra8Unorm surface of the reference: per-blend 8-bit re-quantisation, RGBA8 output
    FP32 = 1    # f32 blending, float4 output


@dataclass
class Configuration:
    """renderer.rs:26-47; defaults are the viewer's literal (showcase.rs:39-50)."""
    depth_sorting: DepthSorting = DepthSorting.GPU
    use_covariance_for_scale: bool = True
    use_unaligned_rectangles: bool = True
    spherical_harmonics_order: int = 2
    max_splat_count: int = 1024 * 1024 * 4
    radix_bits_per_digit: int = 8
    frustum_culling_tolerance: float = 1.1
    ellipse_margin: float = 2.0
    splat_scale: float = 1.0
    field_of_view_y: float = math.pi / 2  # extension (renderer.rs:366 fixes pi/2)
    blend_mode: BlendMode = BlendMode.UNORM8  # extension
    max_pair_count: int = 0  # extension: 0 = 16 x max_splat_count

    def to_c(self):
        c = _lib.SplConfig()
        c.depth_sorting = int(self.depth_sorting)
        c.use_covariance_for_scale = int(bool(self.use_covariance_for_scale))
        c.use_unaligned_rectangles = int(bool(self.use_unaligned_rectangles))
        c.spherical_harmonics_order = int(self.spherical_harmonics_order)
        c.max_splat_count = int(self.max_splat_count)
        c.radix_bits_per_digit = int(self.radix_bits_per_digit)
        c.frustum_culling_tolerance = float(self.frustum_culling_tolerance)
        c.ellipse_margin = float(self.ellipse_margin)
        c.splat_scale = float(self.splat_scale)
        c.field_of_view_y = float(self.field_of_view_y)
        c.blend_mode = int(self.blend_mode)
        c.max_pair_count = int(self.max_pair_count)
        return c


@dataclass
class FrameInfo:
    splat_count: int
    visible_count: int
    draw_count: int
    pair_count: int
    device_error: int
    width: int
    height: int


def _stream_ptr(stream):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _cam(camera_to_world):
    cam = np.ascontiguousarray(np.asarray(camera_to_world, np.float32).reshape(16))
    return cam


def compute_uniforms(config, camera_to_world, width, height):
    """Host math of render_frame (renderer.rs:364-409): the 224-byte uniform block as bytes."""
    lib = _lib.load()
    cam = _cam(camera_to_world)
    out = (ctypes.c_uint8 * 224)()
    check(lib.spl_compute_uniforms(ctypes.byref(config.to_c()), cam.ctypes.data_as(ctypes.c_void_p), int(width),
                                   int(height), out))
    return bytes(out)


class Renderer:
    """Renderer::new (renderer.rs:88)."""

    def __init__(self, config: Configuration = None):
        self.config = config or Configuration()
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.spl_renderer_create(ctypes.byref(self.config.to_c()), ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.spl_renderer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reserve(self, width, height):
        check(self._lib.spl_renderer_reserve(self._h, int(width), int(height)))

    def output_buffer(self, width, height, device=None):
        import torch
        if self.config.blend_mode == BlendMode.UNORM8:
            return torch.empty((height, width, 4), dtype=torch.uint8, device=device or "cuda")
        return torch.empty((height, width, 4), dtype=torch.float32, device=device or "cuda")

    def render_frame(self, scene, camera_to_world, width, height, out=None, stream=None):
        """Renderer::render_frame (renderer.rs:355): renders into `out` (allocated if None) and returns
        it; asynchronous on the stream like queue.submit."""
        if out is None:
            out = self.output_buffer(width, height)
        cam = _cam(camera_to_world)
        check(self._lib.spl_render_frame(self._h, scene.handle, cam.ctypes.data_as(ctypes.c_void_p), int(width),
                                         int(height), ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream)))
        return out

    def render_frame_motor(self, scene, motor, width, height, out=None, stream=None):
        """render_frame with the reference's camera argument, a PGA motor (renderer.rs:355-364):
        8 floats [s, e23, e31, e12, e01, e02, e03, e0123] or a camera.Motor."""
        if out is None:
            out = self.output_buffer(width, height)
        m = np.ascontiguousarray(getattr(motor, "coefficients", motor), dtype=np.float32).reshape(8)
        check(self._lib.spl_render_frame_motor(self._h, scene.handle, m.ctypes.data_as(ctypes.c_void_p), int(width),
                                               int(height), ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream)))
        return out

    def render_frame_ptr(self, scene, camera_to_world, width, height, out_ptr, stream_ptr):
        """Raw-pointer variant (device output pointer and cudaStream_t as ints)."""
        cam = _cam(camera_to_world)
        check(self._lib.spl_render_frame(self._h, scene.handle, cam.ctypes.data_as(ctypes.c_void_p), int(width),
                                         int(height), ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream_ptr)))

    def frame_info(self, check_status=True):
        info = _lib.SplFrameInfo()
        rc = self._lib.spl_renderer_frame_info(self._h, ctypes.byref(info))
        if check_status:
            check(rc)
        return FrameInfo(info.splat_count, info.visible_count, info.draw_count, info.pair_count, info.device_error,
                         info.width, info.height)

    def sorted_entries(self, stream=None):
        """(keys, splat indices) of the last frame in draw order, as CUDA uint32 tensors (int32 dtype)."""
        import torch
        info = self.frame_info()
        v = int(info.visible_count)
        keys = torch.empty(max(v, 1), dtype=torch.int32, device="cuda")
        idx = torch.empty(max(v, 1), dtype=torch.int32, device="cuda")
        check(self._lib.spl_renderer_copy_entries(self._h, ctypes.c_void_p(keys.data_ptr()),
                                                  ctypes.c_void_p(idx.data_ptr()), v, _stream_ptr(stream)))
        return keys[:v], idx[:v], info

    def records(self, stream=None):
        """(V, 16) float32 CUDA tensor of the last frame's screen-space records (compaction order)."""
        import torch
        info = self.frame_info()
        v = int(info.visible_count)
        rec = torch.empty((max(v, 1), 16), dtype=torch.float32, device="cuda")
        check(self._lib.spl_renderer_copy_records(self._h, ctypes.c_void_p(rec.data_ptr()), v, _stream_ptr(stream)))
        return rec[:v]

    def set_profiling(self, enable=True):
        check(self._lib.spl_renderer_set_profiling(self._h, 1 if enable else 0))

    def set_frame_graphs(self, enable=True):
        """Replay frames of a repeated viewport and scene size from a graph the renderer captures
        itself (on by default; the same results as direct launches)."""
        check(self._lib.spl_renderer_set_frame_graphs(self._h, 1 if enable else 0))

    def set_sort_mode(self, mode):
        """SORT_COOPERATIVE (default, one frame on the device at a time) or SORT_ONESWEEP (safe with
        frames of other renderers running concurrently)."""
        check(self._lib.spl_renderer_set_sort_mode(self._h, int(mode)))

    def capture_frame(self, width, height, out=None, max_splats=0):
        """A frame at width x height captured into a CUDA graph writing into `out` (allocated if
        None), grids sized for scenes of up to max_splats splats (0: max_splat_count);
        FrameGraph.launch(scene, camera) replays it for any such scene and any camera."""
        if out is None:
            out = self.output_buffer(width, height)
        h = ctypes.c_void_p()
        check(self._lib.spl_frame_graph_create(self._h, int(width), int(height), int(max_splats),
                                               ctypes.c_void_p(out.data_ptr()), ctypes.byref(h)))
        return FrameGraph(self, out, h)

    def stage_times(self):
        """{stage: milliseconds} of the last frame (needs set_profiling(True) before the frame)."""
        arr = (ctypes.c_float * len(_lib.STAGES))()
        check(self._lib.spl_renderer_stage_times(self._h, arr, len(_lib.STAGES)))
        return {k: float(v) for k, v in zip(_lib.STAGES, arr)}

    def launches_per_frame(self, width, height):
        return int(self._lib.spl_renderer_launches_per_frame(self._h, int(width), int(height)))

    def sort_pairs(self, keys, values, key_bits=32, stream=None):
        """Stable device radix sort of (key, value) uint32 pairs (given as int32 CUDA tensors)."""
        import torch
        n = keys.numel()
        ko = torch.empty_like(keys)
        vo = torch.empty_like(values)
        check(self._lib.spl_sort_pairs(self._h, ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(values.data_ptr()),
                                       ctypes.c_void_p(ko.data_ptr()), ctypes.c_void_p(vo.data_ptr()), n,
                                       int(key_bits), _stream_ptr(stream)))
        return ko, vo


class FrameGraph:
    """A captured frame (spl_frame_graph_*); keeps its renderer and output alive."""

    def __init__(self, renderer, out, handle):
        self._lib = _lib.load()
        self.renderer, self.out, self._h = renderer, out, handle

    def launch(self, scene, camera_to_world, stream=None):
        cam = _cam(camera_to_world)
        check(self._lib.spl_frame_graph_launch(self._h, scene.handle, cam.ctypes.data_as(ctypes.c_void_p),
                                               _stream_ptr(stream)))
        return self.out

    def close(self):
        if getattr(self, "_h", None):
            self._lib.spl_frame_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """Scene::new (scene.rs:45): resident SoA splat arrays for min(splat_count, max_splat_count)."""

    def __init__(self, renderer: Renderer, splat_count: int, _handle=None):
        self._lib = _lib.load()
        self.renderer = renderer
        if _handle is None:
            h = ctypes.c_void_p()
            n = ctypes.c_uint64()
            check(self._lib.spl_scene_create(renderer.handle, int(splat_count), ctypes.byref(h), ctypes.byref(n)))
            self._h = h
        else:
            self._h = _handle

    @classmethod
    def new_dev_test(cls, renderer: Renderer):
        """Scene::new_dev_test (scene.rs:158)."""
        lib = _lib.load()
        h = ctypes.c_void_p()
        check(lib.spl_scene_create_dev_test(renderer.handle, ctypes.byref(h)))
        return cls(renderer, 3, _handle=h)

    @staticmethod
    def parse_file_header(path):
        """Scene::parse_file_header (scene.rs:197): (header length in bytes, splat count)."""
        lib = _lib.load()
        hb = ctypes.c_uint32()
        n = ctypes.c_uint64()
        check(lib.spl_parse_file_header(str(path).encode(), ctypes.byref(hb), ctypes.byref(n)))
        return int(hb.value), int(n.value)

    @staticmethod
    def validate_file_header(path, check_names=True):
        """Validated header of a splat file: binary little-endian PLY with the vertex element first, 62
        float vertex properties (in the standard order when check_names) and a body long enough for the
        declared count; (header length in bytes, splat count), or SplatterError (SPL_ERR_IO)."""
        lib = _lib.load()
        hb = ctypes.c_uint32()
        n = ctypes.c_uint64()
        check(lib.spl_validate_file_header(str(path).encode(), 1 if check_names else 0, ctypes.byref(hb),
                                           ctypes.byref(n)))
        return int(hb.value), int(n.value)

    @classmethod
    def open_file(cls, renderer: Renderer, path, check_names=True):
        """A scene for a splat file's full count (clamped to max_splat_count, scene.rs:46), its header
        validated, nothing loaded yet: (scene, header length in bytes)."""
        hb, n = cls.validate_file_header(path, check_names)
        return cls(renderer, n), hb

    @property
    def handle(self):
        return self._h

    @property
    def splat_count(self):
        return int(self._lib.spl_scene_splat_count(self._h))

    @property
    def device_bytes(self):
        return int(self._lib.spl_scene_device_bytes(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.spl_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_chunk(self, records, start=0, stream=None):
        """Scene::load_chunk (scene.rs:216) from (K, 62) float32 PLY records for splats [start, start+K)."""
        rec = np.ascontiguousarray(records, dtype=np.float32).reshape(-1, 62)
        check(self._lib.spl_scene_load_chunk(self._h, rec.ctypes.data_as(ctypes.c_void_p), int(start), rec.shape[0],
                                             _stream_ptr(stream)))

    def load_chunk_device(self, records, start=0, stream=None):
        """Scene::load_chunk from a CUDA float32 tensor of (K, 62) records (no staging)."""
        assert records.is_cuda and records.dtype.itemsize == 4 and records.is_contiguous()
        k = records.numel() // 62
        check(self._lib.spl_scene_load_chunk_device(self._h, ctypes.c_void_p(records.data_ptr()), int(start), k,
                                                    _stream_ptr(stream)))

    def load_chunk_file(self, path, header_bytes, start, count, stream=None):
        """Scene::load_chunk reading records from a splat file."""
        check(self._lib.spl_scene_load_chunk_file(self._h, str(path).encode(), int(header_bytes), int(start),
                                                  int(count), _stream_ptr(stream)))

    def write_splats(self, splats60, start=0, stream=None):
        """Writes splats in the reference's 60-float device layout (scene.rs:32)."""
        s = np.ascontiguousarray(splats60, dtype=np.float32).reshape(-1, 60)
        check(self._lib.spl_scene_write_splats(self._h, s.ctypes.data_as(ctypes.c_void_p), int(start), s.shape[0],
                                               _stream_ptr(stream)))

    def read_splats(self, start=0, count=None):
        """Reads splats back as a (count, 60) float32 array (synchronous)."""
        n = self.splat_count
        count = n - start if count is None else count
        out = np.empty((count, 60), np.float32)
        check(self._lib.spl_scene_read_splats(self._h, out.ctypes.data_as(ctypes.c_void_p), int(start), int(count)))
        return out


class ProgressiveLoader:
    """Progressive loading as the reference's viewer does it (showcase.rs:13,54-59,98-103): each step
    loads the last chunk not yet loaded, on the given stream, so frames rendered in between show the
    splats loaded so far.  chunk_size 0 loads everything in the first step."""

    def __init__(self, scene: Scene, path, header_bytes, chunk_size):
        self._lib = _lib.load()
        self.scene = scene
        h = ctypes.c_void_p()
        check(self._lib.spl_progressive_loader_create(scene.handle, str(path).encode(), int(header_bytes),
                                                      int(chunk_size), ctypes.byref(h)))
        self._h = h
        n = scene.splat_count
        self.chunks_left = 0 if n == 0 else (1 if chunk_size == 0 else (n + chunk_size - 1) // chunk_size)

    def step(self, stream=None):
        """Loads the next chunk (if any) on `stream`; returns the number of chunks still to load."""
        left = ctypes.c_uint64()
        check(self._lib.spl_progressive_loader_step(self._h, _stream_ptr(stream), ctypes.byref(left)))
        self.chunks_left = int(left.value)
        return self.chunks_left

    def close(self):
        if getattr(self, "_h", None):
            self._lib.spl_progressive_loader_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
