"""Serving runtime (spl_server_*): many resident scenes, continuous admission of render requests
into concurrent slots, captured frame graphs, residency by device footprint with LRU eviction to
page-locked host memory.  No counterpart in the reference, whose Renderer renders one frame per call
(renderer.rs:355-466)."""
import ctypes
from collections import namedtuple

import numpy as np

from . import _lib
from ._lib import check
from .renderer import BlendMode, Configuration, _cam

Completion = namedtuple("Completion", "tag status slot t_submit_ns t_start_ns t_done_ns restored")


def now_ns():
    """The clock of the completions' timestamps (steady clock, ns)."""
    return int(_lib.load().spl_server_now_ns())


class Server:
    def __init__(self, config: Configuration, slots=8, use_graphs=True, scene_memory_budget=0, max_width=1920,
                 max_height=1080):
        self._lib = _lib.load()
        self.config = config
        sc = _lib.SplServerConfig(int(slots), 1 if use_graphs else 0, int(scene_memory_budget), int(max_width),
                                  int(max_height))
        h = ctypes.c_void_p()
        check(self._lib.spl_server_create(ctypes.byref(config.to_c()), ctypes.byref(sc), ctypes.byref(h)))
        self._h = h
        self._pending = {}  # tag -> host buffer (kept alive until its completion)
        self._next_tag = 1
        self.pixel_bytes = 16 if config.blend_mode == BlendMode.FP32 else 4

    def close(self):
        if getattr(self, "_h", None):
            self._lib.spl_server_destroy(self._h)
            self._h = None
            self._pending.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, records):
        """Adds a scene from (N, 62) float32 file records: a numpy array, or a CUDA tensor."""
        sid = ctypes.c_uint32()
        if hasattr(records, "is_cuda") and records.is_cuda:
            assert records.dtype.itemsize == 4 and records.is_contiguous()
            check(self._lib.spl_server_add_scene(self._h, ctypes.c_void_p(records.data_ptr()), records.numel() // 62,
                                                 1, ctypes.byref(sid)))
        else:
            rec = np.ascontiguousarray(records, dtype=np.float32).reshape(-1, 62)
            check(self._lib.spl_server_add_scene(self._h, rec.ctypes.data_as(ctypes.c_void_p), rec.shape[0], 0,
                                                 ctypes.byref(sid)))
        return int(sid.value)

    def output_buffer(self, width, height):
        """A page-locked host buffer for one result ((H, W, 4) uint8, or float32 in the FP32 mode)."""
        import torch
        dt = torch.float32 if self.pixel_bytes == 16 else torch.uint8
        return torch.empty((height, width, 4), dtype=dt, pin_memory=True)

    def submit(self, scene_id, camera_to_world, width, height, host_out, tag=None):
        """Queues a request; the image lands in host_out (a host tensor or numpy array of
        width*height*pixel bytes).  Returns the request's tag."""
        if tag is None:
            tag = self._next_tag
            self._next_tag += 1
        ptr = host_out.data_ptr() if hasattr(host_out, "data_ptr") else host_out.ctypes.data
        nbytes = host_out.numel() * host_out.element_size() if hasattr(host_out, "numel") else host_out.nbytes
        if nbytes < width * height * self.pixel_bytes:
            raise ValueError("host_out is too small for the viewport")
        req = _lib.SplRequest()
        req.tag = int(tag)
        req.scene_id = int(scene_id)
        req.width = int(width)
        req.height = int(height)
        cam = _cam(camera_to_world)
        ctypes.memmove(req.camera_to_world, cam.ctypes.data, 64)
        req.host_out = ctypes.c_void_p(ptr)
        self._pending[int(tag)] = host_out
        try:
            check(self._lib.spl_server_submit(self._h, ctypes.byref(req)))
        except Exception:
            self._pending.pop(int(tag), None)
            raise
        return int(tag)

    def poll(self, capacity=256, timeout_us=0):
        """Completed requests (waits up to timeout_us for the first; < 0 waits forever)."""
        arr = (_lib.SplCompletion * capacity)()
        n = ctypes.c_uint32()
        check(self._lib.spl_server_poll(self._h, arr, capacity, ctypes.byref(n), int(timeout_us)))
        out = []
        for i in range(n.value):
            c = arr[i]
            self._pending.pop(int(c.tag), None)
            out.append(Completion(int(c.tag), int(c.status), int(c.slot), int(c.t_submit_ns), int(c.t_start_ns),
                                  int(c.t_done_ns), bool(c.restored)))
        return out

    def wait_all(self, count, timeout_s=120.0):
        """Polls until `count` completions arrived (raises on timeout)."""
        got = []
        deadline = now_ns() + int(timeout_s * 1e9)
        while len(got) < count:
            if now_ns() > deadline:
                raise TimeoutError(f"{len(got)} of {count} requests completed")
            got.extend(self.poll(timeout_us=20000))
        return got

    def stats(self):
        st = _lib.SplServerStats()
        check(self._lib.spl_server_get_stats(self._h, ctypes.byref(st)))
        return {name: int(getattr(st, name)) for name, _ in _lib.SplServerStats._fields_}
