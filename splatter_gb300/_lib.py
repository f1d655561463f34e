"""ctypes binding of libsplatter_cuda.so (include/splatter.h).

This is the same binding a Python caller of the reference-facing C ABI would write.  The library is
loaded from splatter_gb300/_build/; if it is missing the import of the renderer fails loudly — there
is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsplatter_cuda.so")

SPL_OK = 0
SPL_ERR_INVALID = 1
SPL_ERR_OOM = 2
SPL_ERR_IO = 3
SPL_ERR_LOOKBACK_TIMEOUT = 4
SPL_ERR_CUDA = 5
SPL_ERR_CAPACITY = 6

ERROR_NAMES = {
    SPL_OK: "SPL_OK", SPL_ERR_INVALID: "SPL_ERR_INVALID", SPL_ERR_OOM: "SPL_ERR_OOM", SPL_ERR_IO: "SPL_ERR_IO",
    SPL_ERR_LOOKBACK_TIMEOUT: "SPL_ERR_LOOKBACK_TIMEOUT", SPL_ERR_CUDA: "SPL_ERR_CUDA",
    SPL_ERR_CAPACITY: "SPL_ERR_CAPACITY",
}


class SplConfig(ctypes.Structure):
    _fields_ = [
        ("depth_sorting", ctypes.c_int32),
        ("use_covariance_for_scale", ctypes.c_int32),
        ("use_unaligned_rectangles", ctypes.c_int32),
        ("spherical_harmonics_order", ctypes.c_uint32),
        ("max_splat_count", ctypes.c_uint64),
        ("radix_bits_per_digit", ctypes.c_uint32),
        ("frustum_culling_tolerance", ctypes.c_float),
        ("ellipse_margin", ctypes.c_float),
        ("splat_scale", ctypes.c_float),
        ("field_of_view_y", ctypes.c_float),
        ("blend_mode", ctypes.c_int32),
        ("max_pair_count", ctypes.c_uint64),
    ]


class SplFrameInfo(ctypes.Structure):
    _fields_ = [
        ("splat_count", ctypes.c_uint64),
        ("visible_count", ctypes.c_uint64),
        ("draw_count", ctypes.c_uint64),
        ("pair_count", ctypes.c_uint64),
        ("device_error", ctypes.c_uint32),
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
    ]


class SplServerConfig(ctypes.Structure):
    _fields_ = [
        ("slots", ctypes.c_uint32),
        ("use_graphs", ctypes.c_uint32),
        ("scene_memory_budget", ctypes.c_uint64),
        ("max_width", ctypes.c_uint32),
        ("max_height", ctypes.c_uint32),
    ]


class SplRequest(ctypes.Structure):
    _fields_ = [
        ("tag", ctypes.c_uint64),
        ("scene_id", ctypes.c_uint32),
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
        ("camera_to_world", ctypes.c_float * 16),
        ("host_out", ctypes.c_void_p),
    ]


class SplCompletion(ctypes.Structure):
    _fields_ = [
        ("tag", ctypes.c_uint64),
        ("status", ctypes.c_int32),
        ("slot", ctypes.c_uint32),
        ("t_submit_ns", ctypes.c_uint64),
        ("t_start_ns", ctypes.c_uint64),
        ("t_done_ns", ctypes.c_uint64),
        ("restored", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]


class SplServerStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint64) for name in (
        "submitted", "completed", "failed", "resident_scenes", "resident_bytes", "evictions", "restores",
        "graphs_captured", "graph_launches", "direct_launches", "max_in_flight")]


SORT_COOPERATIVE = 0
SORT_ONESWEEP = 1

# (name, restype, argtypes) for every entry point of include/splatter.h
P = ctypes.c_void_p
U32 = ctypes.c_uint32
U64 = ctypes.c_uint64
I32 = ctypes.c_int
CFG_P = ctypes.POINTER(SplConfig)
SIGNATURES = [
    ("spl_config_default", None, [CFG_P]),
    ("spl_renderer_create", I32, [CFG_P, ctypes.POINTER(P)]),
    ("spl_renderer_destroy", None, [P]),
    ("spl_renderer_reserve", I32, [P, U32, U32]),
    ("spl_render_frame", I32, [P, P, P, U32, U32, P, P]),
    ("spl_renderer_frame_info", I32, [P, ctypes.POINTER(SplFrameInfo)]),
    ("spl_renderer_copy_entries", I32, [P, P, P, U64, P]),
    ("spl_renderer_copy_records", I32, [P, P, U64, P]),
    ("spl_compute_uniforms", I32, [CFG_P, P, U32, U32, P]),
    ("spl_scene_create", I32, [P, U64, ctypes.POINTER(P), ctypes.POINTER(U64)]),
    ("spl_scene_destroy", None, [P]),
    ("spl_scene_splat_count", U64, [P]),
    ("spl_scene_device_bytes", U64, [P]),
    ("spl_scene_create_dev_test", I32, [P, ctypes.POINTER(P)]),
    ("spl_parse_file_header", I32, [ctypes.c_char_p, ctypes.POINTER(U32), ctypes.POINTER(U64)]),
    ("spl_validate_file_header", I32, [ctypes.c_char_p, I32, ctypes.POINTER(U32), ctypes.POINTER(U64)]),
    ("spl_motor_to_mat4", I32, [P, P]),
    ("spl_motor_inverse", I32, [P, P]),
    ("spl_motor_product", I32, [P, P, P]),
    ("spl_motor_from_rotor_translation", I32, [P, P, P]),
    ("spl_render_frame_motor", I32, [P, P, P, U32, U32, P, P]),
    ("spl_progressive_loader_create", I32, [P, ctypes.c_char_p, U32, U64, ctypes.POINTER(P)]),
    ("spl_progressive_loader_step", I32, [P, P, ctypes.POINTER(U64)]),
    ("spl_progressive_loader_destroy", None, [P]),
    ("spl_scene_load_chunk", I32, [P, P, U64, U64, P]),
    ("spl_scene_load_chunk_file", I32, [P, ctypes.c_char_p, U32, U64, U64, P]),
    ("spl_scene_write_splats", I32, [P, P, U64, U64, P]),
    ("spl_scene_read_splats", I32, [P, P, U64, U64]),
    ("spl_sort_pairs", I32, [P, P, P, P, P, U64, U32, P]),
    ("spl_last_error_string", ctypes.c_char_p, []),
    ("spl_debug_lookback_timeout", I32, [U32, ctypes.POINTER(ctypes.c_int)]),
    ("spl_renderer_set_profiling", I32, [P, I32]),
    ("spl_renderer_stage_times", I32, [P, ctypes.POINTER(ctypes.c_float), I32]),
    ("spl_renderer_launches_per_frame", I32, [P, U32, U32]),
    ("spl_renderer_set_frame_graphs", I32, [P, I32]),
    ("spl_sort_pairs_no_alloc", I32, [P, P, P, P, U64, U32, P]),
    ("spl_sort_pairs_no_alloc_status", I32, [P, P]),
    ("spl_scene_wrap", I32, [P, U64, P, P, P, P, P, P, ctypes.POINTER(P)]),
    ("spl_render_backward", I32, [P, P, P, P, P, P, P, P, P, P, P]),
    ("spl_render_backward_accumulate", I32, [P, P, P, P, P, P, P, P, P, P, P]),
    ("spl_renderer_copy_record_gradients", I32, [P, P, U64, P]),
    ("spl_renderer_set_sort_mode", I32, [P, I32]),
    ("spl_frame_graph_create", I32, [P, U32, U32, U64, P, ctypes.POINTER(P)]),
    ("spl_frame_graph_launch", I32, [P, P, P, P]),
    ("spl_frame_graph_destroy", None, [P]),
    ("spl_scene_load_chunk_device", I32, [P, P, U64, U64, P]),
    ("spl_server_create", I32, [CFG_P, ctypes.POINTER(SplServerConfig), ctypes.POINTER(P)]),
    ("spl_server_destroy", None, [P]),
    ("spl_server_add_scene", I32, [P, P, U64, I32, ctypes.POINTER(U32)]),
    ("spl_server_submit", I32, [P, ctypes.POINTER(SplRequest)]),
    ("spl_server_poll", I32, [P, ctypes.POINTER(SplCompletion), U32, ctypes.POINTER(U32), ctypes.c_int64]),
    ("spl_server_get_stats", I32, [P, ctypes.POINTER(SplServerStats)]),
    ("spl_server_now_ns", U64, []),
    ("spl_activate_splats", I32, [U64, P, P, P, P, P, P, P, P, P, P]),
    ("spl_activate_splats_backward", I32, [U64, P, P, P, P, P, P, P, P, P, P, P, P, P, P]),
    ("spl_l2_image_loss_partials", U32, [U64]),
    ("spl_l2_image_loss", I32, [P, P, U64, P, P]),
    ("spl_l2_image_loss_backward", I32, [P, P, U64, P, P, P]),
]

NO_ALLOC_MAX_PAIRS = 262144

STAGES = ["cull", "preprocess", "depth_sort", "bin", "pair_sort", "ranges", "raster", "frame"]

_lib = None


class SplatterError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


def load():
    """Loads the native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with splatter_gb300/build.py "
                              "(or __graft_entry__.build()); there is no CPU fallback")
        lib = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def check(code):
    if code != SPL_OK:
        msg = load().spl_last_error_string()
        raise SplatterError(code, msg.decode() if msg else "")
    return code
