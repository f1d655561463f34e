"""C-ABI contract tests that need no GPU: the library loads, exports every symbol the header declares,
validates configurations like Renderer::new, and its host math matches the oracle bit for bit."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

import oracle
from splatter_gb300 import _lib, build, camera
from splatter_gb300.renderer import Configuration, DepthSorting, compute_uniforms

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def header_functions():
    text = open(os.path.join(ROOT, "include", "splatter.h")).read()
    return sorted(set(re.findall(r"SPL_API\s+[\w\s\*]+?\b(spl_\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(names) == bound


def test_config_default_is_showcase_literal(lib):
    c = _lib.SplConfig()
    lib.spl_config_default(ctypes.byref(c))
    assert c.depth_sorting == 2 and c.use_covariance_for_scale == 1 and c.use_unaligned_rectangles == 1
    assert c.spherical_harmonics_order == 2 and c.max_splat_count == 4 * 1024 * 1024
    assert c.radix_bits_per_digit == 8
    assert c.frustum_culling_tolerance == np.float32(1.1) and c.ellipse_margin == 2.0 and c.splat_scale == 1.0
    assert c.field_of_view_y == np.float32(math.pi / 2)
    py = Configuration()
    assert py.spherical_harmonics_order == c.spherical_harmonics_order and py.max_splat_count == c.max_splat_count


@pytest.mark.parametrize("bits,ok", [(8, True), (4, True), (16, True), (1, True), (32, True), (3, False),
                                     (0, False), (12, False)])
def test_radix_bits_must_divide_32(lib, bits, ok):
    # Renderer::new asserts 32 == places * bits (renderer.rs:89-90); here the C call returns SPL_ERR_INVALID.
    cfg = Configuration(radix_bits_per_digit=bits).to_c()
    out = (ctypes.c_uint8 * 224)()
    cam = camera.look_at([0, 0, -5], [0, 0, 0])
    rc = lib.spl_compute_uniforms(ctypes.byref(cfg), cam.ctypes.data_as(ctypes.c_void_p), 64, 64, out)
    assert (rc == _lib.SPL_OK) == ok
    if not ok:
        assert b"radix_bits_per_digit" in lib.spl_last_error_string()
        h = ctypes.c_void_p()
        assert lib.spl_renderer_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.SPL_ERR_INVALID
        assert not h.value


@pytest.mark.parametrize("field,value", [("spherical_harmonics_order", 4), ("depth_sorting", 7),
                                         ("max_splat_count", 0), ("max_splat_count", 1 << 30),
                                         ("blend_mode", 3), ("field_of_view_y", 0.0),
                                         ("frustum_culling_tolerance", float("nan"))])
def test_invalid_configs_rejected_without_gpu(lib, field, value):
    cfg = Configuration()
    setattr(cfg, field, value)
    h = ctypes.c_void_p()
    assert lib.spl_renderer_create(ctypes.byref(cfg.to_c()), ctypes.byref(h)) == _lib.SPL_ERR_INVALID


@pytest.mark.parametrize("w,h,fovy", [(640, 480, math.radians(60)), (1920, 1080, math.pi / 2), (333, 777, 1.1)])
def test_uniforms_bit_exact_vs_oracle(lib, w, h, fovy):
    for seed in range(4):
        cam = camera.orbit_poses(1, seed)[0]
        cfg = Configuration(field_of_view_y=fovy, frustum_culling_tolerance=1.1, ellipse_margin=2.0, splat_scale=1.3)
        got = np.frombuffer(compute_uniforms(cfg, cam, w, h), np.uint8)
        ref = oracle.uniforms(cam, w, h, fovy=fovy, tol=1.1, margin=2.0, splat_scale=1.3)
        assert np.array_equal(got, np.frombuffer(ref.tobytes(), np.uint8))


def test_parse_file_header(lib, tmp_path):
    body = np.zeros((5, 62), np.float32).tobytes()
    header = ("ply\nformat binary_little_endian 1.0\nelement vertex 5\n" +
              "".join(f"property float p{i}\n" for i in range(62)) + "end_header\n").encode()
    p = tmp_path / "s.ply"
    p.write_bytes(header + body)
    from splatter_gb300 import Scene
    hb, n = Scene.parse_file_header(p)
    assert hb == len(header) and n == 5
    bad = tmp_path / "bad.ply"
    bad.write_bytes(b"ply\nelement vertex 5\n")
    with pytest.raises(_lib.SplatterError) as e:
        Scene.parse_file_header(bad)
    assert e.value.code == _lib.SPL_ERR_IO
    with pytest.raises(_lib.SplatterError):
        Scene.parse_file_header(tmp_path / "missing.ply")


def test_depth_sorting_enum_matches_header():
    text = open(os.path.join(ROOT, "include", "splatter.h")).read()
    for m in DepthSorting:
        assert re.search(rf"#define SPL_DEPTH_SORTING_{m.name} {int(m)}\b", text), m


def test_missing_library_fails_loudly(tmp_path):
    """Without the built library the package raises; there is no CPU fallback to route to."""
    import subprocess
    import sys
    code = ("import splatter_gb300._lib as L\n"
            f"L.LIB_PATH = {str(tmp_path / 'absent.so')!r}\n"
            "try:\n    L.load()\nexcept ImportError as e:\n    print('raised', e)\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("raised") and "no CPU fallback" in r.stdout
