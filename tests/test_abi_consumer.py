"""The C ABI from a compiled caller: tests/abi_consumer.c, built against include/splatter.h and
libsplatter_cuda.so alone (no Python between them), the way the reference's Rust crate would bind it.

Without a GPU: the header compiles as strict C11 and as C++17, its structs have the layouts the
ctypes mirror declares, the program links, and the host-only entry points behave.  With a GPU: the program renders the reference's dev-test scene
(Scene::new_dev_test, scene.rs:158-192) and its images equal the committed golden images of the
oracle (tests/golden/dev_scene.json) byte for byte, with the same visible and drawn counts.
"""
import ctypes
import hashlib
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from splatter_gb300 import build, synthetic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "abi_consumer.c")
STRICT = ["-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-O1"]


def _cc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    return cc


def _compile(out, render=False):
    lib = build.build()
    libdir = os.path.dirname(lib)
    cmd = [_cc(), *STRICT, "-I", os.path.join(ROOT, "include"), SRC, "-o", out, "-L", libdir, "-lsplatter_cuda",
           "-Wl,-rpath," + libdir]
    if render:
        cuda = os.path.dirname(os.path.dirname(build._nvcc()))
        cmd[1:1] = ["-DABI_CONSUMER_RENDER", "-I", os.path.join(cuda, "include")]
        cmd += ["-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_header_is_strict_c11_and_cxx17(tmp_path):
    inc = os.path.join(ROOT, "include", "splatter.h")
    r = subprocess.run([_cc(), *STRICT, "-fsyntax-only", "-x", "c", inc], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx:
        r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only", "-x",
                            "c++", inc], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_host_entry_points_from_c(tmp_path):
    exe = _compile(str(tmp_path / "abi_consumer"))
    ply = str(tmp_path / "s.ply")
    synthetic.write_ply(ply, synthetic.plain_small(37, seed=4, sh_order=3))
    r = subprocess.run([exe, "host", ply], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    assert lines[0].startswith("header ") and int(lines[0].split()[2]) == 37
    assert "host ok" in lines
    bad = str(tmp_path / "bad.ply")
    open(bad, "wb").write(b"ply\nformat ascii 1.0\nend_header\n")
    r = subprocess.run([exe, "host", bad], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "spl_validate_file_header failed (3)" in r.stderr


@pytest.mark.gpu
def test_dev_scene_rendered_from_c_matches_golden(tmp_path):
    exe = _compile(str(tmp_path / "abi_consumer_render"), render=True)
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "dev_scene.json")))
    for case in g["cases"][::3]:
        out = str(tmp_path / (case["name"] + ".rgba"))
        args = [exe, "render", str(case["width"]), str(case["height"]), repr(float(case["fovy"])),
                str(case["depth_sorting"]), str(int(case["covariance"])), str(int(case["rect"])), out]
        args += [repr(float(np.float32(v))) for v in case["camera"]]
        r = subprocess.run(args, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, (case["name"], r.stderr)
        stats = [int(x) for x in r.stdout.split()[1:4]]
        assert stats[:2] == case["stats"][:2], case["name"]
        img = open(out, "rb").read()
        assert len(img) == case["width"] * case["height"] * 4
        assert hashlib.sha256(img).hexdigest() == case["sha256"], case["name"]


def test_struct_layouts_match_the_ctypes_mirror(tmp_path):
    """Every struct of the header has the size and field offsets that splatter_gb300/_lib.py declares
    for ctypes (a mismatch would pass wrong values silently through the ABI)."""
    from splatter_gb300 import _lib
    structs = {"spl_config": _lib.SplConfig, "spl_frame_info": _lib.SplFrameInfo,
               "spl_server_config": _lib.SplServerConfig, "spl_request": _lib.SplRequest,
               "spl_completion": _lib.SplCompletion, "spl_server_stats": _lib.SplServerStats}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "splatter.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'    printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    r = subprocess.run([_cc(), *STRICT, "-I", os.path.join(ROOT, "include"), str(src), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    seen = 0
    for line in out:
        if not line:
            continue
        cname, what, value = line.split()
        py = structs[cname]
        want = ctypes.sizeof(py) if what == "size" else getattr(py, what).offset
        assert int(value) == want, (cname, what, int(value), want)
        seen += 1
    assert seen == len(structs) + sum(len(py._fields_) for py in structs.values())
