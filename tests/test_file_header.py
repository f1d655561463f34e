"""Splat-file header validation (host only, no GPU): spl_validate_file_header against well-formed and
malformed PLY headers.  The reference's parse_file_header (scene.rs:197-213) only counts; the
validator rejects every layout its loader would misread (scene.rs:216-224)."""
import numpy as np
import pytest

from splatter_gb300 import Scene, SplatterError, _lib, synthetic

N = 7


def _records():
    return synthetic.plain_small(N, seed=5, sh_order=3)


def _write(path, lines, n_records=N, nl="\n"):
    header = (nl.join(lines) + nl).encode()
    path.write_bytes(header + np.zeros((n_records, 62), "<f4").tobytes())
    return len(header)


def _standard_lines(count=N, props=None, fmt="format binary_little_endian 1.0"):
    props = synthetic.ply_property_names() if props is None else props
    return ["ply", fmt, f"element vertex {count}", *[f"property float {p}" for p in props], "end_header"]


def _io_error(path, check_names=True):
    with pytest.raises(SplatterError) as e:
        Scene.validate_file_header(path, check_names)
    assert e.value.code == _lib.SPL_ERR_IO
    return str(e.value)


def test_standard_file_agrees_with_the_reference_parser(tmp_path):
    p = tmp_path / "s.ply"
    hb = synthetic.write_ply(p, _records(), comments=["made by a test"])
    assert Scene.validate_file_header(p) == (hb, N)
    assert Scene.parse_file_header(p) == (hb, N)


def test_crlf_header_is_accepted(tmp_path):
    p = tmp_path / "crlf.ply"
    hb = synthetic.write_ply(p, _records(), crlf=True)
    assert Scene.validate_file_header(p) == (hb, N)
    with pytest.raises(SplatterError):  # the reference-style parser wants "\n" lines (scene.rs:203,207)
        Scene.parse_file_header(p)


def test_trailing_element_after_vertex_data_is_accepted(tmp_path):
    p = tmp_path / "trail.ply"
    lines = _standard_lines()[:-1] + ["element face 0", "property list uchar int vertex_indices", "end_header"]
    hb = _write(p, lines)
    assert Scene.validate_file_header(p) == (hb, N)


def test_names_are_checked_only_on_request(tmp_path):
    p = tmp_path / "names.ply"
    hb = _write(p, _standard_lines(props=[f"p{i}" for i in range(62)]))
    assert "expected 'x'" in _io_error(p)
    assert Scene.validate_file_header(p, check_names=False) == (hb, N)


@pytest.mark.parametrize("case", ["ascii", "big_endian", "61_props", "63_props", "double_prop", "face_first",
                                  "no_end", "bad_count", "negative_count", "truncated", "not_ply", "no_format",
                                  "no_vertex", "unknown_line"])
def test_malformed_headers_are_rejected(tmp_path, case):
    names = synthetic.ply_property_names()
    p = tmp_path / f"{case}.ply"
    if case == "ascii":
        _write(p, _standard_lines(fmt="format ascii 1.0"))
    elif case == "big_endian":
        _write(p, _standard_lines(fmt="format binary_big_endian 1.0"))
    elif case == "61_props":
        _write(p, _standard_lines(props=names[:61]))
    elif case == "63_props":
        _write(p, _standard_lines()[:-1] + ["property float extra", "end_header"])
    elif case == "double_prop":
        lines = _standard_lines()
        lines[3] = "property double x"
        _write(p, lines)
    elif case == "face_first":
        lines = _standard_lines()
        _write(p, lines[:2] + ["element face 1", "property list uchar int vertex_indices"] + lines[2:])
    elif case == "no_end":
        p.write_bytes(("\n".join(_standard_lines()[:-1]) + "\n").encode())
    elif case == "bad_count":
        lines = _standard_lines()
        lines[2] = "element vertex 7x"
        _write(p, lines)
    elif case == "negative_count":
        lines = _standard_lines()
        lines[2] = "element vertex -7"
        _write(p, lines)
    elif case == "truncated":
        _write(p, _standard_lines(count=N + 1))  # body holds N records
    elif case == "not_ply":
        _write(p, ["plyx"] + _standard_lines()[1:])
    elif case == "no_format":
        lines = _standard_lines()
        _write(p, lines[:1] + lines[2:])
    elif case == "no_vertex":
        _write(p, ["ply", "format binary_little_endian 1.0", "end_header"])
    elif case == "unknown_line":
        lines = _standard_lines()
        _write(p, lines[:3] + ["bogus line"] + lines[3:])
    _io_error(p)


def test_missing_file_and_null_arguments(tmp_path):
    _io_error(tmp_path / "missing.ply")
