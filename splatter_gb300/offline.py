"""Headless offline renderer: the reference's viewer loop (application_framework.rs:269-301 drives
showcase.rs's render once per window frame) without a window — a camera path rendered into an image
sequence with a per-frame timing log.

    python -m splatter_gb300.offline scene.ply --out frames/ --width 1920 --height 1080 --poses 64

renders 64 orbit poses of a splat file (or, without a file, of a seeded synthetic scene), optionally
loading the file progressively one chunk per frame like the viewer (showcase.rs:98-103), and writes
frame_00000.png ... plus timing.csv (device milliseconds of each frame's render, measured with CUDA
events on the render stream, and the wall milliseconds including the readback and the file write).
The PNG holds the frame's RGB over black (the swapchain clear, renderer.rs:436-447); the alpha
channel of the device image is the final transmittance and is dropped.
"""
import argparse
import math
import os
import struct
import time
import zlib

import numpy as np

__all__ = ["write_png", "read_png", "render_sequence", "main"]


def _chunk(tag, data):
    c = struct.pack(">I", len(data)) + tag + data
    return c + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def write_png(path, rgb):
    """Writes an (H, W, 3) uint8 array as an 8-bit RGB PNG (filter 0 on every row, zlib level 6)."""
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w, c = rgb.shape
    assert c == 3
    raw = np.empty((h, 1 + 3 * w), np.uint8)
    raw[:, 0] = 0
    raw[:, 1:] = rgb.reshape(h, 3 * w)
    data = (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) +
            _chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)) + _chunk(b"IEND", b""))
    with open(path, "wb") as f:
        f.write(data)


def read_png(path):
    """Reads back a PNG written by write_png (8-bit RGB, filter 0): an (H, W, 3) uint8 array."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, w, h, idat = 8, 0, 0, b""
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 2
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 3 * w)
    assert not raw[:, 0].any()
    return raw[:, 1:].reshape(h, w, 3).copy()


def render_sequence(renderer, scene, poses, width, height, out_dir=None, loader=None, keep=False):
    """Renders `poses` (camera-to-world matrices or camera.Motor) one after another on one stream.
    With `loader` (a ProgressiveLoader) one chunk is loaded before each frame.  Writes
    frame_%05d.png and timing.csv into out_dir when given; returns the per-frame timing rows
    (frame, device_ms, wall_ms, chunks_left) and, with keep, the RGB frames."""
    import torch
    from .camera import Motor
    stream = torch.cuda.current_stream()
    out = renderer.output_buffer(width, height)
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
    host = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
    rows, frames = [], []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for k, pose in enumerate(poses):
        t0 = time.perf_counter()
        left = loader.step(stream) if loader is not None else 0
        e0.record(stream)
        if isinstance(pose, Motor):
            renderer.render_frame_motor(scene, pose, width, height, out=out, stream=stream)
        else:
            renderer.render_frame(scene, pose, width, height, out=out, stream=stream)
        e1.record(stream)
        host.copy_(out, non_blocking=True)
        stream.synchronize()
        renderer.frame_info()  # raises on a device-reported error
        rgb = host.numpy()[..., :3]
        if out_dir:
            write_png(os.path.join(out_dir, f"frame_{k:05d}.png"), rgb)
        if keep:
            frames.append(rgb.copy())
        rows.append((k, e0.elapsed_time(e1), 1000.0 * (time.perf_counter() - t0), left))
    if out_dir:
        with open(os.path.join(out_dir, "timing.csv"), "w") as f:
            f.write("frame,device_ms,wall_ms,chunks_left\n")
            for r in rows:
                f.write(f"{r[0]},{r[1]:.4f},{r[2]:.4f},{r[3]}\n")
    return (rows, frames) if keep else rows


def main(argv=None):
    from . import BlendMode, Configuration, DepthSorting, ProgressiveLoader, Renderer, Scene, camera, synthetic
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("ply", nargs="?", help="splat file (binary little-endian PLY, 62 floats per splat)")
    ap.add_argument("--out", default="frames")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--poses", type=int, default=32, help="orbit poses around the origin")
    ap.add_argument("--radius", type=float, nargs=2, default=(6.0, 12.0))
    ap.add_argument("--chunk", type=int, default=0, help="load progressively, this many splats per frame")
    ap.add_argument("--sh", type=int, default=3, help="spherical harmonics order")
    ap.add_argument("--fovy", type=float, default=90.0, help="degrees (the reference fixes 90)")
    ap.add_argument("--depth-sorting", default="gpu", choices=["none", "cpu", "gpu", "gpu-indirect"])
    ap.add_argument("--synthetic", type=int, default=1_000_000, help="splats of the seeded scene when no file")
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    ds = {"none": DepthSorting.NONE, "cpu": DepthSorting.CPU, "gpu": DepthSorting.GPU,
          "gpu-indirect": DepthSorting.GPU_INDIRECT_DRAW}[a.depth_sorting]
    if a.ply:
        hb, n = Scene.validate_file_header(a.ply)
    else:
        n = a.synthetic
    cfg = Configuration(depth_sorting=ds, spherical_harmonics_order=a.sh, max_splat_count=max(n, 1),
                        field_of_view_y=math.radians(a.fovy), blend_mode=BlendMode.UNORM8)
    r = Renderer(cfg)
    loader = None
    if a.ply:
        s = Scene(r, n)
        if a.chunk > 0:
            loader = ProgressiveLoader(s, a.ply, hb, a.chunk)
        else:
            s.load_chunk_file(a.ply, hb, 0, n)
    else:
        s = Scene(r, n)
        s.load_chunk(synthetic.clustered(n, seed=a.seed, sh_order=a.sh))
    poses = camera.orbit_poses(a.poses, a.seed + 1, radius=tuple(a.radius))
    rows = render_sequence(r, s, poses, a.width, a.height, out_dir=a.out, loader=loader)
    dev = np.array([row[1] for row in rows])
    print(f"{len(rows)} frames of {n} splats at {a.width}x{a.height} -> {a.out}: device median "
          f"{np.median(dev):.3f} ms ({1000.0 / max(np.median(dev), 1e-9):.1f} frames/s)")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
