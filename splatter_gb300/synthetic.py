"""Seeded synthetic splat scenes in the reference's file-record layout.

No public dataset is used: the pretrained 3DGS scenes the reference's README points to are not
available, so these generators stand in for them with the shapes, sizes and value distributions
of the benchmark configurations:

* ``plain_small``   100k splats, positions ~ N(0, 2^2), SH degree 0 (640x480, fovy 60 deg).
* ``clustered``     64 Gaussian clusters (sigma 0.5-3, centres uniform in the 40^3 box) plus 20%
                    uniform background, SH degree 3 (band 0 ~ N(0, 0.3^2), higher ~ N(0, 0.05^2)).
                    ``clustered_device`` draws the same distributions on the GPU (serving scenes).

Every generator returns PLY-layout records, shape (N, 62) float32 (scene.rs:15-24): centre[3],
normal[3], colour[48] (coefficient k of channel c at 3k+c, the slot the shader reads,
shaders.wgsl:268-294), alpha logit, log-scale[3], rotation[4] (scalar first).  Log-scales are
~ N(-4, 0.5^2), rotations are uniform unit quaternions (Shoemake), opacity logits ~ N(0, 1.5^2).
The load transform (exp, sigmoid, normalisation; scene.rs:225-250) is applied by the loader.
"""
import math

import numpy as np

__all__ = ["RECORD_FLOATS", "plain_small", "clustered", "clustered_device", "records_to_splats60",
           "dev_test_splats60", "serving_scene_sizes"]

RECORD_FLOATS = 62


def _records(n, rng, centers, sh_order):
    rec = np.zeros((n, RECORD_FLOATS), np.float32)
    rec[:, 0:3] = centers
    rec[:, 6:9] = rng.normal(0.0, 0.3, (n, 3))
    if sh_order > 0:
        ncoef = (sh_order + 1) ** 2
        rec[:, 9:6 + 3 * ncoef] = rng.normal(0.0, 0.05, (n, 3 * ncoef - 3))
    rec[:, 54] = rng.normal(0.0, 1.5, n)
    rec[:, 55:58] = rng.normal(-4.0, 0.5, (n, 3))
    u = rng.random((n, 3))
    a = np.sqrt(1.0 - u[:, 0])
    b = np.sqrt(u[:, 0])
    rec[:, 58] = a * np.sin(2 * math.pi * u[:, 1])
    rec[:, 59] = a * np.cos(2 * math.pi * u[:, 1])
    rec[:, 60] = b * np.sin(2 * math.pi * u[:, 2])
    rec[:, 61] = b * np.cos(2 * math.pi * u[:, 2])
    return rec


def plain_small(n=100_000, seed=0, sh_order=0):
    """Config 'plain path, small scene': positions ~ N(0, 2^2) per axis."""
    rng = np.random.default_rng(seed)
    centers = rng.normal(0.0, 2.0, (n, 3)).astype(np.float32)
    return _records(n, rng, centers, sh_order)


def clustered(n=1_000_000, seed=1, sh_order=3, clusters=64, background=0.2, box=40.0):
    """Configs 'plain path 1M / 6M' and the serving scenes: clustered positions in a box^3 box."""
    rng = np.random.default_rng(seed)
    nb = int(round(n * background))
    nc = n - nb
    cc = rng.uniform(-box / 2, box / 2, (clusters, 3))
    cs = rng.uniform(0.5, 3.0, clusters)
    which = rng.integers(0, clusters, nc)
    centers = np.empty((n, 3), np.float32)
    centers[:nc] = cc[which] + rng.normal(0.0, 1.0, (nc, 3)) * cs[which, None]
    centers[nc:] = rng.uniform(-box / 2, box / 2, (nb, 3))
    perm = rng.permutation(n)
    centers = centers[perm]
    return _records(n, rng, centers, sh_order)


def clustered_device(n, seed=1, sh_order=3, clusters=64, background=0.2, box=40.0, device="cuda"):
    """``clustered`` generated on the GPU with torch's generator (same distributions, a different
    random stream): a (n, 62) float32 CUDA tensor of file records."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    f32 = dict(device=device, dtype=torch.float32)
    nb = int(round(n * background))
    nc = n - nb
    cc = (torch.rand((clusters, 3), generator=g, **f32) - 0.5) * box
    cs = 0.5 + 2.5 * torch.rand(clusters, generator=g, **f32)
    which = torch.randint(0, clusters, (nc,), generator=g, device=device)
    rec = torch.zeros((n, RECORD_FLOATS), **f32)
    centers = torch.empty((n, 3), **f32)
    centers[:nc] = cc[which] + torch.randn((nc, 3), generator=g, **f32) * cs[which, None]
    centers[nc:] = (torch.rand((nb, 3), generator=g, **f32) - 0.5) * box
    rec[:, 0:3] = centers[torch.randperm(n, generator=g, device=device)]
    rec[:, 6:9] = 0.3 * torch.randn((n, 3), generator=g, **f32)
    if sh_order > 0:
        ncoef = (sh_order + 1) ** 2
        rec[:, 9:6 + 3 * ncoef] = 0.05 * torch.randn((n, 3 * ncoef - 3), generator=g, **f32)
    rec[:, 54] = 1.5 * torch.randn(n, generator=g, **f32)
    rec[:, 55:58] = -4.0 + 0.5 * torch.randn((n, 3), generator=g, **f32)
    u = torch.rand((n, 3), generator=g, **f32)
    a = torch.sqrt(1.0 - u[:, 0])
    b = torch.sqrt(u[:, 0])
    rec[:, 58] = a * torch.sin(2 * math.pi * u[:, 1])
    rec[:, 59] = a * torch.cos(2 * math.pi * u[:, 1])
    rec[:, 60] = b * torch.sin(2 * math.pi * u[:, 2])
    rec[:, 61] = b * torch.cos(2 * math.pi * u[:, 2])
    return rec


def records_to_splats60(center, rotation, scale, alpha, sh):
    """SoA arrays -> the reference's 60-float device splat layout (scene.rs:32, shaders.wgsl:28-35):
    rotation[4], centre[3], pad, scale[3], alpha, colourSH[48]."""
    n = center.shape[0]
    s = np.zeros((n, 60), np.float32)
    s[:, 0:4] = rotation
    s[:, 4:7] = center
    s[:, 8:11] = scale
    s[:, 11] = alpha
    s[:, 12:60] = sh
    return s


def dev_test_splats60():
    """Scene::new_dev_test (scene.rs:158-192): three splats on the unit axes, raw scale
    (0.2, 0.1, 0.05), alpha 1, pure R/G/B band-0 colour."""
    s = np.zeros((3, 60), np.float32)
    for i in range(3):
        s[i, 0] = 1.0
        s[i, 4 + i] = 1.0
        s[i, 8:11] = (0.2, 0.1, 0.05)
        s[i, 11] = 1.0
        s[i, 12 + i] = 1.0
    return s


def serving_scene_sizes(count=24, seed=3, lo=200_000, hi=6_000_000):
    """Splat counts of the serving configuration: log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return [int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(count)]


def ply_property_names():
    """The 62 vertex properties of a 3D-Gaussian splat file in record order (SerializedSplat,
    scene.rs:15-24): centre, normal, 48 colour coefficients, opacity logit, log-scales, rotation."""
    return (["x", "y", "z", "nx", "ny", "nz"] + [f"f_dc_{i}" for i in range(3)] + [f"f_rest_{i}" for i in range(45)] +
            ["opacity"] + [f"scale_{i}" for i in range(3)] + [f"rot_{i}" for i in range(4)])


def write_ply(path, records, crlf=False, comments=()):
    """Writes (N, 62) float32 records as a binary little-endian PLY splat file; returns the header
    length in bytes."""
    rec = np.ascontiguousarray(records, dtype=np.float32).reshape(-1, 62)
    nl = "\r\n" if crlf else "\n"
    lines = ["ply", "format binary_little_endian 1.0", *[f"comment {c}" for c in comments],
             f"element vertex {rec.shape[0]}", *[f"property float {p}" for p in ply_property_names()], "end_header"]
    header = (nl.join(lines) + nl).encode()
    with open(path, "wb") as f:
        f.write(header)
        f.write(rec.astype("<f4").tobytes())
    return len(header)
