"""Camera helpers: camera-to-world matrices in the layout `spl_render_frame` takes.

The reference passes a PGA motor and converts it with `motor3d_to_mat4` (utils.rs:31-42), whose
columns are the images of the x, y, z axes and of the origin.  Here the camera is given directly as
that 4x4 matrix, column-major, 16 floats: right, up, forward (+z looks into the scene, as the
reference's projection puts w = view z, utils.rs:45-55) and position.
"""
import math

import numpy as np

__all__ = ["look_at", "orbit_poses", "flythrough_poses", "rotor_translation_to_matrix", "Motor"]


def _normalize(v):
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v)


def look_at(eye, target, up=(0.0, 1.0, 0.0)):
    """Camera-to-world 4x4 (column-major, float32[16]) looking from eye at target."""
    eye = np.asarray(eye, np.float64)
    f = _normalize(np.asarray(target, np.float64) - eye)
    up = np.asarray(up, np.float64)
    if abs(float(np.dot(f, _normalize(up)))) > 0.999:
        up = np.array([0.0, 0.0, 1.0]) if abs(f[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    r = _normalize(np.cross(up, f))
    u = np.cross(f, r)
    m = np.zeros(16, np.float64)
    m[0:3] = r
    m[4:7] = u
    m[8:11] = f
    m[12:15] = eye
    m[15] = 1.0
    return m.astype(np.float32)


def rotor_translation_to_matrix(rotor, translation):
    """Camera-to-world matrix from a unit rotor (scalar, e23, e31, e12 ~ quaternion w, x, y, z) and a
    translation, the rigid motion a PGA motor `translator * rotor` describes (showcase.rs:139)."""
    w, x, y, z = (float(c) for c in rotor)
    n = math.sqrt(w * w + x * x + y * y + z * z)
    w, x, y, z = w / n, x / n, y / n, z / n
    R = np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
    ])
    m = np.zeros(16, np.float64)
    for c in range(3):
        m[4 * c:4 * c + 3] = R[:, c]
    m[12:15] = np.asarray(translation, np.float64)
    m[15] = 1.0
    return m.astype(np.float32)


def orbit_poses(n, seed, radius=(6.0, 12.0), target=(0.0, 0.0, 0.0)):
    """n seeded poses on an orbit (azimuth uniform, elevation in [-30, 30] deg), looking at target."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        az = rng.uniform(0.0, 2.0 * math.pi)
        el = rng.uniform(-math.pi / 6, math.pi / 6)
        r = rng.uniform(*radius)
        eye = np.array([r * math.cos(el) * math.cos(az), r * math.sin(el), r * math.cos(el) * math.sin(az)])
        out.append(look_at(eye + np.asarray(target), target))
    return out


def flythrough_poses(n, seed, radius=(18.0, 32.0), jitter=6.0):
    """n seeded poses of a fly-through that sweeps in and out of a 40^3 box of clusters.

    The camera moves on a wobbling orbit whose radius oscillates between radius[0] and radius[1];
    it looks at a jittered point near the origin, so part of every view is culled and the inner
    poses put the near plane (view z = 1) through clusters."""
    rng = np.random.default_rng(seed)
    out = []
    phase = rng.uniform(0, 2 * math.pi)
    for i in range(n):
        t = i / max(n, 1)
        az = phase + 2.0 * math.pi * t
        el = 0.35 * math.sin(4.0 * math.pi * t + phase)
        r = radius[0] + (radius[1] - radius[0]) * (0.5 + 0.5 * math.cos(6.0 * math.pi * t))
        eye = np.array([r * math.cos(el) * math.cos(az), r * math.sin(el), r * math.cos(el) * math.sin(az)])
        tgt = rng.normal(0.0, jitter, 3)
        out.append(look_at(eye, tgt))
    return out


class Motor:
    """A camera motor of 3D projective geometric algebra, the reference's camera argument
    (renderer.rs:355-366, showcase.rs:140): coefficients [s, e23, e31, e12, e01, e02, e03, e0123],
    computed by the library's C functions (spl_motor_*)."""

    def __init__(self, coefficients):
        self.coefficients = np.ascontiguousarray(coefficients, dtype=np.float32).reshape(8).copy()

    @staticmethod
    def _call(fn, *arrays, n_out=8):
        import ctypes
        from . import _lib
        out = np.empty(n_out, np.float32)
        args = [np.ascontiguousarray(a, dtype=np.float32) for a in arrays]
        _lib.check(getattr(_lib.load(), fn)(*[a.ctypes.data_as(ctypes.c_void_p) for a in args],
                                            out.ctypes.data_as(ctypes.c_void_p)))
        return out

    @classmethod
    def identity(cls):
        return cls([1, 0, 0, 0, 0, 0, 0, 0])

    @classmethod
    def from_rotor_translation(cls, rotor, translation):
        """translator(translation) * rotor, the rotor [s, e23, e31, e12] a unit quaternion (w, x, y, z)."""
        return cls(cls._call("spl_motor_from_rotor_translation", np.asarray(rotor, np.float32).reshape(4),
                             np.asarray(translation, np.float32).reshape(3)))

    @staticmethod
    def rotate_around_axis(angle, axis):
        """The rotor of a right-handed turn by `angle` about the unit `axis` (showcase.rs:16-19)."""
        h = 0.5 * float(angle)
        return np.array([math.cos(h), axis[0] * math.sin(h), axis[1] * math.sin(h), axis[2] * math.sin(h)],
                        np.float32)

    def matrix(self):
        """motor3d_to_mat4 (utils.rs:31-42): camera-to-world, column-major float32[16]."""
        return self._call("spl_motor_to_mat4", self.coefficients, n_out=16)

    def inverse(self):
        """Motor::inverse (renderer.rs:365)."""
        return Motor(self._call("spl_motor_inverse", self.coefficients))

    def __mul__(self, other):
        """Geometric product: self applied after other."""
        return Motor(self._call("spl_motor_product", self.coefficients, other.coefficients))
