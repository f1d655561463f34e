"""Camera motors (host only): spl_motor_* against first principles — rotations by the quaternion
formula, look-at matrices, inverses and composition as 4x4 matrix algebra.  The reference builds its
camera matrices from a PGA motor (renderer.rs:364-365, utils.rs:31-42)."""
import math

import numpy as np
import pytest

from splatter_gb300 import SplatterError, camera
from splatter_gb300.camera import Motor


def _mat(m16):
    return np.asarray(m16, np.float64).reshape(4, 4).T  # column-major float[16] -> 4x4


def _quat_from_rotation(R):
    """Unit quaternion (w, x, y, z) of a rotation matrix (Shepperd's method)."""
    t = np.trace(R)
    if t > 0:
        s = math.sqrt(t + 1.0) * 2
        q = [0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s]
    else:
        i = int(np.argmax(np.diag(R)))
        j, k = (i + 1) % 3, (i + 2) % 3
        s = math.sqrt(1.0 + R[i, i] - R[j, j] - R[k, k]) * 2
        q = [0.0] * 4
        q[0] = (R[k, j] - R[j, k]) / s
        q[1 + i] = 0.25 * s
        q[1 + j] = (R[j, i] + R[i, j]) / s
        q[1 + k] = (R[k, i] + R[i, k]) / s
    return np.array(q)


def test_quarter_turn_about_z_and_translation():
    m = Motor.from_rotor_translation(Motor.rotate_around_axis(math.pi / 2, (0, 0, 1)), (1, 2, 3))
    M = _mat(m.matrix())
    assert np.allclose(M[:3, 0], [0, 1, 0], atol=1e-6)  # x -> y: right-handed
    assert np.allclose(M[:3, 1], [-1, 0, 0], atol=1e-6)
    assert np.allclose(M[:3, 2], [0, 0, 1], atol=1e-6)
    assert np.allclose(M[:, 3], [1, 2, 3, 1], atol=1e-6)
    assert np.allclose(M[3, :3], 0, atol=1e-7)


def test_identity():
    assert np.allclose(_mat(Motor.identity().matrix()), np.eye(4))


@pytest.mark.parametrize("seed", range(8))
def test_rotor_translation_matches_the_quaternion_formula(seed):
    rng = np.random.default_rng(seed)
    q = rng.normal(size=4)
    t = rng.normal(size=3) * 10
    got = Motor.from_rotor_translation(q, t).matrix()
    want = camera.rotor_translation_to_matrix(q, t)
    assert np.allclose(got, want, atol=2e-6)


@pytest.mark.parametrize("seed", range(8))
def test_look_at_matrices_round_trip(seed):
    rng = np.random.default_rng(100 + seed)
    eye, target = rng.normal(size=3) * 20, rng.normal(size=3) * 5
    L = _mat(camera.look_at(eye, target))
    q = _quat_from_rotation(L[:3, :3])
    M = _mat(Motor.from_rotor_translation(q, L[:3, 3]).matrix())
    assert np.allclose(M, L, atol=5e-6)


@pytest.mark.parametrize("seed", range(6))
def test_inverse_and_composition_are_matrix_algebra(seed):
    rng = np.random.default_rng(200 + seed)
    a = Motor.from_rotor_translation(rng.normal(size=4), rng.normal(size=3) * 4)
    b = Motor.from_rotor_translation(rng.normal(size=4), rng.normal(size=3) * 4)
    A, B = _mat(a.matrix()), _mat(b.matrix())
    assert np.allclose(_mat(a.inverse().matrix()), np.linalg.inv(A), atol=1e-5)
    assert np.allclose(_mat((a * b).matrix()), A @ B, atol=1e-5)
    assert np.allclose((a * a.inverse()).coefficients, Motor.identity().coefficients, atol=1e-6)


def test_scaled_motor_inverse_and_degenerate_inputs():
    m = Motor.from_rotor_translation(Motor.rotate_around_axis(0.7, (0.6, 0.0, 0.8)), (3, -1, 2))
    scaled = Motor(m.coefficients * 2.5)  # the sandwich scales points by 2.5^2; the inverse undoes it
    assert np.allclose((scaled * scaled.inverse()).coefficients, Motor.identity().coefficients, atol=1e-6)
    with pytest.raises(SplatterError):
        Motor.from_rotor_translation([0, 0, 0, 0], [0, 0, 0])
    with pytest.raises(SplatterError):
        Motor(np.zeros(8)).inverse()


def test_showcase_motor_moves_the_camera_along_its_view():
    """showcase.rs:113-118: translating by the rotated forward axis moves the camera where it looks."""
    rot = Motor.rotate_around_axis(0.4, (0, 1, 0))
    step = Motor.from_rotor_translation([1, 0, 0, 0], (0, 0, 1.5))
    r = Motor.from_rotor_translation(rot, (0, 0, 0))
    moved = Motor.from_rotor_translation([1, 0, 0, 0], (2, 0, 0)) * r * step
    M = _mat(moved.matrix())
    fwd = _mat(r.matrix())[:3, 2]
    assert np.allclose(M[:3, 3], np.array([2, 0, 0]) + 1.5 * fwd, atol=1e-6)
