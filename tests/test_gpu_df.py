"""The double-float elementary functions of the mixed-precision CBMC stages (grx_df.cuh),
evaluated on the device through grx_probe_df_functions, against FP64: sin and cos of 2 pi v
(the Ewald eik factors and the rotation angles) and the uniform quaternion rotation of the
CBMC orientations (Rotate_Quaternions, mc_utilities.h:423-457). Bars: 1e-14 absolute for sin
and cos of values in [-1, 1], 1e-13 for the rotated unit-size vector (about ten double-float
operations of ~2^-48 each), far inside what the mixed form's 1e-6 energy bar needs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def quaternion_rotate(v, u, vv, w):
    q0, q1 = np.sqrt(1 - u) * np.sin(2 * np.pi * vv), np.sqrt(1 - u) * np.cos(2 * np.pi * vv)
    q2, q3 = np.sqrt(u) * np.sin(2 * np.pi * w), np.sqrt(u) * np.cos(2 * np.pi * w)
    r = np.array([[1 - 2 * (q2 * q2 + q3 * q3), 2 * (q1 * q2 - q0 * q3), 2 * (q1 * q3 + q0 * q2)],
                  [2 * (q1 * q2 + q0 * q3), 1 - 2 * (q1 * q1 + q3 * q3), 2 * (q2 * q3 - q0 * q1)],
                  [2 * (q1 * q3 - q0 * q2), 2 * (q2 * q3 + q0 * q1), 1 - 2 * (q1 * q1 + q2 * q2)]])
    return r @ v


def test_df_sincos_and_rotation(grx_lib):
    rng = np.random.default_rng(3)
    v = np.concatenate([rng.uniform(0, 1, 20000), rng.uniform(-5, 5, 5000),
                        [0.0, 0.125, 0.25, 0.375, 0.5, 0.625, 0.75, 0.875, 1 - 2 ** -32, -0.125, 1e-9]])
    words = rng.integers(0, 2 ** 32, (len(v), 3), dtype=np.uint64).astype(np.uint32)
    words[:3] = [[0, 0, 0], [2 ** 32 - 1, 2 ** 31, 2 ** 30], [1, 255, 256]]
    out = grx_lib.probe_df_functions(v, words)
    # v enters as a float pair (a 48-bit significand): beyond |v| = 1 its own rounding,
    # 2 pi |v| 2^-48, adds to the 1e-14 of the evaluation
    tol = 1e-14 + 2 * np.pi * np.abs(v) * 2.0 ** -48
    assert np.all(np.abs(out[:, 0] - np.sin(2 * np.pi * v)) < tol)
    assert np.all(np.abs(out[:, 1] - np.cos(2 * np.pi * v)) < tol)
    small = np.abs(v) <= 1
    assert np.max(np.abs(out[small, 0] - np.sin(2 * np.pi * v[small]))) < 1e-14
    u = words.astype(np.float64) * 2.0 ** -32
    ref = np.array([quaternion_rotate(np.array([1.0, 0.5, -0.25]), *u[i]) for i in range(len(v))])
    assert np.max(np.abs(out[:, 2:] - ref)) < 1e-13
