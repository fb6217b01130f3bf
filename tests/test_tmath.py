"""Accuracy of the deterministic atan/sin/cos (ecmg_tmath.h) shared by the GPU
kernels and the oracle, against float64 and against the host libm."""
import ctypes as C

import numpy as np


def _ulp(v, ref):
    return np.abs(v.astype(np.float64) - ref) / np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)


def test_tmath_error_bounds(port):
    L = port.lib
    # reach the header through the oracle library's own compiled copies
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(0, 1.2, 20000), np.exp(rng.uniform(-20, 8, 5000)), [0.0, 1.0, 1e-30]])
    x = np.concatenate([x, -x]).astype(np.float32)
    a = np.concatenate([rng.uniform(-np.pi / 2, np.pi / 2, 20000), rng.uniform(-0.01, 0.01, 2000)]).astype(np.float32)
    got_at = np.array([_call_atan(L, v) for v in x], np.float32)
    sc = np.array([_call_sincos(L, v) for v in a], np.float32)
    e_at = _ulp(got_at[x != 0], np.arctan(x[x != 0].astype(np.float64)))
    nz = a != 0
    e_s = _ulp(sc[nz, 0], np.sin(a[nz].astype(np.float64)))
    e_c = _ulp(sc[:, 1], np.cos(a.astype(np.float64)))
    assert e_at.max() <= 2.5 and e_s.max() <= 1.5 and e_c.max() <= 1.5, (e_at.max(), e_s.max(), e_c.max())
    assert got_at[x == 0].tolist() == [0.0] * int((x == 0).sum())


def _call_atan(L, v):
    L.og_test_atanf.restype = C.c_float
    L.og_test_atanf.argtypes = [C.c_float]
    return L.og_test_atanf(float(v))


def _call_sincos(L, v):
    s, c = C.c_float(), C.c_float()
    L.og_test_sincosf.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.og_test_sincosf(float(v), C.byref(s), C.byref(c))
    return s.value, c.value


def test_sincos_is_odd_even_symmetric_bit_for_bit(port):
    """the agent half-plane takes the rotation by -angle from the same
    ecmg_sincosf call as the rotation by +angle (sin(-a) = -sin a,
    cos(-a) = cos a): true bit for bit on every 29th binary32 value of
    (0, pi/2], the range of the atan that produces the angle (a zero angle
    calls it twice: sin(-0) rounds to +0)"""
    L = port.lib
    L.og_test_sincos_symmetry.restype = C.c_long
    L.og_test_sincos_symmetry.argtypes = [C.c_uint]
    assert L.og_test_sincos_symmetry(29) == 0
