"""The library's own single-precision sin, cos, atan2 and acos
(pupiloptixlab_gb300/csrc/pt_trig.h), shared by the GPU kernels and the
oracle so that both sides draw the same directions bit for bit.  Here, on the
host: accuracy against float64 numpy (within 2 ulp for sin, cos and acos,
3 ulp for atan2) and against the C library's functions the reference's
host build would call, plus the special values."""
import numpy as np

import oracle


def ulps(got, exact):
    exact32 = exact.astype(np.float32)
    spacing = np.spacing(np.abs(exact32)).astype(np.float64)
    return np.abs(got.astype(np.float64) - exact) / spacing


def test_sin_cos_within_two_ulp():
    rs = np.random.default_rng(7)
    x = np.concatenate([rs.uniform(0, 2 * np.pi, 400000), rs.uniform(-100, 100, 200000),
                        rs.uniform(-1e5, 1e5, 200000), np.linspace(-7, 7, 100001)]).astype(np.float32)
    xd = x.astype(np.float64)
    assert ulps(oracle.trig(oracle.TRIG_SIN, x), np.sin(xd)).max() <= 2.0
    assert ulps(oracle.trig(oracle.TRIG_COS, x), np.cos(xd)).max() <= 2.0


def test_atan2_within_three_ulp():
    rs = np.random.default_rng(8)
    y = rs.uniform(-2, 2, 600000).astype(np.float32)
    x = rs.uniform(-2, 2, 600000).astype(np.float32)
    y[::3] *= np.float32(1e-3)
    got = oracle.trig(oracle.TRIG_ATAN2, x, y)
    assert ulps(got, np.arctan2(y.astype(np.float64), x.astype(np.float64))).max() <= 3.0


def test_acos_within_two_ulp():
    rs = np.random.default_rng(9)
    x = np.concatenate([rs.uniform(-1, 1, 500000), 1 - rs.uniform(0, 1e-3, 50000), -1 + rs.uniform(0, 1e-3, 50000),
                        np.linspace(-1, 1, 20001)]).astype(np.float32)
    assert ulps(oracle.trig(oracle.TRIG_ACOS, x), np.arccos(x.astype(np.float64))).max() <= 2.0


def test_special_values():
    f = np.float32
    s = oracle.trig(oracle.TRIG_SIN, np.array([0.0, -0.0, np.inf, -np.inf, np.nan], f))
    assert s[0] == 0 and s[1] == 0 and np.isnan(s[2:]).all()
    assert oracle.trig(oracle.TRIG_COS, np.array([0.0], f))[0] == 1.0
    a = oracle.trig(oracle.TRIG_ATAN2, np.array([0.0, -1.0, -1.0, 1.0, np.inf, np.nan], f),
                    np.array([0.0, 0.0, -0.0, np.inf, np.inf, 1.0], f))
    assert a[0] == 0 and a[1] == np.float32(np.pi) and a[2] == -np.float32(np.pi)
    assert a[3] == np.float32(np.pi / 2) and a[4] == np.float32(np.pi / 4) and np.isnan(a[5])
    c = oracle.trig(oracle.TRIG_ACOS, np.array([1.0, -1.0, 0.0, 1.5, np.nan], f))
    assert c[0] == 0 and c[1] == np.float32(np.pi) and c[2] == np.float32(np.pi / 2) and np.isnan(c[3:]).all()


def test_close_to_the_c_library():
    """The reference's host build would call the C library's sinf/cosf: the
    shared functions stay within 2 ulp of them on the sampling range."""
    import ctypes
    import ctypes.util
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.sinf.restype = libm.cosf.restype = ctypes.c_float
    libm.sinf.argtypes = libm.cosf.argtypes = [ctypes.c_float]
    x = np.random.default_rng(10).uniform(0, 2 * np.pi, 20000).astype(np.float32)
    ls = np.array([libm.sinf(float(v)) for v in x], np.float32)
    lc = np.array([libm.cosf(float(v)) for v in x], np.float32)
    assert ulps(oracle.trig(oracle.TRIG_SIN, x), ls.astype(np.float64)).max() <= 2.0
    assert ulps(oracle.trig(oracle.TRIG_COS, x), lc.astype(np.float64)).max() <= 2.0
