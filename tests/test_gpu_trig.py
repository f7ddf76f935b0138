"""The library's trigonometry (pt_trig.h) on the GPU: the device results equal
the oracle's host build of the same source bit for bit (what makes whole
paths bit-identical), stay within 2 ulp (sin, cos, acos) and 3 ulp (atan2)
of the exact values, and within a few ulp of CUDA's own sinf, cosf, atan2f
and acosf, the functions the reference's kernels call."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from pupiloptixlab_gb300 import abi

pytestmark = pytest.mark.gpu


def device_trig(lib, fn, x, y=None):
    xd = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    yd = torch.from_numpy(np.ascontiguousarray(x if y is None else y, np.float32)).cuda()
    out, plat = torch.empty_like(xd), torch.empty_like(xd)
    st = lib.pt_trig_eval(fn, C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), C.c_void_p(out.data_ptr()),
                          C.c_void_p(plat.data_ptr()), xd.numel(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    abi.check(st, "pt_trig_eval", lib)
    return out.cpu().numpy(), plat.cpu().numpy()


def ulps(got, exact):
    spacing = np.spacing(np.abs(exact.astype(np.float32))).astype(np.float64)
    return np.abs(got.astype(np.float64) - exact) / spacing


def inputs():
    rs = np.random.default_rng(11)
    x = np.concatenate([rs.uniform(0, 2 * np.pi, 1 << 20), rs.uniform(-1e4, 1e4, 1 << 18),
                        np.array([0.0, -0.0, np.pi, 2 * np.pi, 1e5], np.float64)]).astype(np.float32)
    u = np.concatenate([rs.uniform(-1, 1, 1 << 20), np.array([-1.0, 1.0, 0.0, 0.5, -0.5])]).astype(np.float32)
    y = rs.uniform(-2, 2, 1 << 20).astype(np.float32)
    z = rs.uniform(-2, 2, 1 << 20).astype(np.float32)
    return x, u, y, z


def test_device_equals_host_bit_for_bit(ptlib):
    x, u, y, z = inputs()
    for fn, a, b in ((oracle.TRIG_SIN, x, None), (oracle.TRIG_COS, x, None), (oracle.TRIG_ATAN2, z, y),
                     (oracle.TRIG_ACOS, u, None)):
        dev, _ = device_trig(ptlib, fn, a, b)
        host = oracle.trig(fn, a, b)
        assert np.array_equal(dev.view(np.uint32), host.view(np.uint32)), fn


def test_accuracy_and_distance_to_cuda_math(ptlib):
    x, u, y, z = inputs()
    xd, ud = x.astype(np.float64), u.astype(np.float64)
    cases = ((oracle.TRIG_SIN, x, None, np.sin(xd), 2.0), (oracle.TRIG_COS, x, None, np.cos(xd), 2.0),
             (oracle.TRIG_ATAN2, z, y, np.arctan2(y.astype(np.float64), z.astype(np.float64)), 3.0),
             (oracle.TRIG_ACOS, u, None, np.arccos(ud), 2.0))
    for fn, a, b, exact, bound in cases:
        ours, cuda = device_trig(ptlib, fn, a, b)
        e_ours, e_cuda = ulps(ours, exact), ulps(cuda, exact)
        print(f"fn {fn}: ours max {e_ours.max():.2f} ulp, CUDA max {e_cuda.max():.2f} ulp, "
              f"bit-equal to CUDA {np.mean(ours == cuda) * 100:.2f}%")
        assert e_ours.max() <= bound
        assert ulps(ours, cuda.astype(np.float64)).max() <= bound + 4.0
