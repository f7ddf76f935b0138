"""CPU oracle for the path-tracing-with-MIS path -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_build/liboracle.so (the C++ restatement of the reference's
integrator and material math, oracle/pt_oracle.cpp) and, when it was built
in a container holding the PupilOptixLab tree, oracle/_ref/libpupil_ref.so
(the reference's own headers compiled for the host, oracle/ref_kat.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs may import this package.  The product library never uses it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libpupil_ref.so"

_lib = None
_ref = None

_VP = C.c_void_p


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def build() -> None:
    subprocess.run(["make", "-C", str(HERE), "-s", "all"], check=True)


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = C.CDLL(str(LIB))
        from pupiloptixlab_gb300 import abi
        lib.oracle_scene_create.argtypes = [C.POINTER(abi.SceneDesc), C.c_int, C.POINTER(C.c_void_p)]
        lib.oracle_scene_destroy.argtypes = [_VP]
        lib.oracle_scene_destroy.restype = None
        lib.oracle_scene_num_prims.argtypes = [_VP, _VP, _VP]
        lib.oracle_scene_num_curves.argtypes = [_VP, _VP, _VP]
        lib.oracle_curve.argtypes = [C.c_uint32, _VP, _VP, _VP, _VP, C.c_uint32]
        lib.oracle_scene_curve_pieces.argtypes = [_VP, _VP]
        lib.oracle_scene_world_triangles.argtypes = [_VP, _VP]
        lib.oracle_trace_rays.argtypes = [_VP, _VP, _VP, C.c_uint32, C.c_int, C.c_int, C.c_int]
        lib.oracle_camera_rays.argtypes = [_VP, C.c_uint32, C.c_uint32, _VP]
        lib.oracle_render.argtypes = [_VP, C.POINTER(abi.RenderParams), _VP, _VP, _VP, _VP, _VP, _VP, C.c_uint32,
                                      C.c_int]
        lib.oracle_render_samples.argtypes = [_VP, C.POINTER(abi.RenderParams), C.c_uint32, _VP, C.c_uint32, _VP,
                                              C.c_int]
        lib.oracle_bsdf_eval.argtypes = [_VP] * 5 + [C.c_uint32]
        lib.oracle_bsdf_sample.argtypes = [_VP] * 7 + [C.c_uint32]
        lib.oracle_material_local_bsdf.argtypes = [C.POINTER(abi.MaterialDesc), C.c_float, C.c_float, _VP]
        lib.oracle_rng_stream.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _VP]
        lib.oracle_pcg32_raw.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, _VP]
        lib.oracle_emitter_sample.argtypes = [_VP, C.c_int, _VP, _VP, C.c_uint32]
        lib.oracle_emitter_table.argtypes = [_VP, _VP, _VP, C.c_uint32]
        for nm in ("oracle_fresnel_dielectric", "oracle_fresnel_conductor", "oracle_fresnel_diffuse", "oracle_ggx",
                   "oracle_sampling"):
            getattr(lib, nm).argtypes = [_VP, _VP, C.c_uint32]
        lib.oracle_emitter_sample_raw.argtypes = [C.c_int, _VP, _VP, _VP, C.c_uint32]
        lib.oracle_select_emitter.argtypes = [_VP, C.c_uint32, C.c_int, _VP, _VP, C.c_uint32]
        lib.oracle_envmap.argtypes = [C.c_int, _VP, C.c_uint32, C.c_uint32, C.c_float, _VP, _VP, _VP, _VP,
                                      C.c_uint32, _VP]
        lib.oracle_camera_make.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, _VP,
                                           C.POINTER(abi.CameraDesc)]
        lib.oracle_trig.argtypes = [C.c_uint32, _VP, _VP, _VP, C.c_uint32]
        _lib = lib
    return _lib


def load_ref() -> C.CDLL | None:
    """The reference-compiled KAT library, or None where it was not built."""
    global _ref
    if _ref is None and REF_LIB.exists():
        r = C.CDLL(str(REF_LIB))
        r.ref_bsdf_eval.argtypes = [_VP] * 5 + [C.c_uint32]
        r.ref_bsdf_sample.argtypes = [_VP] * 7 + [C.c_uint32]
        r.ref_rng_stream.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, _VP]
        r.ref_fresnel_dielectric.argtypes = [_VP, _VP, C.c_uint32]
        r.ref_fresnel_conductor.argtypes = [_VP, _VP, C.c_uint32]
        r.ref_fresnel_diffuse.argtypes = [_VP, _VP, C.c_uint32]
        r.ref_ggx.argtypes = [_VP, _VP, C.c_uint32]
        r.ref_sampling.argtypes = [_VP, _VP, C.c_uint32]
        r.ref_emitter_sample.argtypes = [C.c_int, _VP, _VP, _VP, C.c_uint32]
        r.ref_select_emitter.argtypes = [_VP, C.c_uint32, C.c_int, _VP, _VP, C.c_uint32]
        r.ref_envmap.argtypes = [C.c_int, _VP, C.c_uint32, C.c_uint32, C.c_float, _VP, _VP, _VP, _VP, _VP,
                                 C.c_float, _VP, _VP, C.c_uint32]
        r.ref_curve.argtypes = [C.c_uint32, _VP, _VP, _VP, _VP, C.c_uint32]
        _ref = r
    return _ref


class OracleScene:
    """The oracle's copy of a scene (host BVH2 optional)."""

    def __init__(self, scene, bvh: bool = True):
        from pupiloptixlab_gb300 import abi
        self.lib = load()
        self.scene = scene
        desc = scene.desc()
        h = C.c_void_p()
        st = self.lib.oracle_scene_create(C.byref(desc), 1 if bvh else 0, C.byref(h))
        if st != 0:
            raise RuntimeError(f"oracle_scene_create failed: {abi.STATUS_NAMES.get(st, st)}")
        self.handle = h
        self.width, self.height = scene.width, scene.height

    def __del__(self):
        if getattr(self, "handle", None):
            self.lib.oracle_scene_destroy(self.handle)
            self.handle = None

    def num_prims(self):
        a, b = C.c_uint32(), C.c_uint32()
        self.lib.oracle_scene_num_prims(self.handle, C.byref(a), C.byref(b))
        return a.value, b.value

    def num_curves(self):
        a, b = C.c_uint32(), C.c_uint32()
        self.lib.oracle_scene_num_curves(self.handle, C.byref(a), C.byref(b))
        return a.value, b.value

    def curve_pieces(self) -> np.ndarray:
        """(pieces, 12): c0 xyz, r0, c1 xyz, r1, u0, u1, kind, segment."""
        _, n = self.num_curves()
        out = np.zeros((n, 12), np.float32)
        if n:
            self.lib.oracle_scene_curve_pieces(self.handle, _ptr(out))
        return out

    def world_triangles(self) -> np.ndarray:
        nt, _ = self.num_prims()
        out = np.zeros((nt, 9), np.float32)
        self.lib.oracle_scene_world_triangles(self.handle, _ptr(out))
        return out

    def camera_rays(self, rng_mode: int, seed: int) -> np.ndarray:
        out = np.zeros((self.width * self.height, 8), np.float32)
        self.lib.oracle_camera_rays(self.handle, rng_mode, seed, _ptr(out))
        return out

    def trace(self, rays: np.ndarray, anyhit: bool = False, brute_force: bool = False, threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32)
        hits = np.zeros((rays.shape[0], 4), np.float32)
        self.lib.oracle_trace_rays(self.handle, _ptr(rays), _ptr(hits), rays.shape[0], 1 if anyhit else 0,
                                   1 if brute_force else 0, threads)
        return hits

    def render(self, params, pixels: np.ndarray | None = None, threads: int = 0, accum: np.ndarray | None = None):
        n = self.width * self.height
        acc = np.zeros((n, 4), np.float32) if accum is None else accum
        frame = np.zeros((n, 4), np.float32)
        albedo = np.zeros((n, 3), np.float32)
        normal = np.zeros((n, 3), np.float32)
        test = np.zeros(n, np.float32)
        px = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
        st = self.lib.oracle_render(self.handle, C.byref(params), _ptr(acc), _ptr(frame), _ptr(albedo), _ptr(normal),
                                    _ptr(test), _ptr(px), 0 if px is None else px.shape[0], threads)
        if st != 0:
            raise RuntimeError(f"oracle_render failed: {st}")
        return {"accum": acc, "frame": frame, "albedo": albedo, "normal": normal, "test": test}

    def render_samples(self, params, frame_seed: int, pixels: np.ndarray | None = None, threads: int = 0):
        px = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
        n = self.width * self.height if px is None else px.shape[0]
        out = np.zeros((n, 3), np.float32)
        self.lib.oracle_render_samples(self.handle, C.byref(params), frame_seed, _ptr(px),
                                       0 if px is None else px.shape[0], _ptr(out), threads)
        return out

    def emitter_sample(self, index: int, inp: np.ndarray) -> np.ndarray:
        inp = np.ascontiguousarray(inp, np.float32)
        out = np.zeros((inp.shape[0], 12), np.float32)
        st = self.lib.oracle_emitter_sample(self.handle, index, _ptr(inp), _ptr(out), inp.shape[0])
        if st != 0:
            raise RuntimeError(f"oracle_emitter_sample failed: {st}")
        return out

    def emitter_table(self) -> np.ndarray:
        cnt = C.c_uint32()
        buf = np.zeros((4096, 2), np.float32)
        self.lib.oracle_emitter_table(self.handle, C.byref(cnt), _ptr(buf), 4096)
        return buf[: min(cnt.value, 4096)]


def envmap(mode: int, pixels: np.ndarray, scale: float, to_world3: np.ndarray, to_local3: np.ndarray,
           inp: np.ndarray):
    """EnvMapEmitter sample (mode 0, inp (n, 2) xi -> (n, 7)) or eval (mode 1,
    inp (n, 6) origin+direction -> (n, 4)); also returns the CDF tables."""
    lib = load()
    px = np.ascontiguousarray(pixels, np.float32)
    h, w = px.shape[:2]
    inp = np.ascontiguousarray(inp, np.float32)
    n = inp.shape[0]
    out = np.zeros((n, 7 if mode == 0 else 4), np.float32)
    tables = np.zeros((h + 1) + (w + 1) * h + h + 1, np.float32)
    tw = np.ascontiguousarray(to_world3, np.float32)
    tl = np.ascontiguousarray(to_local3, np.float32)
    st = lib.oracle_envmap(mode, _ptr(px), w, h, scale, _ptr(tw), _ptr(tl), _ptr(inp), _ptr(out), n, _ptr(tables))
    if st != 0:
        raise RuntimeError(f"oracle_envmap failed: {st}")
    return out, tables


def curve(curve_type: int, ctrl: np.ndarray, u: np.ndarray, ps: np.ndarray, lib=None) -> np.ndarray:
    """Curve evaluation KAT: ctrl (n, 4, 4) control points, u (n,), ps (n, 3)
    -> (n, 15) position4, velocity4, acceleration3, surface normal3, 0.
    lib = load_ref() evaluates the reference's own interpolators instead."""
    ctrl = np.ascontiguousarray(ctrl, np.float32)
    u = np.ascontiguousarray(u, np.float32)
    ps = np.ascontiguousarray(ps, np.float32)
    n = u.shape[0]
    out = np.zeros((n, 15), np.float32)
    if lib is None:
        st = load().oracle_curve(curve_type, _ptr(ctrl), _ptr(u), _ptr(ps), _ptr(out), n)
    else:
        st = lib.ref_curve(curve_type, _ptr(ctrl), _ptr(u), _ptr(ps), _ptr(out), n)
    if st != 0:
        raise RuntimeError(f"curve KAT failed: {st}")
    return out


def bsdf_eval(bsdf, wo, wi):
    lib = load()
    n = bsdf.shape[0]
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    lib.oracle_bsdf_eval(_ptr(np.ascontiguousarray(bsdf, np.float32)), _ptr(np.ascontiguousarray(wo, np.float32)),
                         _ptr(np.ascontiguousarray(wi, np.float32)), _ptr(f), _ptr(pdf), n)
    return f, pdf


def bsdf_sample(bsdf, wo, rng_state):
    lib = load()
    n = bsdf.shape[0]
    rng = np.ascontiguousarray(rng_state, np.uint32).copy()
    wi = np.zeros((n, 3), np.float32)
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    typ = np.zeros(n, np.uint32)
    lib.oracle_bsdf_sample(_ptr(np.ascontiguousarray(bsdf, np.float32)), _ptr(np.ascontiguousarray(wo, np.float32)),
                           _ptr(rng), _ptr(wi), _ptr(f), _ptr(pdf), _ptr(typ), n)
    return wi, f, pdf, typ, rng


def material_local_bsdf(mat, u: float = 0.0, v: float = 0.0) -> np.ndarray:
    out = np.zeros(16, np.float32)
    load().oracle_material_local_bsdf(C.byref(mat), u, v, _ptr(out))
    return out


def rng_stream(mode: int, pixel: int, seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float32)
    load().oracle_rng_stream(mode, pixel, seed, n, _ptr(out))
    return out


def pcg32_raw(initstate: int, initseq: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    load().oracle_pcg32_raw(initstate, initseq, n, _ptr(out))
    return out


def camera_make(fov_y, aspect, near, far, to_world):
    from pupiloptixlab_gb300 import abi
    cam = abi.CameraDesc()
    tw = np.ascontiguousarray(np.asarray(to_world, np.float32).reshape(16))
    st = load().oracle_camera_make(fov_y, aspect, near, far, _ptr(tw), C.byref(cam))
    if st != 0:
        raise RuntimeError("oracle_camera_make failed")
    return cam


TRIG_SIN, TRIG_COS, TRIG_ATAN2, TRIG_ACOS = 0, 1, 2, 3


def trig(fn: int, x, y=None) -> np.ndarray:
    """The shared trigonometry of pt_trig.h evaluated on the host."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(x if y is None else y, np.float32)
    out = np.empty_like(x)
    if load().oracle_trig(fn, _ptr(x), _ptr(y), _ptr(out), x.size) != 0:
        raise RuntimeError("oracle_trig failed")
    return out
