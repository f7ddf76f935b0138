"""ctypes access to the C++ host layer (libpupil_host.so): the mitsuba-style
scene loader and the headless System + WavefrontPTPass."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .build import HOST_LIB

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        abi.load()  # libpt_gb300.so first (libpupil_host.so links it)
        if not HOST_LIB.exists():
            raise RuntimeError(f"{HOST_LIB} is missing: run __graft_entry__.build()")
        lib = C.CDLL(str(HOST_LIB))
        lib.pupil_host_last_error.argtypes = [C.c_char_p, C.c_size_t]
        lib.pupil_scene_load.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]
        lib.pupil_scene_desc.argtypes = [C.c_void_p]
        lib.pupil_scene_desc.restype = C.POINTER(abi.SceneDesc)
        lib.pupil_scene_free.argtypes = [C.c_void_p]
        lib.pupil_scene_free.restype = None
        lib.pupil_run_scene.argtypes = [C.c_char_p, C.c_int, C.c_uint32, C.c_uint32, C.c_void_p,
                                        C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        lib.pupil_write_pfm.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32]
        lib.pupil_run_scene_ex.argtypes = [C.c_char_p, C.c_int, C.c_uint32, C.c_uint32, C.c_char_p, C.c_char_p,
                                           C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        lib.pupil_write_exr.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32]
        _lib = lib
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().pupil_host_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class XmlScene:
    """A scene loaded by the C++ loader; usable wherever a scenes.Scene is
    (GpuScene, the oracle): .desc(), .width, .height, .max_depth."""

    def __init__(self, path_or_text: str, is_text: bool = False):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.pupil_scene_load(path_or_text.encode(), 1 if is_text else 0, C.byref(h))
        if st != 0:
            raise abi.PtError(st, "pupil_scene_load", last_error())
        self.handle = h
        d = self.desc()
        self.width, self.height, self.max_depth = d.width, d.height, d.max_depth

    def desc(self) -> abi.SceneDesc:
        return self.lib.pupil_scene_desc(self.handle).contents

    def __del__(self):
        if getattr(self, "handle", None):
            self.lib.pupil_scene_free(self.handle)
            self.handle = None


def run_scene(path_or_text: str, frames: int, rng: int = abi.RNG_REF_LCG, is_text: bool = False) -> np.ndarray:
    """System + WavefrontPTPass for `frames` frames; returns the final frame (h*w, 4)."""
    lib = load()
    w, h = C.c_uint32(), C.c_uint32()
    st = lib.pupil_run_scene(path_or_text.encode(), 1 if is_text else 0, frames, rng, None, C.byref(w), C.byref(h))
    if st != 0:
        raise abi.PtError(st, "pupil_run_scene", last_error())
    out = np.zeros((w.value * h.value, 4), np.float32)
    st = lib.pupil_run_scene(path_or_text.encode(), 1 if is_text else 0, frames, rng,
                             out.ctypes.data_as(C.c_void_p), C.byref(w), C.byref(h))
    if st != 0:
        raise abi.PtError(st, "pupil_run_scene", last_error())
    return out


def run_scene_ex(path_or_text: str, frames: int, rng: int = abi.RNG_REF_LCG, is_text: bool = False,
                 resume_from: str | None = None, save_to: str | None = None, change_after: int = 0,
                 positions: np.ndarray | None = None, camera=None) -> np.ndarray:
    """System + WavefrontPTPass with the world changing through its events
    (pupil_run_scene_ex); returns the final frame (h*w, 4)."""
    lib = load()
    xs = XmlScene(path_or_text, is_text=is_text)
    out = np.zeros((xs.width * xs.height, 4), np.float32)
    pos = None if positions is None else np.ascontiguousarray(positions, np.float32)
    w, h = C.c_uint32(), C.c_uint32()
    st = lib.pupil_run_scene_ex(path_or_text.encode(), 1 if is_text else 0, frames, rng,
                                resume_from.encode() if resume_from else None, save_to.encode() if save_to else None,
                                change_after, pos.ctypes.data_as(C.c_void_p) if pos is not None else None,
                                C.byref(camera) if camera is not None else None, out.ctypes.data_as(C.c_void_p),
                                C.byref(w), C.byref(h))
    if st != 0:
        raise abi.PtError(st, "pupil_run_scene_ex", last_error())
    return out


def write_exr(path: str, rgba: np.ndarray) -> None:
    """(h, w, 4) float32, first row = top -> uncompressed scanline OpenEXR."""
    lib = load()
    px = np.ascontiguousarray(rgba, np.float32)
    st = lib.pupil_write_exr(str(path).encode(), px.ctypes.data_as(C.c_void_p), px.shape[1], px.shape[0])
    if st != 0:
        raise abi.PtError(st, "pupil_write_exr", last_error())
