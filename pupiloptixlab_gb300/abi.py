"""ctypes mirror of include/pt_api.h and the loader of libpt_gb300.so.

The structures here must match the C header field for field; the tests
check their sizes against the header through the library.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .build import LIB

c_float_p = C.POINTER(C.c_float)
c_uint_p = C.POINTER(C.c_uint32)

PT_OK = 0
PT_ERR_UNSUPPORTED = 6
MAX_PRIMITIVES = (1 << 27) - 1  # PT_MAX_PRIMITIVES: per scene after instancing, and per multi-scene launch
STATUS_NAMES = {0: "PT_OK", 1: "PT_ERR_INVALID", 2: "PT_ERR_CUDA", 3: "PT_ERR_OOM", 4: "PT_ERR_TIMEOUT",
                5: "PT_ERR_NAN", 6: "PT_ERR_UNSUPPORTED", 7: "PT_ERR_OOB", 8: "PT_ERR_STATE"}

MAT_DIFFUSE, MAT_DIELECTRIC, MAT_ROUGH_DIELECTRIC, MAT_CONDUCTOR, MAT_ROUGH_CONDUCTOR, MAT_PLASTIC, MAT_ROUGH_PLASTIC = range(1, 8)
MATERIAL_NAMES = {1: "diffuse", 2: "dielectric", 3: "roughdielectric", 4: "conductor", 5: "roughconductor",
                  6: "plastic", 7: "roughplastic"}
TEX_RGB, TEX_BITMAP, TEX_CHECKERBOARD = 0, 1, 2
SHAPE_MESH, SHAPE_SPHERE, SHAPE_CURVES = 0, 1, 2
CURVE_LINEAR, CURVE_QUADRATIC_BSPLINE, CURVE_CUBIC_BSPLINE, CURVE_CATMULL_ROM = 0, 1, 2, 3
INST_FLIP_NORMALS, INST_FLIP_TEXCOORDS = 1, 2
ENV_NONE, ENV_CONST, ENV_MAP = 0, 1, 2
TEX_ADDRESS_WRAP, TEX_ADDRESS_CLAMP, TEX_ADDRESS_MIRROR = 0, 1, 2
TEX_FILTER_POINT, TEX_FILTER_LINEAR = 0, 1
RNG_REF_LCG, RNG_PCG32 = 0, 1
RENDER_NO_MATERIAL_SORT, RENDER_COUNTERS, RENDER_NO_GRAPH, RENDER_KERNEL_TIMING = 1, 2, 4, 8
RENDER_DROP_NONFINITE = 16
RENDER_CHECK_FINITE = 32
LOBE_DELTA = (1 << 5) | (1 << 6)


class TextureDesc(C.Structure):
    _fields_ = [("type", C.c_uint32), ("color0", C.c_float * 3), ("color1", C.c_float * 3),
                ("uv_transform", C.c_float * 8), ("pixels", C.c_void_p), ("width", C.c_uint32),
                ("height", C.c_uint32), ("address_mode", C.c_uint32), ("filter", C.c_uint32)]


class MaterialDesc(C.Structure):
    _fields_ = [("type", C.c_uint32), ("twosided", C.c_uint32), ("nonlinear", C.c_uint32),
                ("int_ior", C.c_float), ("ext_ior", C.c_float), ("tex", TextureDesc * 4)]


class MeshDesc(C.Structure):
    _fields_ = [("positions", c_float_p), ("normals", c_float_p), ("texcoords", c_float_p),
                ("indices", c_uint_p), ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32)]


class SphereDesc(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("radius", C.c_float)]


class InstanceDesc(C.Structure):
    _fields_ = [("shape_type", C.c_uint32), ("shape_index", C.c_uint32), ("material", C.c_uint32),
                ("flags", C.c_uint32), ("to_world", C.c_float * 16), ("is_emitter", C.c_uint32),
                ("radiance", C.c_float * 3), ("radiance_textured", C.c_uint32), ("radiance_tex", TextureDesc)]


class CameraDesc(C.Structure):
    _fields_ = [("sample_to_camera", C.c_float * 16), ("camera_to_world", C.c_float * 16)]


class EnvDesc(C.Structure):
    _fields_ = [("type", C.c_uint32), ("radiance", C.c_float * 3), ("pixels", C.c_void_p), ("width", C.c_uint32),
                ("height", C.c_uint32), ("scale", C.c_float), ("to_world", C.c_float * 16)]


class CurvesDesc(C.Structure):
    _fields_ = [("positions", c_float_p), ("radii", c_float_p), ("segments", c_uint_p),
                ("num_points", C.c_uint32), ("num_segments", C.c_uint32), ("type", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(MeshDesc)), ("num_meshes", C.c_uint32),
                ("spheres", C.POINTER(SphereDesc)), ("num_spheres", C.c_uint32),
                ("materials", C.POINTER(MaterialDesc)), ("num_materials", C.c_uint32),
                ("instances", C.POINTER(InstanceDesc)), ("num_instances", C.c_uint32),
                ("env", EnvDesc), ("camera", CameraDesc),
                ("width", C.c_uint32), ("height", C.c_uint32), ("max_depth", C.c_uint32),
                ("curves", C.POINTER(CurvesDesc)), ("num_curves", C.c_uint32)]


class DeviceOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("flags", C.c_uint32)]


class BvhOpts(C.Structure):
    _fields_ = [("width", C.c_uint32), ("max_leaf_size", C.c_uint32), ("smem_nodes", C.c_uint32),
                ("flags", C.c_uint32)]


BVH_FAST_BUILD = 1
BVH_BUILDER_RADIX, BVH_BUILDER_PLOC = 0, 1


class BvhStats(C.Structure):
    _fields_ = [("width", C.c_uint32), ("num_nodes", C.c_uint32), ("num_leaves", C.c_uint32),
                ("num_prims", C.c_uint32), ("max_depth", C.c_uint32), ("sah_cost", C.c_float),
                ("build_ms", C.c_float), ("node_bytes", C.c_uint64), ("prim_bytes", C.c_uint64),
                ("builder", C.c_uint32)]


class RenderParams(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("max_depth", C.c_uint32), ("seed", C.c_uint32), ("sample_cnt", C.c_uint32),
                ("accumulate", C.c_uint32), ("rng", C.c_uint32), ("wave_spp", C.c_uint32),
                ("block_size", C.c_uint32), ("flags", C.c_uint32)]


class FrameBuffers(C.Structure):
    _fields_ = [("accum", C.c_void_p), ("frame", C.c_void_p), ("albedo", C.c_void_p), ("normal", C.c_void_p),
                ("test", C.c_void_p)]


class RenderStats(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("nodes_visited", C.c_uint64), ("prims_tested", C.c_uint64), ("shadow_nodes_visited", C.c_uint64),
                ("shadow_prims_tested", C.c_uint64), ("render_ms", C.c_float), ("extend_ms", C.c_float),
                ("shadow_ms", C.c_float), ("shade_ms", C.c_float), ("extend_launches", C.c_uint32),
                ("shadow_launches", C.c_uint32), ("shade_launches", C.c_uint32), ("kernel_launches", C.c_uint32),
                ("waves", C.c_uint32), ("overflow", C.c_uint32), ("nonfinite_samples", C.c_uint32)]


class TuneResult(C.Structure):
    _fields_ = [("bvh_width", C.c_uint32), ("block_size", C.c_uint32), ("wave_paths", C.c_uint32),
                ("trials", C.c_uint32), ("msamples_per_s", C.c_float), ("baseline_msamples_per_s", C.c_float)]


# (name, restype, argtypes) of every entry point declared in include/pt_api.h.
class DenoiserOpts(C.Structure):
    _fields_ = [("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("seed", C.c_uint64)]


class DenoiseIO(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("color", C.c_void_p), ("albedo", C.c_void_p),
                ("normal", C.c_void_p), ("output", C.c_void_p), ("tile", C.c_uint32), ("fallback_rel", C.c_float),
                ("fallback_sigma", C.c_float), ("tile_fallback", C.c_void_p), ("flags", C.c_uint32)]


DENOISE_FLIP_ENSEMBLE = 1


class DenoiseStats(C.Structure):
    _fields_ = [("tiles", C.c_uint32), ("fallback_tiles", C.c_uint32), ("last_ms", C.c_float)]


PROTOTYPES = [
    ("pt_api_version", C.c_int, []),
    ("pt_last_error", C.c_int, [C.c_char_p, C.c_size_t]),
    ("pt_context_create", C.c_int, [C.POINTER(DeviceOpts), C.POINTER(C.c_void_p)]),
    ("pt_context_destroy", C.c_int, [C.c_void_p]),
    ("pt_scene_upload", C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(C.c_void_p)]),
    ("pt_scene_destroy", C.c_int, [C.c_void_p]),
    ("pt_scene_set_camera", C.c_int, [C.c_void_p, C.POINTER(CameraDesc)]),
    ("pt_scene_update_vertices", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
    ("pt_scene_update_all_vertices", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("pt_scene_num_prims", C.c_int, [C.c_void_p, c_uint_p, c_uint_p]),
    ("pt_scene_num_curves", C.c_int, [C.c_void_p, c_uint_p, c_uint_p]),
    ("pt_bvh_build", C.c_int, [C.c_void_p, C.POINTER(BvhOpts), C.c_void_p]),
    ("pt_bvh_refit", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pt_bvh_get_stats", C.c_int, [C.c_void_p, C.POINTER(BvhStats)]),
    ("pt_render", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.POINTER(FrameBuffers), C.c_void_p]),
    ("pt_render_get_stats", C.c_int, [C.c_void_p, C.POINTER(RenderStats)]),
    ("pt_render_batch", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(RenderParams), C.c_void_p, C.c_uint32,
                                  C.c_void_p]),
    ("pt_render_batch_get_stats", C.c_int, [C.c_void_p, C.POINTER(RenderStats)]),
    ("pt_render_noalloc", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.POINTER(FrameBuffers), C.c_void_p]),
    ("pt_autotune", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.POINTER(FrameBuffers), C.POINTER(TuneResult),
                              C.c_void_p]),
    ("pt_trace_rays", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p]),
    ("pt_bsdf_eval_batch", C.c_int, [C.c_void_p] * 5 + [C.c_uint32, C.c_void_p]),
    ("pt_bsdf_sample_batch", C.c_int, [C.c_void_p] * 7 + [C.c_uint32, C.c_void_p]),
    ("pt_trig_eval", C.c_int, [C.c_uint32] + [C.c_void_p] * 4 + [C.c_uint32, C.c_void_p]),
    ("pt_conv_set_wait_limit", C.c_int, [C.c_uint64, C.c_uint32]),
    ("pt_denoiser_create", C.c_int, [C.c_void_p, C.POINTER(DenoiserOpts), C.POINTER(C.c_void_p)]),
    ("pt_denoiser_destroy", None, [C.c_void_p]),
    ("pt_denoiser_num_params", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    ("pt_denoiser_layer", C.c_int, [C.c_void_p, C.c_uint32, c_uint_p, c_uint_p, C.POINTER(C.c_uint64)]),
    ("pt_denoiser_get_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pt_denoiser_set_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pt_denoiser_get_state", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pt_denoiser_set_state", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pt_denoiser_compute_grads", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                            C.POINTER(C.c_float), C.c_void_p]),
    ("pt_denoiser_get_grads", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pt_denoiser_train_step", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]),
    ("pt_denoiser_read_loss", C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    ("pt_denoiser_set_lr", C.c_int, [C.c_void_p, C.c_float]),
    ("pt_denoiser_forward", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                                      C.c_void_p]),
    ("pt_denoise", C.c_int, [C.c_void_p, C.POINTER(DenoiseIO), C.c_void_p]),
    ("pt_denoise_get_stats", C.c_int, [C.c_void_p, C.POINTER(DenoiseStats)]),
    ("pt_denoise_pack", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                  C.c_void_p]),
    ("pt_conv3x3_forward", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                                     C.c_void_p, C.c_uint32, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("pt_conv3x3_backward_data", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                                           C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("pt_conv3x3_backward_weights", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                                              C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("pt_camera_make", C.c_int, [C.c_float, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_float),
                                 C.POINTER(CameraDesc)]),
]

_lib = None


def lib_path() -> Path:
    return LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load libpt_gb300.so.  Raises if it has not been built: there is no
    fallback implementation."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        if build_if_missing:
            from .build import build_library
            build_library()
        else:
            raise RuntimeError(f"{LIB} is missing: run __graft_entry__.build() (python -m pupiloptixlab_gb300.build)")
    lib = C.CDLL(str(LIB))
    for name, res, args in PROTOTYPES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PtError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def last_error(lib=None) -> str:
    lib = lib or load()
    buf = C.create_string_buffer(1024)
    lib.pt_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, where: str, lib=None) -> None:
    if status != PT_OK:
        raise PtError(status, where, last_error(lib))
