"""C-ABI checks that need no GPU: the library loads, exports every entry
point include/pt_api.h declares, the ctypes mirror has the C layouts, the
host-only helpers agree with the oracle, and calls that need a device fail
with a status instead of crashing."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from pupiloptixlab_gb300 import abi

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "pt_api.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|void)\s+(pt_\w+)\s*\(", text, re.M)))


def test_header_declares_expected_api():
    names = declared_functions()
    for n in ("pt_context_create", "pt_scene_upload", "pt_bvh_build", "pt_bvh_refit", "pt_render",
              "pt_trace_rays", "pt_bsdf_eval_batch", "pt_bsdf_sample_batch", "pt_camera_make", "pt_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(ptlib):
    for name in declared_functions():
        assert hasattr(ptlib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.lib_path())], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (pt_\w+)", out))
    assert set(declared_functions()) <= exported
    assert {p[0] for p in abi.PROTOTYPES} == set(declared_functions())


STRUCTS = ["pt_texture_desc", "pt_material_desc", "pt_mesh_desc", "pt_sphere_desc", "pt_instance_desc",
           "pt_camera_desc", "pt_env_desc", "pt_scene_desc", "pt_device_opts", "pt_bvh_opts", "pt_bvh_stats",
           "pt_render_params", "pt_frame_buffers", "pt_render_stats", "pt_tune_result"]
MIRROR = {"pt_texture_desc": abi.TextureDesc, "pt_material_desc": abi.MaterialDesc, "pt_mesh_desc": abi.MeshDesc,
          "pt_sphere_desc": abi.SphereDesc, "pt_instance_desc": abi.InstanceDesc, "pt_camera_desc": abi.CameraDesc,
          "pt_env_desc": abi.EnvDesc, "pt_scene_desc": abi.SceneDesc, "pt_device_opts": abi.DeviceOpts,
          "pt_bvh_opts": abi.BvhOpts, "pt_bvh_stats": abi.BvhStats, "pt_render_params": abi.RenderParams,
          "pt_frame_buffers": abi.FrameBuffers, "pt_render_stats": abi.RenderStats,
          "pt_tune_result": abi.TuneResult}


def test_ctypes_layouts_match_header(tmp_path):
    src = tmp_path / "sizes.c"
    body = "\n".join(f'printf("{s} %zu\\n", sizeof({s}));' for s in STRUCTS)
    src.write_text(f'#include <stdio.h>\n#include "pt_api.h"\nint main(void) {{ {body} return 0; }}\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    sizes = dict((l.split()[0], int(l.split()[1])) for l in out.strip().splitlines())
    for s in STRUCTS:
        assert C.sizeof(MIRROR[s]) == sizes[s], s


def test_header_constants_match_the_mirror(tmp_path):
    src = tmp_path / "consts.c"
    src.write_text('#include <stdio.h>\n#include "pt_api.h"\n'
                   'int main(void) { printf("%u %d\\n", PT_MAX_PRIMITIVES, PT_ERR_UNSUPPORTED); return 0; }\n')
    exe = tmp_path / "consts"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == abi.MAX_PRIMITIVES == (1 << 27) - 1
    assert int(out[1]) == abi.PT_ERR_UNSUPPORTED


def test_camera_make_matches_oracle(ptlib):
    import oracle
    from pupiloptixlab_gb300 import scenes
    tw = scenes.look_at_to_world((1.0, 2.0, 5.0), (0.0, 0.5, 0.0))
    cam = scenes.camera(40.0, 16 / 9, tw)
    ref = oracle.camera_make(40.0, 16 / 9, 0.01, 10000.0, tw.astype(np.float32))
    assert np.array_equal(np.array(cam.sample_to_camera[:]), np.array(ref.sample_to_camera[:]))
    assert np.array_equal(np.array(cam.camera_to_world[:]), np.array(ref.camera_to_world[:]))
    # the centre of the film maps to the view direction (-Z in camera space)
    s2c = np.array(cam.sample_to_camera[:]).reshape(4, 4)
    d = s2c @ np.array([0.5, 0.5, 0.0, 1.0])
    d = d[:3] / d[3]
    assert abs(d[0]) < 1e-6 and abs(d[1]) < 1e-6 and d[2] < 0


def test_camera_make_rejects_bad_input(ptlib):
    cam = abi.CameraDesc()
    tw = (C.c_float * 16)(*np.eye(4).reshape(-1))
    assert ptlib.pt_camera_make(40.0, 0.0, 0.01, 100.0, tw, C.byref(cam)) == 1
    assert "invalid" in abi.last_error(ptlib)


def test_entry_points_validate_without_a_device(ptlib):
    assert ptlib.pt_api_version() == 2
    # NULL arguments are rejected before any device work
    assert ptlib.pt_render(None, None, None, None) == 1
    assert ptlib.pt_trace_rays(None, None, None, 4, 0, None) == 1
    assert ptlib.pt_bvh_build(None, None, None) == 1
    assert ptlib.pt_scene_upload(None, None, None) == 1
    import torch
    if not torch.cuda.is_available():
        h = C.c_void_p()
        st = ptlib.pt_context_create(C.byref(abi.DeviceOpts(0, 0)), C.byref(h))
        assert st == 6 and not h.value  # PT_ERR_UNSUPPORTED, no context
        assert "no CUDA device" in abi.last_error(ptlib)
