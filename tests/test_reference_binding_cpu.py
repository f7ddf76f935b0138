"""The reference-side binding (pupiloptixlab_gb300/host/reference_binding/):
the WavefrontPTPass a PupilOptixLab maintainer adds and the resource::Scene ->
pt_scene_desc conversion (ToPtSceneDesc) compile against the declaration
subset of the reference's framework headers, and the conversion of
tests/scenes/box.xml built in the reference's data model (shared built-in
shapes, per-instance materials, an area emitter, the flipped sensor) gives
the descriptor the library's own XML loader gives for the same file: per
instance the same mesh arrays, flags, material and emitter, bit for bit, the
same camera, film and depth; transforms within 2 ulp (the reference
composes them in float, the loader in double).  No GPU is needed."""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from pupiloptixlab_gb300 import abi, build

ROOT = Path(__file__).resolve().parents[1]
RB = ROOT / "pupiloptixlab_gb300" / "host" / "reference_binding"
DRIVER_SRC = ROOT / "tests" / "reference_binding" / "box_scene_driver.cpp"


def compile_driver(out: Path) -> Path:
    cuda = build._cuda_root() if hasattr(build, "_cuda_root") else Path("/usr/local/cuda")
    cmd = ["g++", "-std=c++20", "-O1", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
           "-I", str(RB / "framework_subset"), "-I", str(RB), "-I", str(ROOT / "include"),
           "-I", str(Path(cuda) / "include"), str(RB / "to_pt_scene_desc.cpp"), str(RB / "wavefront_pass.cpp"),
           str(DRIVER_SRC), "-L", str(build.LIB.parent), "-lpt_gb300", "-L", str(Path(cuda) / "lib64"), "-lcudart",
           f"-Wl,-rpath,{build.LIB.parent}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.fixture(scope="module")
def driver(ptlib, tmp_path_factory):
    return compile_driver(tmp_path_factory.mktemp("rb") / "box_driver")


def u32(a):
    return [int(x) for x in np.ascontiguousarray(a, np.float32).view(np.uint32)]


def loader_dump():
    """The same expansion of the XML loader's descriptor."""
    import ctypes as C

    from pupiloptixlab_gb300 import host_api
    s = host_api.XmlScene(str(ROOT / "tests" / "scenes" / "box.xml"))
    d = s.desc()
    arr = lambda p, n, t=C.c_float: np.ctypeslib.as_array(C.cast(p, C.POINTER(t)), shape=(n,)) if (p and n) else []  # noqa
    insts = []
    for i in range(d.num_instances):
        ins = d.instances[i]
        m = d.meshes[ins.shape_index]
        mt = d.materials[ins.material]
        texs = [{"type": t.type, "color0": u32(list(t.color0)), "color1": u32(list(t.color1)),
                 "uv": u32(list(t.uv_transform)), "wh": [t.width, t.height]} for t in mt.tex]
        insts.append({"shape_type": ins.shape_type, "flags": ins.flags, "is_emitter": ins.is_emitter,
                      "radiance": u32(list(ins.radiance)), "to_world": u32(list(ins.to_world)),
                      "positions": u32(arr(m.positions, 3 * m.num_vertices)),
                      "normals": u32(arr(m.normals, 3 * m.num_vertices)),
                      "texcoords": u32(arr(m.texcoords, 2 * m.num_vertices)),
                      "indices": [int(x) for x in arr(m.indices, 3 * m.num_triangles, C.c_uint32)],
                      "material": {"type": mt.type, "twosided": mt.twosided, "nonlinear": mt.nonlinear,
                                   "ior": u32([mt.int_ior, mt.ext_ior]), "tex": texs}})
    cam = u32(list(d.camera.sample_to_camera) + list(d.camera.camera_to_world))
    return {"width": d.width, "height": d.height, "max_depth": d.max_depth, "env_type": d.env.type,
            "camera": cam, "instances": insts, "num_meshes": d.num_meshes}


def test_binding_compiles_against_the_framework_subset(driver):
    assert driver.exists()


def test_to_pt_scene_desc_equals_the_xml_loader(driver):
    r = subprocess.run([str(driver), "dump"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    got = json.loads(r.stdout)
    ref = loader_dump()
    # the reference model shares one rectangle and one cube shape between instances
    assert got["num_meshes"] == 2 and ref["num_meshes"] == len(ref["instances"])
    for k in ("width", "height", "max_depth", "env_type", "camera"):
        assert got[k] == ref[k], k
    assert len(got["instances"]) == len(ref["instances"]) == 8
    for gi, ri in zip(got["instances"], ref["instances"]):
        tw_g = np.array(gi.pop("to_world"), np.uint32).view(np.float32)
        tw_r = np.array(ri.pop("to_world"), np.uint32).view(np.float32)
        assert np.allclose(tw_g, tw_r, rtol=0, atol=2.5e-7 * np.abs(tw_r).max()), (tw_g, tw_r)
        assert gi == ri
