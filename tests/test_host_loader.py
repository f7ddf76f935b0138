"""The C++ host layer's mitsuba-style loader (pupiloptixlab_gb300/host):
parsing, <default>/$ substitution, <ref>, transforms, BSDF defaults, named
IORs, OBJ meshes, camera set-up and error reporting.  No GPU needed."""
import ctypes as C
import math
from pathlib import Path

import numpy as np
import pytest

from pupiloptixlab_gb300 import abi, build

HERE = Path(__file__).resolve().parent / "scenes"


@pytest.fixture(scope="module")
def host():
    if not build.HOST_LIB.exists():
        build.build_library()
        build.build_host()
    from pupiloptixlab_gb300 import host_api
    host_api.load()
    return host_api


def mat4(a):
    return np.array(a[:], np.float64).reshape(4, 4)


def test_box_scene_structure(host):
    s = host.XmlScene(str(HERE / "box.xml"))
    d = s.desc()
    assert (d.width, d.height, d.max_depth) == (48, 48, 5)  # $res and $max_depth
    assert d.num_instances == 8 and d.num_spheres == 0
    assert d.num_materials == 4  # the four named BSDFs, shared through <ref>
    for i in range(d.num_materials):
        m = d.materials[i]
        assert m.type == abi.MAT_DIFFUSE and m.twosided == 1
    assert list(d.materials[1].tex[0].color0) == pytest.approx([0.65, 0.05, 0.05])
    assert list(d.materials[2].tex[0].color0) == pytest.approx([0.12, 0.45, 0.15])  # space-separated rgb
    lamp = d.instances[7]
    assert lamp.is_emitter == 1 and list(lamp.radiance) == [17.0, 12.0, 4.0]
    assert sum(d.instances[i].is_emitter for i in range(8)) == 1
    # cube and rectangle built-in meshes
    assert d.meshes[d.instances[5].shape_index].num_triangles == 12
    assert d.meshes[0].num_triangles == 2


def test_transform_order_is_translate_rotate_scale(host):
    s = host.XmlScene(str(HERE / "box.xml"))
    d = s.desc()
    m = mat4(d.instances[5].to_world)  # tall box: scale, rotate 15 about y, translate
    a = math.radians(15.0)
    R = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    want = np.eye(4)
    want[:3, :3] = R @ np.diag([0.3, 0.6, 0.3])
    want[:3, 3] = (-0.33, 0.6, -0.29)
    assert np.allclose(m, want, atol=1e-6)


def test_sensor_matrix_flip_and_camera(host, ptlib):
    from pupiloptixlab_gb300 import scenes
    s = host.XmlScene(str(HERE / "box.xml"))
    cam = s.desc().camera
    c2w = mat4(cam.camera_to_world)
    # mitsuba "-1 0 0 0 / 0 1 0 1 / 0 0 -1 3.8": X and Z columns flipped -> identity rotation
    assert np.allclose(c2w, scenes.translate(0.0, 1.0, 3.8), atol=0)
    ref = scenes.camera(40.0, 1.0, c2w)  # fov_axis y: no conversion
    assert np.array_equal(np.array(cam.sample_to_camera[:]), np.array(ref.sample_to_camera[:]))


def test_fov_axis_x_conversion_and_lookat(host, ptlib):
    from pupiloptixlab_gb300 import scenes
    s = host.XmlScene(str(HERE / "materials.xml"))
    d = s.desc()
    # fov 45 along x on a 64x40 film -> vertical fov (resource/scene.cpp:119-124)
    fov_y = 2 * math.degrees(math.atan(math.tan(math.radians(45.0) * 0.5) * 40 / 64))
    c2w = mat4(d.camera.camera_to_world)
    want = scenes.look_at_to_world((0, 3, 12), (0, 1, 0))
    assert np.allclose(c2w, want, atol=1e-6)
    ref = scenes.camera(np.float32(fov_y), 64 / 40, c2w)
    assert np.allclose(np.array(d.camera.sample_to_camera[:]), np.array(ref.sample_to_camera[:]), rtol=1e-5)


def test_materials_defaults_and_names(host):
    s = host.XmlScene(str(HERE / "materials.xml"))
    d = s.desc()
    types = [d.materials[d.instances[i].material].type for i in range(d.num_instances)]
    assert types[1:8] == [1, 2, 3, 4, 5, 6, 7]
    diel = d.materials[d.instances[2].material]
    assert diel.int_ior == pytest.approx(1.5046) and diel.ext_ior == pytest.approx(1.000277)
    rough = d.materials[d.instances[3].material]
    assert rough.int_ior == pytest.approx(1.7) and rough.ext_ior == pytest.approx(1.000277)
    assert rough.tex[2].color0[0] == pytest.approx(0.2)  # alpha
    gold = d.materials[d.instances[4].material]
    assert list(gold.tex[1].color0) == pytest.approx([0.143, 0.374, 1.442])   # eta
    assert list(gold.tex[0].color0) == [1.0, 1.0, 1.0]                        # specular_reflectance default
    plastic = d.materials[d.instances[6].material]
    assert plastic.nonlinear == 1 and plastic.int_ior == pytest.approx(1.49)
    floor = d.materials[d.instances[0].material]
    assert floor.tex[0].type == abi.TEX_CHECKERBOARD and floor.tex[0].uv_transform[0] == 8.0
    lamp = d.instances[d.num_instances - 1]
    assert lamp.shape_type == abi.SHAPE_SPHERE and lamp.is_emitter == 1
    assert d.materials[lamp.material].twosided == 1
    assert d.env.type == abi.ENV_CONST and list(d.env.radiance) == pytest.approx([0.3, 0.35, 0.4])


def test_obj_mesh(host):
    s = host.XmlScene(str(HERE / "materials.xml"))
    d = s.desc()
    obj = d.instances[7]
    m = d.meshes[obj.shape_index]
    assert m.num_triangles == 4
    assert not m.normals  # one face has no vn: geometric normals for the whole mesh
    assert m.texcoords
    idx = np.ctypeslib.as_array(m.indices, (m.num_triangles * 3,))
    assert idx.max() < m.num_vertices


@pytest.mark.parametrize("text,needle", [
    ("<scene><shape type='cube'>", "unexpected end"),
    ("<scene><bsdf type='velvet' id='a'/></scene>", "unknown bsdf"),
    ("<scene><shape type='cube'><ref id='nope'/></shape></scene>", "unknown bsdf id"),
    ("<scene><emitter type='envmap'/></scene>", "not supported"),
    ("<scene><shape type='rectangle'><bsdf type='diffuse'><texture type='bitmap' name='reflectance'/>"
     "</bsdf></shape></scene>", "not supported"),
    ("<scene><sensor type='thinlens'/></scene>", "perspective"),
    ("<notascene/>", "<scene>"),
    ("<scene><a></b></scene>", "mismatched"),
])
def test_errors_are_reported(host, text, needle):
    with pytest.raises(abi.PtError) as e:
        host.XmlScene(text, is_text=True)
    assert needle in str(e.value)


def test_loaded_scene_feeds_the_oracle(host):
    import oracle
    s = host.XmlScene(str(HERE / "box.xml"))
    o = oracle.OracleScene(s)
    nt, ns = o.num_prims()
    assert nt == 5 * 2 + 2 * 12 + 2 and ns == 0
    out = o.render(abi.RenderParams(spp=2, seed=0, accumulate=1, rng=abi.RNG_REF_LCG))
    assert np.isfinite(out["accum"]).all() and out["accum"][:, :3].mean() > 0
