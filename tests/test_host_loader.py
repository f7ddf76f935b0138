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
    ("<scene><emitter type='envmap'/></scene>", "without a filename"),
    ("<scene><emitter type='spot'/></scene>", "not supported"),
    ("<scene><shape type='rectangle'><bsdf type='diffuse'><texture type='bitmap' name='reflectance'/>"
     "</bsdf></shape></scene>", "without a filename"),
    ("<scene><shape type='rectangle'><bsdf type='diffuse'><texture type='bitmap' name='reflectance'>"
     "<string name='filename' value='a.gif'/></texture></bsdf></shape></scene>", "images can be read"),
    ("<scene><sensor type='thinlens'/></scene>", "perspective"),
    ("<scene><shape type='cube'><transform name='to_world'><translate x='abc'/></transform></shape></scene>",
     "malformed number"),
    ("<scene><shape type='cube'><transform name='to_world'><rotate y='1' angle='1e999'/></transform></shape></scene>",
     "out of range"),
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


def _write_pfm(path, img, little=True):
    """img (h, w, 3) float32, top row first; PFM stores rows bottom-up."""
    h, w, _ = img.shape
    data = img[::-1].astype("<f4" if little else ">f4").tobytes()
    path.write_bytes(f"PF\n{w} {h}\n{-1.0 if little else 1.0}\n".encode() + data)


def _rgbe(rgb):
    """float RGB -> RGBE bytes (mantissa = value * 2^(136 - e))."""
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    m = rgb.max(axis=-1)
    nz = m > 1e-32
    e = np.floor(np.log2(np.where(nz, m, 1.0))).astype(np.int32) + 1
    scale = np.ldexp(1.0, 8 - e)
    out[..., :3] = np.where(nz[..., None], np.clip(np.floor(rgb * scale[..., None]), 0, 255), 0).astype(np.uint8)
    out[..., 3] = np.where(nz, e + 128, 0).astype(np.uint8)
    return out


def _write_hdr(path, img, rle=True):
    h, w, _ = img.shape
    px = _rgbe(img)
    body = bytearray()
    for y in range(h):
        if rle:
            body += bytes([2, 2, w >> 8, w & 255])
            for c in range(4):
                row = px[y, :, c]
                x = 0
                while x < w:  # runs of equal bytes (>= 3) or literals
                    run = 1
                    while x + run < w and run < 127 and row[x + run] == row[x]:
                        run += 1
                    if run >= 3:
                        body += bytes([128 + run, int(row[x])])
                        x += run
                    else:
                        n = min(128, w - x)
                        body += bytes([n]) + bytes(int(v) for v in row[x:x + n])
                        x += n
        else:
            body += px[y].tobytes()
    path.write_bytes(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {h} +X {w}\n".encode() + bytes(body))


def test_bitmap_texture_and_envmap_images(host, tmp_path):
    """bitmap textures (.pfm) and an envmap emitter (.hdr, RLE and flat) load
    into the descriptor with the reference's sampling modes."""
    rng = np.random.default_rng(3)
    tex = rng.uniform(0, 1, (6, 9, 3)).astype(np.float32)
    env = rng.uniform(0, 4, (8, 16, 3)).astype(np.float32)
    env[2, 3:9] = [5.0, 5.0, 5.0]  # a run for the RLE encoder
    _write_pfm(tmp_path / "tex.pfm", tex)
    _write_pfm(tmp_path / "texbig.pfm", tex, little=False)
    _write_hdr(tmp_path / "env.hdr", env, rle=True)
    _write_hdr(tmp_path / "envflat.hdr", env, rle=False)
    for envfile in ("env.hdr", "envflat.hdr"):
        xml = f"""<scene version="3.0.0">
          <integrator type="path"><integer name="max_depth" value="4"/></integrator>
          <sensor type="perspective"><float name="fov" value="40"/>
            <film type="hdrfilm"><integer name="width" value="32"/><integer name="height" value="24"/></film></sensor>
          <bsdf type="diffuse" id="floor"><texture type="bitmap" name="reflectance">
            <string name="filename" value="tex.pfm"/><string name="filter_type" value="bilinear"/>
            <string name="wrap_mode" value="mirror"/>
            <transform name="to_uv"><scale value="3"/></transform></texture></bsdf>
          <bsdf type="diffuse" id="wall"><texture type="bitmap" name="reflectance">
            <string name="filename" value="texbig.pfm"/><string name="filter_type" value="nearest"/></texture></bsdf>
          <shape type="rectangle"><ref id="floor"/></shape>
          <shape type="rectangle"><ref id="wall"/></shape>
          <emitter type="envmap"><string name="filename" value="{envfile}"/><float name="scale" value="2.5"/>
            <transform name="to_world"><rotate y="1" angle="90"/></transform></emitter>
        </scene>"""
        (tmp_path / "s.xml").write_text(xml)
        s = host.XmlScene(str(tmp_path / "s.xml"))
        d = s.desc()
        t0, t1 = d.materials[0].tex[0], d.materials[1].tex[0]
        assert (t0.type, t0.width, t0.height) == (abi.TEX_BITMAP, 9, 6)
        assert (t0.filter, t0.address_mode) == (abi.TEX_FILTER_LINEAR, abi.TEX_ADDRESS_MIRROR)
        assert (t1.filter, t1.address_mode) == (abi.TEX_FILTER_POINT, abi.TEX_ADDRESS_WRAP)
        assert t0.uv_transform[0] == 3.0 and t0.uv_transform[5] == 3.0
        for t in (t0, t1):
            px = np.ctypeslib.as_array(C.cast(t.pixels, C.POINTER(C.c_float)), shape=(6, 9, 4))
            assert np.array_equal(px[..., :3], tex) and np.all(px[..., 3] == 1.0)
        e = d.env
        assert (e.type, e.width, e.height, e.scale) == (abi.ENV_MAP, 16, 8, 2.5)
        px = np.ctypeslib.as_array(C.cast(e.pixels, C.POINTER(C.c_float)), shape=(8, 16, 4))
        q = _rgbe(env).astype(np.float64)
        expect = q[..., :3] * np.ldexp(1.0, q[..., 3:4].astype(np.int32) - 136)
        assert np.allclose(px[..., :3], expect, rtol=0, atol=0)
        tw = np.array(e.to_world[:]).reshape(4, 4)
        assert np.allclose(tw[:3, :3], [[0, 0, 1], [0, 1, 0], [-1, 0, 0]], atol=1e-6)


REFERENCE_SCENES = Path(__file__).resolve().parent / "golden" / "ref_scenes"


@pytest.mark.parametrize("name", ["cornellbox", "default", "denoised_scene", "material_test", "mis", "restir_test"])
def test_reference_bundled_scenes_load_and_render(host, name):
    """The reference's own sample scenes (data/static/*.xml, copied byte for
    byte into tests/golden/ref_scenes/) load through the C++ loader and the
    oracle renders them: finite, non-black pixels."""
    path = REFERENCE_SCENES / f"{name}.xml"
    import hashlib
    sums = dict(reversed(l.split("  ")) for l in (REFERENCE_SCENES / "SHA256SUMS").read_text().split("\n") if l)
    assert hashlib.sha256(path.read_bytes()).hexdigest() == sums[f"{name}.xml"]
    import oracle
    s = host.XmlScene(str(path))
    d = s.desc()
    assert d.num_instances > 0 and d.num_materials > 0 and d.width > 0 and d.height > 0
    o = oracle.OracleScene(s, bvh=True)
    px = np.arange(0, d.width * d.height, max(1, d.width * d.height // 256), dtype=np.uint32)
    p = abi.RenderParams(spp=2, max_depth=0, seed=0, sample_cnt=0, accumulate=1, rng=abi.RNG_REF_LCG)
    img = o.render(p, pixels=px)["accum"][px, :3]
    assert np.isfinite(img).all() and img.max() > 0.0


def _parse_exr_header(data: bytes):
    """Independent reading of an OpenEXR header: magic, version, attributes."""
    import struct
    assert struct.unpack_from("<I", data, 0)[0] == 20000630
    version = struct.unpack_from("<I", data, 4)[0]
    p, attrs = 8, {}
    while data[p] != 0:
        name_end = data.index(0, p)
        name = data[p:name_end].decode()
        type_end = data.index(0, name_end + 1)
        typ = data[name_end + 1:type_end].decode()
        size = struct.unpack_from("<I", data, type_end + 1)[0]
        attrs[name] = (typ, data[type_end + 5:type_end + 5 + size])
        p = type_end + 5 + size
    return version, attrs, p + 1


def test_exr_writer_and_reader(host, tmp_path):
    """pupil_write_exr writes uncompressed scanline OpenEXR (checked against
    the file-format layout by an independent parser), and the loader reads it
    back as an env map bit for bit."""
    import struct
    rng = np.random.default_rng(9)
    img = rng.uniform(0, 8, (5, 7, 4)).astype(np.float32)
    img[..., 3] = 1.0
    path = tmp_path / "env.exr"
    host.write_exr(str(path), img)
    data = path.read_bytes()
    version, attrs, table = _parse_exr_header(data)
    assert version == 2
    assert attrs["compression"] == ("compression", b"\x00")
    assert struct.unpack("<4i", attrs["dataWindow"][1]) == (0, 0, 6, 4)
    chans = attrs["channels"][1].split(b"\x00")
    assert [c for c in chans if c in (b"A", b"B", b"G", b"R")] == [b"A", b"B", b"G", b"R"]
    first = struct.unpack_from("<Q", data, table)[0]
    y, nbytes = struct.unpack_from("<ii", data, first)
    assert y == 0 and nbytes == 4 * 4 * 7
    r0 = np.frombuffer(data, "<f4", 7, first + 8 + 3 * 4 * 7)  # R is the last channel of the row
    assert np.array_equal(r0, img[0, :, 0])
    xml = f"""<scene version="3.0.0"><integrator type="path"><integer name="max_depth" value="3"/></integrator>
      <sensor type="perspective"><film type="hdrfilm"><integer name="width" value="8"/><integer name="height" value="8"/>
      </film></sensor><shape type="rectangle"><bsdf type="diffuse"/></shape>
      <emitter type="envmap"><string name="filename" value="{path}"/></emitter></scene>"""
    s = host.XmlScene(xml, is_text=True)
    e = s.desc().env
    assert (e.type, e.width, e.height) == (abi.ENV_MAP, 7, 5)
    px = np.ctypeslib.as_array(C.cast(e.pixels, C.POINTER(C.c_float)), shape=(5, 7, 4))
    assert np.array_equal(px, img)


def _write_hair(path, strands, thickness=None, default_segments=None, default_thickness=0.01):
    """Cem Yuksel's HAIR layout: 128-byte header, then (by flag bit) the
    per-strand segment counts (u16), points (3 f32), thickness (f32)."""
    import struct
    seg = np.array([len(s) - 1 for s in strands], np.uint16)
    pts = np.concatenate(strands).astype("<f4")
    flags = 2 | (0 if default_segments is not None else 1) | (4 if thickness is not None else 0)
    head = struct.pack("<4sIIIIff3f", b"HAIR", len(strands), pts.shape[0], flags,
                       default_segments or 0, default_thickness, 1.0, 0.5, 0.5, 0.5)
    head += b"test".ljust(88, b"\0")
    body = b"" if default_segments is not None else seg.astype("<u2").tobytes()
    body += pts.tobytes()
    if thickness is not None:
        body += np.asarray(thickness, "<f4").tobytes()
    path.write_bytes(head + body)


def test_hair_shape(host, tmp_path):
    """<shape type="hair"> (resource/shape.cpp:153-181, 369-420): the HAIR file's
    points become curve control points, the segments start at every point of a
    strand up to its count minus the spline degree, radius overrides the file
    thickness, tapered strands fall linearly to zero; the descriptor renders
    through the oracle."""
    import oracle
    rng = np.random.default_rng(4)
    strands = [np.cumsum(rng.normal(size=(n, 3)) * 0.2, 0) + [0, 1, 0] for n in (6, 9, 5)]
    npts = sum(len(s) for s in strands)
    thick = rng.uniform(0.01, 0.03, npts)
    _write_hair(tmp_path / "a.hair", strands, thick)
    _write_hair(tmp_path / "b.hair", [s[:5] for s in strands], None, default_segments=4, default_thickness=0.02)
    modes = {"linear": (abi.CURVE_LINEAR, 1), "quadratic": (abi.CURVE_QUADRATIC_BSPLINE, 2),
             "cubic": (abi.CURVE_CUBIC_BSPLINE, 3), "catrom": (abi.CURVE_CATMULL_ROM, 3)}
    for mode, (ctype, deg) in modes.items():
        xml = f"""<scene version="3.0.0">
          <sensor type="perspective"><float name="fov" value="40"/>
            <transform name="to_world"><lookat origin="0, 1, 6" target="0, 1, 0" up="0, 1, 0"/></transform>
            <film type="hdrfilm"><integer name="width" value="24"/><integer name="height" value="16"/></film></sensor>
          <shape type="hair"><string name="filename" value="a.hair"/><string name="spline_mode" value="{mode}"/>
            <bsdf type="roughconductor"/></shape>
          <shape type="hair"><string name="filename" value="a.hair"/><string name="spline_mode" value="{mode}"/>
            <float name="radius" value="0.05"/><boolean name="tapered" value="true"/>
            <transform name="to_world"><translate x="1"/></transform></shape>
          <shape type="hair"><string name="filename" value="b.hair"/><float name="radius" value="0.04"/></shape>
          <emitter type="constant"><rgb name="radiance" value="0.5"/></emitter>
        </scene>"""
        (tmp_path / "h.xml").write_text(xml)
        s = host.XmlScene(str(tmp_path / "h.xml"))
        d = s.desc()
        assert d.num_curves == 3
        c0, c1, c2 = d.curves[0], d.curves[1], d.curves[2]
        assert (c0.type, c1.type, c2.type) == (ctype, ctype, abi.CURVE_CUBIC_BSPLINE)
        assert c0.num_points == npts
        pos = np.ctypeslib.as_array(c0.positions, (npts * 3,)).reshape(-1, 3)
        assert np.array_equal(pos, np.concatenate(strands).astype(np.float32))
        r0 = np.ctypeslib.as_array(c0.radii, (npts,))
        assert np.array_equal(r0, thick.astype(np.float32))
        segs = np.ctypeslib.as_array(c0.segments, (c0.num_segments,))
        starts = np.cumsum([0] + [len(s) for s in strands])
        expect = np.concatenate([np.arange(a, b - deg) for a, b in zip(starts[:-1], starts[1:])])
        assert np.array_equal(segs, expect)
        r1 = np.ctypeslib.as_array(c1.radii, (npts,))
        taper = np.concatenate([0.05 * (len(s) - 1 - np.arange(len(s))) / (len(s) - 1) for s in strands])
        assert np.allclose(r1, taper, rtol=1e-6, atol=0)
        r2 = np.ctypeslib.as_array(c2.radii, (15,))
        assert np.all(r2 == np.float32(0.04)) and c2.num_segments == 3 * (5 - 3)
        insts = [d.instances[i] for i in range(d.num_instances)]
        assert [i.shape_type for i in insts] == [abi.SHAPE_CURVES] * 3
        assert insts[1].to_world[3] == 1.0
        o = oracle.OracleScene(s)
        assert o.num_curves()[0] == c0.num_segments + c1.num_segments + c2.num_segments
        out = o.render(abi.RenderParams(spp=1, seed=0, accumulate=1, rng=abi.RNG_PCG32))
        assert np.isfinite(out["accum"]).all()
    (tmp_path / "bad.hair").write_bytes(b"HAIX" + bytes(124))
    (tmp_path / "h2.xml").write_text("<scene><shape type='hair'><string name='filename' value='bad.hair'/></shape></scene>")
    with pytest.raises(abi.PtError) as e:
        host.XmlScene(str(tmp_path / "h2.xml"))
    assert "not a HAIR file" in str(e.value)


def _hair_header(strands, points, flags, default_segments=0):
    import struct
    return struct.pack("<4sIIIIff3f", b"HAIR", strands, points, flags, default_segments, 0.01, 1.0, 0.5, 0.5,
                       0.5) + bytes(88)


@pytest.mark.parametrize("body, needle", [
    (b"HAIR" + bytes(60), "truncated HAIR header"),
    (_hair_header(3, 12, 3) + bytes(4), "truncated segment array"),
    (_hair_header(2, 8, 1) + np.array([3, 3], "<u2").tobytes(), "has no points"),
    (_hair_header(2, 6, 3) + np.array([3, 3], "<u2").tobytes() + bytes(72), "need more points"),
    (_hair_header(2, 8, 3) + np.array([3, 3], "<u2").tobytes() + bytes(40), "truncated point array"),
    (_hair_header(1, 4, 6, default_segments=3) + bytes(48) + bytes(8), "truncated thickness array"),
])
def test_malformed_hair_files_are_reported(host, tmp_path, body, needle):
    """A HAIR file cut short anywhere, or with strands that need more points
    than it holds, is refused with a message naming the part that is wrong."""
    (tmp_path / "x.hair").write_bytes(body)
    (tmp_path / "x.xml").write_text("<scene><shape type='hair'><string name='filename' value='x.hair'/></shape></scene>")
    with pytest.raises(abi.PtError) as e:
        host.XmlScene(str(tmp_path / "x.xml"))
    assert needle in str(e.value)


def test_hair_counts_beyond_the_file_are_refused_before_allocation(host, tmp_path):
    """A HAIR header announcing billions of strands or points in a file of a
    few bytes is refused from the file size, without allocating for it."""
    for strands, points, flags in ((0xffffffff, 0xffffffff, 3), (0xfffffff0, 4, 2), (4, 0x40000000, 6)):
        (tmp_path / "x.hair").write_bytes(_hair_header(strands, points, flags, default_segments=3) + bytes(64))
        (tmp_path / "x.xml").write_text("<scene><shape type='hair'><string name='filename' value='x.hair'/></shape></scene>")
        with pytest.raises(abi.PtError):
            host.XmlScene(str(tmp_path / "x.xml"))


def test_point_emitters_are_dropped_as_the_reference_does(host):
    """<emitter type="point"> is parsed by the reference (resource/scene.cpp:194-202)
    but never enters its emitter tables (world/emitter.cpp:314-315), so it
    lights nothing: the scene loads and equals the same scene without it."""
    base = """<scene version="3.0.0"><sensor type="perspective"><film type="hdrfilm">
      <integer name="width" value="8"/><integer name="height" value="8"/></film></sensor>
      <shape type="rectangle"><bsdf type="diffuse"/></shape>{extra}
      <emitter type="constant"><rgb name="radiance" value="0.5"/></emitter></scene>"""
    point = """<emitter type="point"><point name="position" x="0" y="2" z="0"/>
      <rgb name="intensity" value="10"/></emitter>"""
    a = host.XmlScene(base.format(extra=point), is_text=True).desc()
    b = host.XmlScene(base.format(extra=""), is_text=True).desc()
    assert (a.num_instances, a.num_materials, a.num_meshes, a.env.type) == \
           (b.num_instances, b.num_materials, b.num_meshes, b.env.type)
    assert [a.instances[i].is_emitter for i in range(a.num_instances)] == \
           [b.instances[i].is_emitter for i in range(b.num_instances)]


@pytest.mark.parametrize("args", [[], ["a.xml"], ["a.xml", "o.pfm", "x"], ["a.xml", "o.pfm", "0"],
                                  ["a.xml", "o.pfm", "-3"], ["a.xml", "o.pfm", "4", "xorshift"],
                                  ["a.xml", "o.pfm", "4", "pcg32", "extra"]])
def test_cli_rejects_bad_arguments(host, args):
    """pupil_pt checks its arguments before touching the device: a missing
    output, a frame count that is not a positive integer or an unknown random
    stream prints the usage line and exits with status 2."""
    import subprocess
    r = subprocess.run([str(build.HOST_CLI), *args], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage:" in r.stderr


def test_cli_reports_an_unloadable_scene(host, tmp_path):
    """Well-formed arguments naming a missing scene end with status 1 and a
    message (on a machine without a GPU the device set-up reports first)."""
    import subprocess
    r = subprocess.run([str(build.HOST_CLI), str(tmp_path / "missing.xml"), str(tmp_path / "o.pfm"), "2", "lcg"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and r.stderr.strip()
    assert not (tmp_path / "o.pfm").exists()


def test_malformed_obj_face_is_reported(host, tmp_path):
    """A face token that is not an index ends the load with the file, the line
    and the token in the message, not with an exception through the C API."""
    (tmp_path / "m.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 x3\n")
    (tmp_path / "m.xml").write_text("<scene><shape type='obj'><string name='filename' value='m.obj'/></shape></scene>")
    with pytest.raises(abi.PtError) as e:
        host.XmlScene(str(tmp_path / "m.xml"))
    assert "m.obj:4: malformed face index 'x3'" in str(e.value)


def test_pass_enable_switch_and_buffer_desc(host, tmp_path):
    """Pupil::Pass keeps the reference's enable switch (system/pass.h:37-39,
    pass.cpp:6-13): Run() skips OnRun while the pass is disabled; Toggle and
    SetEnablility flip it.  BufferManager takes the reference's BufferDesc
    (buffer.h:25-31) and lists buffer names in allocation order; without a
    device an allocation fails cleanly and lists nothing.  System::Run runs
    no pass while render_flag is clear (system.h:26).  Compiled against the
    host headers, no GPU needed."""
    import subprocess
    src = tmp_path / "pass_switch.cpp"
    src.write_text(r'''
#include <cstdio>
#include "pass.h"
struct Count : Pupil::Pass {
    int runs = 0;
    Count() noexcept : Pupil::Pass("count") {}
    void OnRun() noexcept override { runs++; }
};
int main() {
    Count p;
    p.Run();
    p.SetEnablility(false);
    p.Run();
    const bool off = !p.IsEnabled();
    p.Toggle();
    p.Run();
    Pupil::System sys;
    Count q;
    sys.AddPass(&q);
    sys.render_flag = false;
    sys.Run(3);
    const int paused_runs = q.runs;
    sys.render_flag = true;
    sys.Run(3);
    Pupil::BufferManager bm;
    Pupil::BufferManager::BufferDesc none{};
    Pupil::BufferManager::BufferDesc d{"pt accum buffer", 0, 4, 2, 16};
    auto *b = bm.AllocBuffer(d);  // fails cleanly where no device is present
    const bool consistent = (b != nullptr) == (bm.GetBufferNameList().size() == 1) &&
                            (!b || (b->bytes == 128 && bm.GetBufferNameList()[0] == "pt accum buffer"));
    std::printf("%d %d %d %d %d %d %d %d\n", p.runs, off ? 1 : 0, p.IsEnabled() ? 1 : 0, bm.AllocBuffer(none) == nullptr,
                consistent ? 1 : 0, Pupil::BufferManager::DEFAULT_FINAL_RESULT_BUFFER_NAME == "final result",
                paused_runs, q.runs);
    return 0;
}
''')
    exe = tmp_path / "pass_switch"
    cuda_inc = build._cuda_include()
    subprocess.run(["g++", "-std=c++17", "-I", str(build.ROOT / "include"), "-I", str(build.HOST), "-I", cuda_inc,
                    str(src), "-o", str(exe), "-L", str(build.BUILD), "-lpupil_host", "-lpt_gb300",
                    "-L", build._cuda_lib_dir(), "-lcudart", f"-Wl,-rpath,{build.BUILD}",
                    f"-Wl,-rpath,{build._cuda_lib_dir()}"], check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True, timeout=60).stdout.split()
    assert out == ["2", "1", "1", "1", "1", "1", "0", "3"]


def test_textured_area_emitter_radiance(host):
    """<emitter type="area"> with a checkerboard radiance texture (as
    resource/emitter.h:17-19 allows) becomes a textured emitter instance."""
    text = """<scene>
      <sensor type='perspective'><film type='hdrfilm'><integer name='width' value='8'/>
        <integer name='height' value='8'/></film></sensor>
      <shape type='rectangle'>
        <emitter type='area'>
          <texture name='radiance' type='checkerboard'>
            <rgb name='color0' value='5, 4, 3'/><rgb name='color1' value='1, 2, 3'/>
            <transform name='to_uv'><scale x='4' y='2'/></transform>
          </texture>
        </emitter>
      </shape>
      <shape type='sphere'><emitter type='area'><rgb name='radiance' value='2, 3, 4'/></emitter></shape>
    </scene>"""
    s = host.XmlScene(text, is_text=True)
    d = s.desc()
    a, b = d.instances[0], d.instances[1]
    assert a.is_emitter and a.radiance_textured and a.radiance_tex.type == abi.TEX_CHECKERBOARD
    assert list(a.radiance_tex.color0) == [5.0, 4.0, 3.0] and list(a.radiance_tex.color1) == [1.0, 2.0, 3.0]
    assert a.radiance_tex.uv_transform[0] == 4.0 and a.radiance_tex.uv_transform[5] == 2.0
    assert b.is_emitter and not b.radiance_textured and list(b.radiance) == [2.0, 3.0, 4.0]



# ---- PNG and compressed OpenEXR, written here by independent encoders ------

def _png_bytes(samples, ctype, depth, interlace=False, palette=None, trns=None):
    """A PNG file per the specification: samples (h, w, channels) integers,
    rows filtered with filter types cycling through 0..4, Adam7 passes when
    interlaced, one zlib stream split over two IDAT chunks."""
    import struct
    import zlib
    h, w = samples.shape[:2]
    ch = samples.shape[2]

    def pack_row(row):
        if depth >= 8:
            return row.astype(">u2" if depth == 16 else "u1").tobytes()
        bits = "".join(format(int(v), f"0{depth}b") for v in row.reshape(-1))
        bits += "0" * (-len(bits) % 8)
        return bytes(int(bits[i:i + 8], 2) for i in range(0, len(bits), 8))

    bpp = max(1, ch * depth // 8)

    def filt(lines):
        out, prev = b"", bytes(len(lines[0])) if lines else b""
        for k, cur in enumerate(lines):
            f = k % 5
            enc = bytearray()
            for i, x in enumerate(cur):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                if f == 0:
                    pred = 0
                elif f == 1:
                    pred = a
                elif f == 2:
                    pred = b
                elif f == 3:
                    pred = (a + b) >> 1
                else:
                    pp = a + b - c
                    pa, pb, pc = abs(pp - a), abs(pp - b), abs(pp - c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                enc.append((x - pred) & 0xFF)
            out += bytes([f]) + bytes(enc)
            prev = cur
        return out

    passes = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)] \
        if interlace else [(0, 0, 1, 1)]
    raw = b""
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        raw += filt([pack_row(r) for r in sub])
    comp = zlib.compress(raw, 9)

    def chunk(t, body):
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xFFFFFFFF)

    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        out += chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        out += chunk(b"tRNS", bytes(np.asarray(trns, np.uint8)))
    out += chunk(b"tEXt", b"Comment\x00written by the test")
    half = len(comp) // 2
    return out + chunk(b"IDAT", comp[:half]) + chunk(b"IDAT", comp[half:]) + chunk(b"IEND", b"")


def _load_env(host, path):
    xml = f"""<scene version="3.0.0"><sensor type="perspective"><film type="hdrfilm"><integer name="width" value="8"/>
      <integer name="height" value="8"/></film></sensor><shape type="rectangle"><bsdf type="diffuse"/></shape>
      <emitter type="envmap"><string name="filename" value="{path}"/></emitter></scene>"""
    s = host.XmlScene(xml, is_text=True)
    e = s.desc().env
    return np.ctypeslib.as_array(C.cast(e.pixels, C.POINTER(C.c_float)), shape=(e.height, e.width, 4)).copy()


def _expect_rgba(img8, c):
    """The reference's 8-bit conversion (framework/util/texture.cpp:106-118) of
    samples with c channels: (v / 255)^2.2 of three consecutive bytes, alpha
    byte / 255 for 4 channels; bytes past the end read as 0."""
    flat = img8.reshape(-1).astype(np.float32)
    n = flat.shape[0] // c
    pad = np.concatenate([flat, np.zeros(4, np.float32)])
    out = np.empty((n, 4), np.float32)
    for k in range(3):
        out[:, k] = np.power(pad[np.arange(n) * c + k] / np.float32(255.0), np.float32(2.2))
    out[:, 3] = pad[np.arange(n) * c + 3] / np.float32(255.0) if c == 4 else 1.0
    return out


@pytest.mark.parametrize("ctype,depth,interlace", [(2, 8, False), (6, 8, True), (6, 16, False), (2, 16, True),
                                                   (0, 8, False), (4, 8, True), (0, 4, True), (0, 1, False),
                                                   (3, 8, False), (3, 2, True)])
def test_png_reader(host, tmp_path, ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 100 + depth + interlace)
    h, w = 11, 13
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    palette = trns = None
    if ctype == 3:
        n = 1 << depth
        palette = rng.integers(0, 256, (n, 3))
        trns = rng.integers(0, 256, n // 2) if depth == 8 else None
        samples = rng.integers(0, n, (h, w, 1))
    else:
        samples = rng.integers(0, 1 << depth, (h, w, chans))
    path = tmp_path / "t.png"
    path.write_bytes(_png_bytes(samples, ctype, depth, interlace, palette, trns))
    got = _load_env(host, path)
    # what an 8-bit load delivers
    if ctype == 3:
        rgb = np.asarray(palette, np.uint8)[samples[..., 0]]
        if trns is not None:
            a = np.array([trns[i] if i < len(trns) else 255 for i in samples.reshape(-1)], np.uint8).reshape(h, w, 1)
            img8, c = np.concatenate([rgb, a], 2), 4
        else:
            img8, c = rgb, 3
    elif depth == 16:
        img8, c = (samples >> 8).astype(np.uint8), chans
    elif depth < 8:
        img8, c = (samples * (255 // ((1 << depth) - 1))).astype(np.uint8), chans
    else:
        img8, c = samples.astype(np.uint8), chans
    expect = _expect_rgba(img8, c).reshape(h, w, 4)
    assert np.allclose(got, expect, rtol=2e-7, atol=0), np.abs(got - expect).max()
    if c == 4:
        assert np.array_equal(got[..., 3], expect[..., 3])


@pytest.mark.parametrize("kind", ["exr_window", "hdr", "pfm", "png"])
def test_image_sizes_beyond_the_limit_are_refused(host, tmp_path, kind):
    """Headers asking for more than 65,536 pixels on a side (or 2^28 pixels)
    are refused before anything is allocated for them."""
    import struct
    import zlib
    if kind == "exr_window":
        good = _exr_bytes(np.zeros((2, 3, 4), np.float32), 1, True)
        i = good.index(b"dataWindow\0box2i\0") + len(b"dataWindow\0box2i\0") + 4
        data = good[:i] + struct.pack("<iiii", -2000000000, 0, 2000000000, 1) + good[i + 16:]
        name = "t.exr"
    elif kind == "hdr":
        data, name = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 100000 +X 100000\n" + bytes(64), "t.hdr"
    elif kind == "pfm":
        data, name = b"PF\n300000 300000\n-1.0\n" + bytes(64), "t.pfm"
    else:
        ihdr = struct.pack(">IIBBBBB", 1 << 20, 1 << 20, 8, 2, 0, 0, 0)
        chunk = lambda t, b: struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xffffffff)
        data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(b"\0" * 16)) + chunk(b"IEND", b"")
        name = "t.png"
    path = tmp_path / name
    path.write_bytes(data)
    with pytest.raises(abi.PtError) as e:
        _load_env(host, path)
    assert "out of range" in str(e.value)


def _exr_bytes(img, compression, half):
    """A scanline OpenEXR file with channels A B G R (HALF or FLOAT), RLE
    (1), ZIPS (2) or ZIP (3) compressed blocks per the file-format
    description: bytes split into even / odd halves, delta-predicted (+128),
    then run-length or zlib coded."""
    import struct
    import zlib
    h, w = img.shape[:2]
    lpb = 16 if compression == 3 else 1
    typ = 1 if half else 2

    def attr(name, t, value):
        return name.encode() + b"\0" + t.encode() + b"\0" + struct.pack("<i", len(value)) + value

    chl = b"".join(c + b"\0" + struct.pack("<iB3xii", typ, 0, 1, 1) for c in (b"A", b"B", b"G", b"R")) + b"\0"
    head = struct.pack("<ii", 20000630, 2)
    head += attr("channels", "chlist", chl) + attr("compression", "compression", bytes([compression]))
    head += attr("dataWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    head += attr("displayWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    head += attr("lineOrder", "lineOrder", b"\0") + attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    head += attr("screenWindowCenter", "v2f", struct.pack("<ff", 0, 0)) + attr("screenWindowWidth", "float",
                                                                                struct.pack("<f", 1.0)) + b"\0"
    dt = "<f2" if half else "<f4"
    blocks = []
    for y0 in range(0, h, lpb):
        raw = b"".join(img[y, :, ci].astype(dt).tobytes() for y in range(y0, min(h, y0 + lpb)) for ci in (3, 2, 1, 0))
        t = bytearray(raw[0::2] + raw[1::2])
        for i in range(len(t) - 1, 0, -1):
            t[i] = (t[i] - t[i - 1] + 128) & 0xFF
        if compression == 1:
            enc, i = bytearray(), 0
            while i < len(t):
                run = 1
                while i + run < len(t) and t[i + run] == t[i] and run < 128:
                    run += 1
                if run >= 3:
                    enc += bytes([run - 1, t[i]])
                    i += run
                else:
                    j = i
                    while j < len(t) and j - i < 127 and not (j + 2 < len(t) and t[j] == t[j + 1] == t[j + 2]):
                        j += 1
                    enc += bytes([(256 - (j - i)) & 0xFF]) + bytes(t[i:j])
                    i = j
            data = bytes(enc)
        else:
            data = zlib.compress(bytes(t), 6)
        if len(data) >= len(raw):
            data = raw
        blocks.append(struct.pack("<ii", y0, len(data)) + data)
    table_at = len(head)
    offsets, pos = [], table_at + 8 * len(blocks)
    for b in blocks:
        offsets.append(pos)
        pos += len(b)
    return head + b"".join(struct.pack("<Q", o) for o in offsets) + b"".join(blocks)


@pytest.mark.parametrize("compression,half", [(1, True), (2, False), (3, True), (3, False)])
def test_compressed_exr_reader(host, tmp_path, compression, half):
    rng = np.random.default_rng(compression * 10 + half)
    h, w = 37, 21
    img = rng.uniform(0, 4, (h, w, 4)).astype(np.float32)
    img[5:20, 3:9, :3] = 1.5  # runs for the run-length coder
    img[..., 3] = rng.uniform(0.5, 1.0, (h, w)).astype(np.float32)
    if half:
        img = img.astype(np.float16).astype(np.float32)
    path = tmp_path / "t.exr"
    path.write_bytes(_exr_bytes(img, compression, half))
    got = _load_env(host, path)
    assert np.array_equal(got, img)


def test_compression_the_reader_does_not_take_is_reported(host, tmp_path):
    data = bytearray(_exr_bytes(np.ones((4, 4, 4), np.float32), 3, False))
    i = data.index(b"compression\0compression\0") + len(b"compression\0compression\0") + 4
    data[i] = 4  # PIZ
    path = tmp_path / "piz.exr"
    path.write_bytes(bytes(data))
    with pytest.raises(abi.PtError) as e:
        _load_env(host, path)
    assert "PIZ" in str(e.value)


# ---- JPEG: an independent baseline encoder (ITU-T T.81) and the expected decode

def _jpeg_bytes(rgb, subsample, quality_q, restart=0, grey=False):
    """A baseline JPEG of an (h, w, 3) uint8 image (or (h, w) grey): JFIF
    YCbCr, 4:2:0 (subsample) or 4:4:4, one quantisation table value, forward
    DCT from its definition, every Huffman code 8 bits long (a valid table for
    up to 255 symbols), byte stuffing, optional restart markers.  Returns the
    file and the quantised coefficients per component."""
    import struct
    h, w = rgb.shape[:2]
    x = rgb.astype(np.float64)
    if grey:
        planes = [x]
        samp = [(1, 1)]
    else:
        r, g, b = x[..., 0], x[..., 1], x[..., 2]
        Y = 0.299 * r + 0.587 * g + 0.114 * b
        Cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
        Cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
        planes = [Y, Cb, Cr]
        samp = [(2, 2), (1, 1), (1, 1)] if subsample else [(1, 1), (1, 1), (1, 1)]
    hmax = max(s[0] for s in samp)
    vmax = max(s[1] for s in samp)
    if grey:
        hmax = vmax = 1
    mw, mh = 8 * hmax, 8 * vmax
    W, H = -(-w // mw) * mw, -(-h // mh) * mh
    cu = np.array([np.sqrt(0.5)] + [1.0] * 7)
    cosm = np.array([[cu[u] * np.cos((2 * xx + 1) * u * np.pi / 16) for u in range(8)] for xx in range(8)])
    zz = [0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14,
          21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60,
          61, 54, 47, 55, 62, 63]
    comps = []
    for pl, (sh, sv) in zip(planes, samp):
        padded = np.pad(pl, ((0, H - h), (0, W - w)), mode="edge")
        fx, fy = hmax // sh, vmax // sv
        sub = padded.reshape(H // fy, fy, W // fx, fx).mean(axis=(1, 3)) if (fx > 1 or fy > 1) else padded
        bh, bw = sub.shape[0] // 8, sub.shape[1] // 8
        q = np.zeros((bh, bw, 64), np.int64)
        for by in range(bh):
            for bx in range(bw):
                blk = sub[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] - 128.0
                S = 0.25 * cosm.T @ blk @ cosm  # S[v, u]
                nat = S.reshape(-1)
                q[by, bx] = np.round(np.array([nat[zz[k]] for k in range(64)]) / quality_q).astype(np.int64)
        comps.append(q)
    # entropy coding
    def cat(v):
        return 0 if v == 0 else int(abs(v)).bit_length()

    def bits_of(v, s):
        return v if v >= 0 else v + (1 << s) - 1

    mcux, mcuy = W // mw, H // mh
    units = []  # (comp index, block) in coding order
    for my in range(mcuy):
        for mx in range(mcux):
            for ci, (sh, sv) in enumerate(samp):
                ch, cv = (1, 1) if grey else (sh, sv)
                for by in range(cv):
                    for bx in range(ch):
                        units.append((my * mcux + mx, ci, comps[ci][my * cv + by, mx * ch + bx]))
    dc_syms = [set(), set()]
    ac_syms = [set(), set()]
    pred = [0] * len(comps)
    seq = []
    last_mcu = -1
    for mcu, ci, blk in units:
        if restart and mcu != last_mcu and mcu > 0 and mcu % restart == 0:
            pred = [0] * len(comps)
            seq.append(("RST", mcu // restart - 1))
        last_mcu = mcu
        t = 0 if ci == 0 else 1
        diff = int(blk[0]) - pred[ci]
        pred[ci] = int(blk[0])
        s = cat(diff)
        dc_syms[t].add(s)
        seq.append(("DC", t, s, bits_of(diff, s)))
        run = 0
        last_nz = max([k for k in range(1, 64) if blk[k] != 0], default=0)
        for k in range(1, last_nz + 1):
            v = int(blk[k])
            if v == 0:
                run += 1
                continue
            while run > 15:
                ac_syms[t].add(0xF0)
                seq.append(("AC", t, 0xF0, 0, 0))
                run -= 16
            s = cat(v)
            ac_syms[t].add((run << 4) | s)
            seq.append(("AC", t, (run << 4) | s, s, bits_of(v, s)))
            run = 0
        if last_nz < 63:
            ac_syms[t].add(0x00)
            seq.append(("AC", t, 0x00, 0, 0))
    tables = {}
    for cls, syms in ((0, dc_syms), (1, ac_syms)):
        for t in (0, 1):
            ss = sorted(syms[t]) or [0]
            tables[(cls, t)] = {s: i for i, s in enumerate(ss)}
    out, acc, nacc = bytearray(), 0, 0

    def put(v, n):
        nonlocal acc, nacc
        for i in range(n - 1, -1, -1):
            acc = (acc << 1) | ((v >> i) & 1)
            nacc += 1
            if nacc == 8:
                out.append(acc)
                if acc == 0xFF:
                    out.append(0)
                acc, nacc = 0, 0

    def flush():
        nonlocal acc, nacc
        if nacc:
            put((1 << (8 - nacc)) - 1, 8 - nacc)

    for e in seq:
        if e[0] == "RST":
            flush()
            out += bytes([0xFF, 0xD0 + (e[1] % 8)])
        elif e[0] == "DC":
            put(tables[(0, e[1])][e[2]], 8)
            put(e[3], e[2])
        else:
            put(tables[(1, e[1])][e[2]], 8)
            put(e[4], e[3])
    flush()
    ncomp = len(comps)
    f = bytearray(b"\xFF\xD8")
    f += b"\xFF\xE0" + struct.pack(">H", 16) + b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00"
    f += b"\xFF\xDB" + struct.pack(">H", 67) + bytes([0]) + bytes([quality_q] * 64)
    f += b"\xFF\xC0" + struct.pack(">HBHHB", 8 + 3 * ncomp, 8, h, w, ncomp)
    for ci, (sh, sv) in enumerate(samp):
        f += bytes([ci + 1, (sh << 4) | sv, 0])
    for (cls, t), mp in tables.items():
        syms = sorted(mp, key=lambda s: mp[s])
        counts = [0] * 16
        counts[7] = len(syms)
        f += b"\xFF\xC4" + struct.pack(">H", 2 + 17 + len(syms)) + bytes([(cls << 4) | t] + counts + syms)
    if restart:
        f += b"\xFF\xDD" + struct.pack(">HH", 4, restart)
    f += b"\xFF\xDA" + struct.pack(">HB", 6 + 2 * ncomp, ncomp)
    for ci in range(ncomp):
        t = 0 if ci == 0 else 1
        f += bytes([ci + 1, (t << 4) | t])
    f += bytes([0, 63, 0]) + out + b"\xFF\xD9"
    return bytes(f), comps, samp, (mcux, mcuy, hmax, vmax)


def _jpeg_expected(comps, samp, layout, h, w, q, grey):
    """The decoder's arithmetic restated: dequantise, IDCT from the definition,
    round half away from zero, clamp; replicate chroma; JFIF YCbCr -> RGB."""
    mcux, mcuy, hmax, vmax = layout
    cu = np.array([np.sqrt(0.5)] + [1.0] * 7)
    cosm = np.array([[cu[u] * np.cos((2 * xx + 1) * u * np.pi / 16) for u in range(8)] for xx in range(8)])
    zz = [0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14,
          21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60,
          61, 54, 47, 55, 62, 63]
    rnd = lambda v: np.sign(v) * np.floor(np.abs(v) + 0.5)  # noqa: E731
    planes = []
    for blocks in comps:
        bh, bw = blocks.shape[:2]
        pl = np.zeros((bh * 8, bw * 8))
        for by in range(bh):
            for bx in range(bw):
                nat = np.zeros(64)
                for k in range(64):
                    nat[zz[k]] = blocks[by, bx, k] * q
                S = nat.reshape(8, 8)
                pl[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] = np.clip(rnd(cosm @ S @ cosm.T / 4.0 + 128.0), 0, 255)
        planes.append(pl)
    if grey:
        return planes[0][:h, :w].astype(np.uint8)[..., None]
    ys, xs = np.arange(h), np.arange(w)
    up = [p[(ys * s[1] // vmax)[:, None], (xs * s[0] // hmax)[None, :]] for p, s in zip(planes, samp)]
    Y, cb, cr = up[0], up[1] - 128.0, up[2] - 128.0
    rgb = np.stack([Y + 1.402 * cr, Y - 0.344136 * cb - 0.714136 * cr, Y + 1.772 * cb], -1)
    return np.clip(rnd(rgb), 0, 255).astype(np.uint8)


@pytest.mark.parametrize("subsample,restart,grey,size", [(True, 0, False, (37, 29)), (False, 3, False, (16, 24)),
                                                          (True, 2, False, (40, 41)), (False, 0, True, (21, 18))])
def test_jpeg_reader(host, tmp_path, subsample, restart, grey, size):
    rng = np.random.default_rng(size[0] * 7 + size[1])
    h, w = size
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.stack([128 + 90 * np.sin(xx / 5.0), 128 + 80 * np.cos(yy / 4.0), (xx * 3 + yy * 2) % 256], -1)
    img = np.clip(img + rng.normal(0, 12, img.shape), 0, 255).astype(np.uint8)
    src = img[..., 1] if grey else img
    q = 3
    data, comps, samp, layout = _jpeg_bytes(src, subsample, q, restart, grey)
    path = tmp_path / "t.jpg"
    path.write_bytes(data)
    got = _load_env(host, path)
    img8 = _jpeg_expected(comps, samp, layout, h, w, q, grey)
    c = img8.shape[-1]
    expect = _expect_rgba(img8, c).reshape(h, w, 4)
    # every sample within one level of the restated arithmetic (rounding of
    # exact halves may differ with the summation order), almost all exact
    lvl = np.round(np.power(got[..., :3], 1 / 2.2) * 255).astype(int)
    ref = np.round(np.power(expect[..., :3], 1 / 2.2) * 255).astype(int)
    assert np.abs(lvl - ref).max() <= 1 and (lvl == ref).mean() > 0.999
    # and close to the source image (a sanity check of the whole round trip)
    srcf = (src[..., None] if grey else src).astype(float)
    dec = np.round(np.power(got[..., :3], 1 / 2.2) * 255)[..., :c] if not grey else lvl[..., :1]
    assert np.abs(dec - srcf).mean() < (10.0 if subsample else 4.0)  # 4:2:0 averages noisy chroma


def test_progressive_jpeg_is_reported(host, tmp_path):
    data = bytearray(_jpeg_bytes(np.zeros((8, 8, 3), np.uint8), False, 2)[0])
    i = data.index(b"\xFF\xC0")
    data[i + 1] = 0xC2
    path = tmp_path / "p.jpg"
    path.write_bytes(bytes(data))
    with pytest.raises(abi.PtError) as e:
        _load_env(host, path)
    assert "progressive" in str(e.value)
