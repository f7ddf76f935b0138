"""Scene descriptions for the tracer: a builder that produces the C-ABI
``pt_scene_desc`` from numpy arrays, material constructors with the
reference loader's defaults (framework/resource/material.cpp:18-157), and
the seeded procedural scenes the benchmarks and tests run on.

Procedural scenes (seeded, synthetic; no external assets):

* ``cornell_box`` -- 5 walls (10 triangles), two boxes (24 triangles)
  rotated +15 / -18 degrees about y, a 0.25 x 0.25 ceiling light with
  radiance (17, 12, 4); white 0.73, red (0.65, 0.05, 0.05), green
  (0.12, 0.45, 0.15); 40 degree pinhole; 256 x 256, max depth 4.
* ``icosphere_field`` -- 200 instances of a 4-times subdivided icosahedron
  (5120 triangles each) displaced by seeded FBM value noise (amplitude 0.1),
  placed uniformly in a 20^3 box over a tessellated ground plane; each
  instance draws one of the seven materials (alpha ~ U(0.05, 0.6), IOR ~
  U(1.3, 1.8), albedo ~ U(0.1, 0.9)^3); constant environment 0.5 and four
  emissive spheres; 1920 x 1080, max depth 8 (1,024,000 instance triangles +
  8,192 ground triangles + 4 spheres).
"""
from __future__ import annotations

import contextlib
import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

# ----------------------------------------------------------------------------- materials

_IDENTITY_UV = (1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0)


def rgb(value) -> abi.TextureDesc:
    t = abi.TextureDesc()
    t.type = abi.TEX_RGB
    v = np.broadcast_to(np.asarray(value, np.float32), (3,))
    t.color0[:] = [float(x) for x in v]
    t.color1[:] = [0.0, 0.0, 0.0]
    t.uv_transform[:] = _IDENTITY_UV
    return t


def checkerboard(patch1=(0.4, 0.4, 0.4), patch2=(0.2, 0.2, 0.2), uv_scale=1.0) -> abi.TextureDesc:
    t = abi.TextureDesc()
    t.type = abi.TEX_CHECKERBOARD
    t.color0[:] = [float(x) for x in patch1]
    t.color1[:] = [float(x) for x in patch2]
    t.uv_transform[:] = (uv_scale, 0.0, 0.0, 0.0, 0.0, uv_scale, 0.0, 0.0)
    return t


def bitmap(pixels: np.ndarray, address=abi.TEX_ADDRESS_WRAP, filter=abi.TEX_FILTER_LINEAR,
           uv_scale=1.0) -> abi.TextureDesc:
    """A bitmap texture over (h, w, 4) RGBA float32 pixels (row 0 first).  The
    array must stay alive until the scene is uploaded: Scene.add_material keeps
    it when the material is added through Scene."""
    px = np.ascontiguousarray(pixels, np.float32)
    assert px.ndim == 3 and px.shape[2] == 4
    t = abi.TextureDesc()
    t.type = abi.TEX_BITMAP
    t.uv_transform[:] = (uv_scale, 0.0, 0.0, 0.0, 0.0, uv_scale, 0.0, 0.0)
    t.pixels = px.ctypes.data
    t.height, t.width = px.shape[0], px.shape[1]
    t.address_mode = address
    t.filter = filter
    _BITMAP_KEEP[t.pixels] = px
    return t


# pixels of bitmap textures by address, kept alive for the scenes that use them
_BITMAP_KEEP: dict = {}


@dataclass
class EnvMap:
    """An equirectangular environment map: (h, w, 4) RGBA float32 radiance."""
    pixels: np.ndarray
    scale: float = 1.0
    to_world: np.ndarray | None = None


def _mat(type_, texs, int_ior=1.0, ext_ior=1.0, nonlinear=False, twosided=False) -> abi.MaterialDesc:
    m = abi.MaterialDesc()
    m.type = type_
    m.twosided = 1 if twosided else 0
    m.nonlinear = 1 if nonlinear else 0
    m.int_ior = int_ior
    m.ext_ior = ext_ior
    for i in range(4):
        m.tex[i] = texs[i] if i < len(texs) else rgb(0.0)
    return m


def _tex(v):
    return v if isinstance(v, abi.TextureDesc) else rgb(v)


def diffuse(reflectance=0.5, twosided=False):
    return _mat(abi.MAT_DIFFUSE, [_tex(reflectance)], twosided=twosided)


def dielectric(int_ior=1.5046, ext_ior=1.000277, specular_reflectance=1.0, specular_transmittance=1.0, twosided=False):
    return _mat(abi.MAT_DIELECTRIC, [_tex(specular_reflectance), _tex(specular_transmittance)], int_ior, ext_ior,
                twosided=twosided)


def rough_dielectric(alpha=0.1, int_ior=1.5046, ext_ior=1.000277, specular_reflectance=1.0,
                     specular_transmittance=1.0, twosided=False):
    return _mat(abi.MAT_ROUGH_DIELECTRIC, [_tex(specular_reflectance), _tex(specular_transmittance), _tex(alpha)],
                int_ior, ext_ior, twosided=twosided)


def conductor(eta=(0.0, 0.0, 0.0), k=(1.0, 1.0, 1.0), specular_reflectance=1.0, twosided=False):
    return _mat(abi.MAT_CONDUCTOR, [_tex(specular_reflectance), _tex(eta), _tex(k)], twosided=twosided)


def rough_conductor(alpha=0.1, eta=(0.0, 0.0, 0.0), k=(1.0, 1.0, 1.0), specular_reflectance=1.0, twosided=False):
    return _mat(abi.MAT_ROUGH_CONDUCTOR, [_tex(specular_reflectance), _tex(eta), _tex(k), _tex(alpha)],
                twosided=twosided)


def plastic(diffuse_reflectance=0.5, int_ior=1.49, ext_ior=1.000277, nonlinear=False, specular_reflectance=1.0,
            twosided=False):
    return _mat(abi.MAT_PLASTIC, [_tex(diffuse_reflectance), _tex(specular_reflectance)], int_ior, ext_ior,
                nonlinear=nonlinear, twosided=twosided)


def rough_plastic(alpha=0.1, diffuse_reflectance=0.5, int_ior=1.49, ext_ior=1.000277, nonlinear=False,
                  specular_reflectance=1.0, twosided=False):
    return _mat(abi.MAT_ROUGH_PLASTIC, [_tex(diffuse_reflectance), _tex(specular_reflectance), _tex(alpha)],
                int_ior, ext_ior, nonlinear=nonlinear, twosided=twosided)


# ----------------------------------------------------------------------------- transforms

def translate(x, y, z):
    m = np.eye(4, dtype=np.float64)
    m[:3, 3] = (x, y, z)
    return m


def scale(sx, sy=None, sz=None):
    sy = sx if sy is None else sy
    sz = sx if sz is None else sz
    return np.diag([sx, sy, sz, 1.0])


def rotate_y(deg):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    m = np.eye(4)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    return m


def rotate_axis(axis, deg):
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    x, y, z = axis
    r = np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                  [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                  [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])
    m = np.eye(4)
    m[:3, :3] = r
    return m


def look_at_to_world(eye, target, up=(0.0, 1.0, 0.0)):
    """Camera-to-world in Pupil's convention: +X right, +Y up, +Z points away
    from the view direction (the camera looks down -Z)."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    z = -f
    x = np.cross(np.asarray(up, np.float64), z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = x, y, z, eye
    return m


_camera_maker = None


@contextlib.contextmanager
def camera_maker(fn):
    """Within the block, scene cameras are made by `fn(fov_y, aspect, near,
    far, to_world) -> CameraDesc` instead of the library's pt_camera_make, so
    that a CPU-only caller (the timed CPU restatement of the integrator) can
    build the procedural scenes without loading libpt_gb300.so."""
    global _camera_maker
    prev, _camera_maker = _camera_maker, fn
    try:
        yield
    finally:
        _camera_maker = prev


def camera(fov_y_deg: float, aspect: float, to_world, near_clip=0.01, far_clip=10000.0) -> abi.CameraDesc:
    """sample_to_camera / camera_to_world through the library's pt_camera_make
    (or the maker installed by camera_maker)."""
    if _camera_maker is not None:
        return _camera_maker(fov_y_deg, aspect, near_clip, far_clip,
                             np.asarray(to_world, np.float64).reshape(-1).astype(np.float32))
    lib = abi.load()
    cam = abi.CameraDesc()
    tw = (C.c_float * 16)(*[float(v) for v in np.asarray(to_world, np.float64).reshape(-1)])
    abi.check(lib.pt_camera_make(fov_y_deg, aspect, near_clip, far_clip, tw, C.byref(cam)), "pt_camera_make", lib)
    return cam


# ----------------------------------------------------------------------------- builder

@dataclass
class Mesh:
    positions: np.ndarray          # (V, 3) float32
    indices: np.ndarray            # (T, 3) uint32
    normals: np.ndarray | None = None
    texcoords: np.ndarray | None = None

    def __post_init__(self):
        self.positions = np.ascontiguousarray(self.positions, np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(self.indices, np.uint32).reshape(-1, 3)
        if self.normals is not None:
            self.normals = np.ascontiguousarray(self.normals, np.float32).reshape(-1, 3)
        if self.texcoords is not None:
            self.texcoords = np.ascontiguousarray(self.texcoords, np.float32).reshape(-1, 2)


@dataclass
class Curves:
    """Curve strands (pt_curves_desc): control points, per-point radii, the
    first control point of every segment and the curve type (abi.CURVE_*)."""
    positions: np.ndarray          # (P, 3) float32
    radii: np.ndarray              # (P,) float32
    segments: np.ndarray           # (S,) uint32
    type: int = abi.CURVE_CUBIC_BSPLINE

    def __post_init__(self):
        self.positions = np.ascontiguousarray(self.positions, np.float32).reshape(-1, 3)
        self.radii = np.ascontiguousarray(self.radii, np.float32).reshape(-1)
        self.segments = np.ascontiguousarray(self.segments, np.uint32).reshape(-1)

    @staticmethod
    def from_strands(strands, radii, type=abi.CURVE_CUBIC_BSPLINE) -> "Curves":
        """Strands given as point lists; segments as the reference's hair
        loader forms them (framework/resource/shape.cpp:401-408): every start
        index of a strand up to its point count minus the degree."""
        deg = 3 if type > 2 else type + 1
        pos = [np.asarray(p, np.float32).reshape(-1, 3) for p in strands]
        counts = np.array([p.shape[0] for p in pos], np.int64)
        rad = [np.broadcast_to(np.asarray(r, np.float32), (c,)) for r, c in zip(radii, counts)]
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
        seg = np.concatenate([np.arange(a, a + max(0, c - deg)) for a, c in zip(starts, counts)])
        return Curves(np.concatenate(pos), np.concatenate(rad), seg.astype(np.uint32), type)


@dataclass
class Scene:
    """Host-side scene: what resource::Scene holds for the path-tracing pass."""
    width: int
    height: int
    max_depth: int
    meshes: list = field(default_factory=list)
    spheres: list = field(default_factory=list)     # (center(3), radius)
    materials: list = field(default_factory=list)   # abi.MaterialDesc
    instances: list = field(default_factory=list)   # dicts
    curves: list = field(default_factory=list)      # Curves
    env: tuple | EnvMap | None = None                # constant environment radiance or a map
    camera: abi.CameraDesc | None = None
    name: str = "scene"

    def add_mesh(self, mesh: Mesh) -> int:
        self.meshes.append(mesh)
        return len(self.meshes) - 1

    def add_sphere(self, center, radius) -> int:
        self.spheres.append((tuple(float(c) for c in center), float(radius)))
        return len(self.spheres) - 1

    def add_curves(self, curves: Curves) -> int:
        self.curves.append(curves)
        return len(self.curves) - 1

    def add_material(self, m: abi.MaterialDesc) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def add_instance(self, shape_type, shape_index, material, to_world=None, radiance=None, flags=0) -> int:
        self.instances.append(dict(shape_type=shape_type, shape_index=shape_index, material=material,
                                   to_world=np.eye(4) if to_world is None else np.asarray(to_world, np.float64),
                                   radiance=radiance, flags=flags))
        return len(self.instances) - 1

    @property
    def num_triangles(self) -> int:
        return sum(self.meshes[i["shape_index"]].indices.shape[0] for i in self.instances
                   if i["shape_type"] == abi.SHAPE_MESH)

    def desc(self) -> abi.SceneDesc:
        """Build the C descriptor.  The returned object keeps every array it
        points to alive (attribute ``_keep``)."""
        keep = []
        meshes = (abi.MeshDesc * max(1, len(self.meshes)))()
        for i, m in enumerate(self.meshes):
            d = meshes[i]
            d.positions = m.positions.ctypes.data_as(abi.c_float_p)
            d.normals = m.normals.ctypes.data_as(abi.c_float_p) if m.normals is not None else None
            d.texcoords = m.texcoords.ctypes.data_as(abi.c_float_p) if m.texcoords is not None else None
            d.indices = m.indices.ctypes.data_as(abi.c_uint_p)
            d.num_vertices = m.positions.shape[0]
            d.num_triangles = m.indices.shape[0]
            keep.append(m)
        spheres = (abi.SphereDesc * max(1, len(self.spheres)))()
        for i, (c, r) in enumerate(self.spheres):
            spheres[i].center[:] = list(c)
            spheres[i].radius = r
        curves = (abi.CurvesDesc * max(1, len(self.curves)))()
        for i, cv in enumerate(self.curves):
            d = curves[i]
            d.positions = cv.positions.ctypes.data_as(abi.c_float_p)
            d.radii = cv.radii.ctypes.data_as(abi.c_float_p)
            d.segments = cv.segments.ctypes.data_as(abi.c_uint_p)
            d.num_points = cv.positions.shape[0]
            d.num_segments = cv.segments.shape[0]
            d.type = cv.type
            keep.append(cv)
        mats = (abi.MaterialDesc * max(1, len(self.materials)))(*self.materials)
        insts = (abi.InstanceDesc * max(1, len(self.instances)))()
        for i, inst in enumerate(self.instances):
            d = insts[i]
            d.shape_type = inst["shape_type"]
            d.shape_index = inst["shape_index"]
            d.material = inst["material"]
            d.flags = inst["flags"]
            d.to_world[:] = [float(v) for v in np.asarray(inst["to_world"], np.float32).reshape(-1)]
            if inst["radiance"] is not None:
                d.is_emitter = 1
                if isinstance(inst["radiance"], abi.TextureDesc):  # a textured area emitter
                    d.radiance_textured = 1
                    d.radiance_tex = inst["radiance"]
                else:
                    d.radiance[:] = [float(v) for v in inst["radiance"]]
        sd = abi.SceneDesc()
        sd.meshes = C.cast(meshes, C.POINTER(abi.MeshDesc))
        sd.num_meshes = len(self.meshes)
        sd.spheres = C.cast(spheres, C.POINTER(abi.SphereDesc))
        sd.num_spheres = len(self.spheres)
        sd.materials = C.cast(mats, C.POINTER(abi.MaterialDesc))
        sd.num_materials = len(self.materials)
        sd.instances = C.cast(insts, C.POINTER(abi.InstanceDesc))
        sd.num_instances = len(self.instances)
        sd.curves = C.cast(curves, C.POINTER(abi.CurvesDesc))
        sd.num_curves = len(self.curves)
        if isinstance(self.env, EnvMap):
            px = np.ascontiguousarray(self.env.pixels, np.float32)
            keep.append(px)
            sd.env.type = abi.ENV_MAP
            sd.env.pixels = px.ctypes.data
            sd.env.height, sd.env.width = px.shape[0], px.shape[1]
            sd.env.scale = float(self.env.scale)
            tw = np.eye(4) if self.env.to_world is None else np.asarray(self.env.to_world, np.float64)
            sd.env.to_world[:] = [float(v) for v in tw.astype(np.float32).reshape(-1)]
        elif self.env is not None:
            sd.env.type = abi.ENV_CONST
            sd.env.radiance[:] = [float(v) for v in self.env]
        if self.camera is not None:
            sd.camera = self.camera
        sd.width, sd.height, sd.max_depth = self.width, self.height, self.max_depth
        sd._keep = (keep, meshes, spheres, mats, insts, curves)
        return sd


# ----------------------------------------------------------------------------- shapes

def quad(p0, p1, p2, p3, normal=None) -> Mesh:
    """Two triangles (p0,p1,p2), (p0,p2,p3) with uvs (0,0),(1,0),(1,1),(0,1)."""
    pos = np.array([p0, p1, p2, p3], np.float32)
    if normal is None:
        n = np.cross(pos[1] - pos[0], pos[2] - pos[0])
        normal = n / np.linalg.norm(n)
    nrm = np.tile(np.asarray(normal, np.float32), (4, 1))
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    return Mesh(pos, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), nrm, uv)


def cube() -> Mesh:
    """Unit cube [-1,1]^3: 6 faces x 4 vertices with face normals, 12 triangles."""
    faces = []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            n = np.zeros(3)
            n[axis] = sign
            u = np.zeros(3)
            u[(axis + 1) % 3] = 1.0
            v = np.cross(n, u)
            c = n
            corners = [c - u - v, c + u - v, c + u + v, c - u + v]
            faces.append((corners, n))
    pos, nrm, uv, idx = [], [], [], []
    for f, (corners, n) in enumerate(faces):
        pos += corners
        nrm += [n] * 4
        uv += [[0, 0], [1, 0], [1, 1], [0, 1]]
        b = 4 * f
        idx += [[b, b + 1, b + 2], [b, b + 2, b + 3]]
    return Mesh(np.array(pos), np.array(idx), np.array(nrm), np.array(uv))


def grid(nx: int, nz: int, half: float, y: float = 0.0) -> Mesh:
    xs = np.linspace(-half, half, nx + 1, dtype=np.float64)
    zs = np.linspace(-half, half, nz + 1, dtype=np.float64)
    X, Z = np.meshgrid(xs, zs, indexing="xy")
    pos = np.stack([X.ravel(), np.full(X.size, y), Z.ravel()], 1)
    uv = np.stack([(X.ravel() + half) / (2 * half), (Z.ravel() + half) / (2 * half)], 1)
    i = np.arange(nz)[:, None] * (nx + 1) + np.arange(nx)[None, :]
    a, b, c, d = i, i + 1, i + nx + 2, i + nx + 1
    # winding so that the geometric normal points up (+y)
    idx = np.concatenate([np.stack([a, d, c], -1).reshape(-1, 3), np.stack([a, c, b], -1).reshape(-1, 3)])
    nrm = np.tile([0.0, 1.0, 0.0], (pos.shape[0], 1))
    return Mesh(pos, idx, nrm, uv)


def icosphere(subdivisions: int = 4) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: 20 * 4^s triangles.  Returns (vertices (V,3) float64, faces (F,3))."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdivisions):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = v.shape[0]
        v = np.concatenate([v, mid])
        nf = f.shape[0]
        ab, bc, ca = inv[:nf] + base, inv[nf:2 * nf] + base, inv[2 * nf:] + base
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                            np.stack([ab, bc, ca], 1)])
    return v, f


def _hash_u32(x):
    x = x.astype(np.uint32)
    x ^= x >> np.uint32(16)
    x *= np.uint32(0x7FEB352D)
    x ^= x >> np.uint32(15)
    x *= np.uint32(0x846CA68B)
    x ^= x >> np.uint32(16)
    return x


def value_noise3(p: np.ndarray, seed: int) -> np.ndarray:
    """Trilinear value noise in [-1, 1] on the integer lattice (smoothstep fade)."""
    pi = np.floor(p).astype(np.int64)
    fr = p - pi
    w = fr * fr * (3.0 - 2.0 * fr)
    out = np.zeros(p.shape[0])
    s = np.uint32((seed * 0x9E3779B1) & 0xFFFFFFFF)
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                ix = (pi[:, 0] + dx).astype(np.uint32)
                iy = (pi[:, 1] + dy).astype(np.uint32)
                iz = (pi[:, 2] + dz).astype(np.uint32)
                h = _hash_u32(ix * np.uint32(0x8DA6B343) ^ iy * np.uint32(0xD8163841) ^ iz * np.uint32(0xCB1AB31F) ^ s)
                val = h.astype(np.float64) / 4294967295.0 * 2.0 - 1.0
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out += wx * wy * wz * val
    return out


def fbm(p: np.ndarray, seed: int, octaves: int = 4) -> np.ndarray:
    total = np.zeros(p.shape[0])
    amp, freq, norm = 1.0, 1.0, 0.0
    for o in range(octaves):
        total += amp * value_noise3(p * freq, seed * 31 + o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def vertex_normals(pos: np.ndarray, faces: np.ndarray) -> np.ndarray:
    fn = np.cross(pos[faces[:, 1]] - pos[faces[:, 0]], pos[faces[:, 2]] - pos[faces[:, 0]])
    n = np.zeros_like(pos)
    for k in range(3):
        np.add.at(n, faces[:, k], fn)
    return n / np.linalg.norm(n, axis=1, keepdims=True)


def displaced_icosphere(seed: int, amplitude: float = 0.1, subdivisions: int = 4, base=None) -> Mesh:
    v, f = base if base is not None else icosphere(subdivisions)
    offset = np.array([seed * 1.7, seed * 2.3, seed * 3.1]) % 97.0
    d = fbm(v * 2.0 + offset, seed)
    pos = v * (1.0 + amplitude * d)[:, None]
    nrm = vertex_normals(pos, f)
    uv = np.stack([0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * math.pi), np.arccos(np.clip(v[:, 1], -1, 1)) / math.pi], 1)
    return Mesh(pos, f, nrm, uv)


# ----------------------------------------------------------------------------- the procedural scenes

def cornell_box(width: int = 256, height: int = 256, max_depth: int = 4) -> Scene:
    s = Scene(width, height, max_depth, name="cornell_box")
    white = s.add_material(diffuse(0.73, twosided=True))
    red = s.add_material(diffuse((0.65, 0.05, 0.05), twosided=True))
    green = s.add_material(diffuse((0.12, 0.45, 0.15), twosided=True))
    black = s.add_material(diffuse(0.0, twosided=True))
    walls = [
        (quad((-1, 0, 1), (1, 0, 1), (1, 0, -1), (-1, 0, -1), (0, 1, 0)), white),      # floor
        (quad((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1), (0, -1, 0)), white),     # ceiling
        (quad((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1), (0, 0, 1)), white),    # back
        (quad((-1, 0, 1), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1), (1, 0, 0)), red),      # left
        (quad((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1), (-1, 0, 0)), green),       # right
    ]
    for mesh, mat in walls:
        s.add_instance(abi.SHAPE_MESH, s.add_mesh(mesh), mat)
    box = s.add_mesh(cube())
    s.add_instance(abi.SHAPE_MESH, box, white,
                   translate(-0.33, 0.6, -0.29) @ rotate_y(15.0) @ scale(0.3, 0.6, 0.3))    # tall box
    s.add_instance(abi.SHAPE_MESH, box, white,
                   translate(0.33, 0.3, 0.37) @ rotate_y(-18.0) @ scale(0.3, 0.3, 0.3))     # short box
    h = 0.125
    light = quad((-h, 1.98, -h), (-h, 1.98, h), (h, 1.98, h), (h, 1.98, -h), (0, -1, 0))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(light), black, radiance=(17.0, 12.0, 4.0))
    s.camera = camera(40.0, width / height, look_at_to_world((0.0, 1.0, 3.8), (0.0, 1.0, 0.0)))
    return s


def _conductor_params(rng):
    # a few measured-metal-like (eta, k) triples (gold, copper, silver, aluminium)
    table = [((0.143, 0.374, 1.442), (3.983, 2.385, 1.603)), ((0.200, 0.924, 1.102), (3.912, 2.452, 2.142)),
             ((0.155, 0.117, 0.138), (4.828, 3.122, 2.147)), ((1.657, 0.880, 0.521), (9.224, 6.270, 4.837))]
    return table[int(rng.integers(0, len(table)))]


def random_material(rng, kind: int) -> abi.MaterialDesc:
    alpha = float(rng.uniform(0.05, 0.6))
    ior = float(rng.uniform(1.3, 1.8))
    albedo = tuple(float(x) for x in rng.uniform(0.1, 0.9, 3))
    if kind == abi.MAT_DIFFUSE:
        return diffuse(albedo)
    if kind == abi.MAT_DIELECTRIC:
        return dielectric(ior, 1.0)
    if kind == abi.MAT_ROUGH_DIELECTRIC:
        return rough_dielectric(alpha, ior, 1.0)
    if kind == abi.MAT_CONDUCTOR:
        eta, k = _conductor_params(rng)
        return conductor(eta, k, albedo)
    if kind == abi.MAT_ROUGH_CONDUCTOR:
        eta, k = _conductor_params(rng)
        return rough_conductor(alpha, eta, k, albedo)
    if kind == abi.MAT_PLASTIC:
        return plastic(albedo, ior, 1.0, nonlinear=bool(rng.integers(0, 2)))
    return rough_plastic(alpha, albedo, ior, 1.0, nonlinear=bool(rng.integers(0, 2)))


def random_rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    m = np.eye(4)
    m[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                 [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                 [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
    return m


def icosphere_field(width: int = 1920, height: int = 1080, max_depth: int = 8, num_instances: int = 200,
                    subdivisions: int = 4, seed: int = 0, amplitude: float = 0.1) -> Scene:
    s = Scene(width, height, max_depth, name=f"icosphere_field_{num_instances}")
    rng = np.random.default_rng(seed)
    base = icosphere(subdivisions)
    ground_mat = s.add_material(diffuse(0.5))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(grid(64, 64, 40.0, 0.0)), ground_mat)
    for i in range(num_instances):
        mesh = displaced_icosphere(seed * 100003 + i, amplitude, subdivisions, base)
        kind = int(rng.integers(1, 8))
        mat = s.add_material(random_material(rng, kind))
        pos = (rng.uniform(-10, 10), rng.uniform(1.5, 21.5), rng.uniform(-10, 10))
        sc = float(rng.uniform(0.6, 1.4))
        tw = translate(*pos) @ random_rotation(rng) @ scale(sc)
        s.add_instance(abi.SHAPE_MESH, s.add_mesh(mesh), mat, tw)
    light_mat = s.add_material(diffuse(0.0))
    for (x, y, z) in [(-8.0, 24.0, -8.0), (8.0, 24.0, -8.0), (-8.0, 24.0, 8.0), (8.0, 24.0, 8.0)]:
        s.add_instance(abi.SHAPE_SPHERE, s.add_sphere((0.0, 0.0, 0.0), 1.0), light_mat, translate(x, y, z) @ scale(1.5),
                       radiance=(12.0, 11.0, 9.0))
    s.env = (0.5, 0.5, 0.5)
    s.camera = camera(40.0, width / height, look_at_to_world((0.0, 14.0, 38.0), (0.0, 10.0, 0.0)))
    return s


def mesh_pool(count: int = 32, subdivisions: int = 4, amplitude: float = 0.1, seed: int = 0) -> list:
    """`count` seeded displaced icospheres that several scenes can instance."""
    base = icosphere(subdivisions)
    return [displaced_icosphere(seed * 100003 + i, amplitude, subdivisions, base) for i in range(count)]


def pooled_field(seed: int, num_instances: int, width: int, height: int, max_depth: int = 8, pool=None) -> Scene:
    """An icosphere field like icosphere_field (7 random materials, ground,
    constant environment 0.5, 4 sphere lights) whose instances reuse the
    meshes of `pool`; the field's box grows with the instance count so the
    density stays that of the 200-instance field."""
    pool = pool if pool is not None else mesh_pool()
    s = Scene(width, height, max_depth, name=f"pooled_field_{seed}_{num_instances}")
    rng = np.random.default_rng(seed)
    half = 10.0 * (max(num_instances, 1) / 200.0) ** (1.0 / 3.0)
    ground_mat = s.add_material(diffuse(0.5))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(grid(64, 64, 4.0 * half, 0.0)), ground_mat)
    mesh_ids = {}
    for i in range(num_instances):
        j = int(rng.integers(0, len(pool)))
        if j not in mesh_ids:
            mesh_ids[j] = s.add_mesh(pool[j])
        mat = s.add_material(random_material(rng, int(rng.integers(1, 8))))
        pos = (rng.uniform(-half, half), rng.uniform(1.5, 1.5 + 2 * half), rng.uniform(-half, half))
        tw = translate(*pos) @ random_rotation(rng) @ scale(float(rng.uniform(0.6, 1.4)))
        s.add_instance(abi.SHAPE_MESH, mesh_ids[j], mat, tw)
    light_mat = s.add_material(diffuse(0.0))
    l = 0.8 * half
    sphere = s.add_sphere((0.0, 0.0, 0.0), 1.0)
    for (x, z) in [(-l, -l), (l, -l), (-l, l), (l, l)]:
        s.add_instance(abi.SHAPE_SPHERE, sphere, light_mat, translate(x, 2.4 * half, z) @ scale(0.15 * half),
                       radiance=(12.0, 11.0, 9.0))
    s.env = (0.5, 0.5, 0.5)
    s.camera = camera(40.0, width / height, look_at_to_world((0.0, 1.4 * half, 3.8 * half), (0.0, half, 0.0)))
    return s


def material_spheres(width: int = 96, height: int = 64, max_depth: int = 6) -> Scene:
    """Seven spheres (mesh icospheres, one per material) over a checkerboard
    floor, lit by the environment and one emissive sphere: small parity scene."""
    s = Scene(width, height, max_depth, name="material_spheres")
    rng = np.random.default_rng(7)
    base = icosphere(3)
    floor = s.add_material(diffuse(checkerboard((0.8, 0.8, 0.8), (0.2, 0.2, 0.2), 8.0)))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(grid(8, 8, 10.0, 0.0)), floor)
    mesh = s.add_mesh(displaced_icosphere(3, 0.0, 3, base))
    for k in range(1, 8):
        m = s.add_material(random_material(rng, k))
        s.add_instance(abi.SHAPE_MESH, mesh, m, translate(-6.0 + 2.0 * (k - 1), 1.0, 0.0) @ scale(0.9))
    lm = s.add_material(diffuse(0.0, twosided=True))
    s.add_instance(abi.SHAPE_SPHERE, s.add_sphere((0.0, 0.0, 0.0), 1.0), lm, translate(0.0, 6.0, 3.0),
                   radiance=(8.0, 8.0, 8.0))
    s.env = (0.3, 0.35, 0.4)
    s.camera = camera(35.0, width / height, look_at_to_world((0.0, 3.0, 12.0), (0.0, 1.0, 0.0)))
    return s


def hair_strands(num_strands: int, points: int = 10, length: float = 1.2, radius: float = 0.012, tapered: bool = False,
                 seed: int = 0, curl: float = 0.25) -> tuple[list, list]:
    """Strands grown from the upper half of a unit sphere: each root steps out
    along its normal, bends down under a constant pull and wanders with a
    seeded curl.  Returns (point lists, radius lists); radii taper to zero
    along a strand as the reference's tapered hair does
    (framework/resource/shape.cpp:385-393) when tapered is set."""
    rng = np.random.default_rng(seed)
    roots = rng.normal(size=(num_strands, 3))
    roots[:, 1] = np.abs(roots[:, 1]) + 0.2
    roots /= np.linalg.norm(roots, axis=1, keepdims=True)
    step = length / (points - 1)
    noise = rng.normal(size=(points - 1, num_strands, 3)) * curl
    p, d = roots.copy(), roots.copy()
    pts = [p]
    for k in range(points - 1):  # all strands advance together
        d = d + np.array([0.0, -0.35, 0.0]) + noise[k]
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        p = p + d * step
        pts.append(p)
    strands = list(np.stack(pts, 1).astype(np.float32))
    r = radius * (points - 1 - np.arange(points)) / (points - 1) if tapered else np.full(points, radius)
    return strands, [r] * num_strands


def hair_scene(width: int = 64, height: int = 48, curve_type: int = abi.CURVE_CUBIC_BSPLINE, num_strands: int = 300,
               points: int = 10, radius: float = 0.012, tapered: bool = False, max_depth: int = 6, seed: int = 0,
               env: bool = True, curl: float = 0.25) -> Scene:
    """A sphere ("head", mesh) carrying curve strands of one curve type over a
    floor, lit by a sphere light and a constant environment; the strands'
    instance has a rotation, a uniform scale and a translation."""
    s = Scene(width, height, max_depth, name=f"hair_t{curve_type}")
    floor = s.add_material(diffuse(checkerboard((0.7, 0.7, 0.7), (0.3, 0.3, 0.3), 6.0)))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(grid(4, 4, 6.0, 0.0)), floor)
    head = s.add_material(plastic((0.6, 0.5, 0.4), 1.5, 1.0))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(displaced_icosphere(1, 0.0, 3)), head,
                   translate(0.0, 1.4, 0.0) @ scale(0.95))
    strands, radii = hair_strands(num_strands, points, radius=radius, tapered=tapered, seed=seed, curl=curl)
    hair = s.add_material(rough_conductor(0.25, eta=(0.2, 0.4, 1.4), k=(3.5, 2.5, 2.0)))
    cv = s.add_curves(Curves.from_strands(strands, radii, curve_type))
    s.add_instance(abi.SHAPE_CURVES, cv, hair, translate(0.0, 1.4, 0.0) @ rotate_y(25.0) @ scale(1.0))
    lm = s.add_material(diffuse(0.0, twosided=True))
    s.add_instance(abi.SHAPE_SPHERE, s.add_sphere((0.0, 0.0, 0.0), 0.6), lm, translate(2.0, 5.0, 3.0),
                   radiance=(14.0, 13.0, 12.0))
    if env:
        s.env = (0.25, 0.3, 0.35)
    s.camera = camera(35.0, width / height, look_at_to_world((0.0, 2.2, 5.5), (0.0, 1.3, 0.0)))
    return s
