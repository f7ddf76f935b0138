"""Edge cases of the path against the oracle: scenes without geometry, with
only spheres or only curves, degenerate triangles, geometry far from the
origin, one-pixel and ragged images, and a zero-sample call."""
import numpy as np
import pytest
import torch

import oracle
from pupiloptixlab_gb300 import abi, scenes
from pupiloptixlab_gb300.api import GpuScene
from _parity import assert_bit_identical

pytestmark = pytest.mark.gpu


def params(spp, seed=0, rng=abi.RNG_PCG32):
    return abi.RenderParams(spp=spp, max_depth=0, seed=seed, sample_cnt=0, accumulate=1, rng=rng)


def gpu_trace(g, rays, anyhit=False):
    return g.trace(torch.from_numpy(np.ascontiguousarray(rays)).cuda(), anyhit=anyhit).cpu().numpy()


def agree(a, b, rel=1e-4):
    return np.all(np.abs(a - b) <= rel * np.maximum(1.0, np.abs(b)), axis=1)


def random_rays(rng, n, center, half):
    o = rng.uniform(-1, 1, (n, 3)) * half + center
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = o, 1e-3, d, 1e16
    return r


def bare_scene(w=16, h=12, env=None):
    s = scenes.Scene(w, h, 4, name="bare")
    s.add_material(scenes.diffuse(0.5))
    s.env = env
    s.camera = scenes.camera(40.0, w / h, scenes.look_at_to_world((0, 0, 5), (0, 0, 0)))
    return s


@pytest.mark.parametrize("env", [None, (0.25, 0.5, 0.75)])
def test_scene_without_geometry(cuda_ctx, env):
    sc = bare_scene(env=env)
    g = GpuScene(cuda_ctx, sc)
    out = g.render(3, seed=1)
    acc = out["accum"].cpu().numpy()
    ref = oracle.OracleScene(sc).render(params(3, seed=1))["accum"]
    assert np.array_equal(acc, ref)
    expect = np.zeros(3) if env is None else np.array(env)
    assert np.allclose(acc[:, :3], expect, atol=1e-6)
    g.close()


@pytest.mark.parametrize("size", [(1, 1), (1, 37), (37, 1), (13, 7)])
def test_one_pixel_and_ragged_images(cuda_ctx, size):
    w, h = size
    sc = scenes.cornell_box(w, h)
    g = GpuScene(cuda_ctx, sc)
    ref = oracle.OracleScene(sc).render(params(4, seed=2, rng=abi.RNG_REF_LCG))
    got = {k: v.cpu().numpy() for k, v in g.render(4, seed=2, rng=abi.RNG_REF_LCG).items()}
    ok = agree(got["accum"][:, :3], ref["accum"][:, :3])
    assert (~ok).sum() <= max(0, int(0.03 * w * h)), f"{(~ok).sum()} of {w * h} pixels differ"
    assert np.array_equal(got["test"], ref["test"])
    assert np.array_equal(got["albedo"], ref["albedo"])
    g.close()


def test_sphere_only_and_curve_only_scenes(cuda_ctx):
    rng = np.random.default_rng(4)
    s = bare_scene(24, 16, env=(0.3, 0.3, 0.3))
    for k in range(6):
        c = rng.uniform(-1.5, 1.5, 3)
        s.add_instance(abi.SHAPE_SPHERE, s.add_sphere(c, rng.uniform(0.1, 0.5)), 0, flags=abi.INST_FLIP_NORMALS * (k % 2))
    s.add_instance(abi.SHAPE_SPHERE, s.add_sphere((0, 3, 0), 0.4), 0, radiance=(5, 5, 5))
    h = bare_scene(24, 16, env=(0.3, 0.3, 0.3))
    strands, radii = scenes.hair_strands(40, 8, radius=0.03, seed=5)
    h.add_instance(abi.SHAPE_CURVES, h.add_curves(scenes.Curves.from_strands(strands, radii, abi.CURVE_CATMULL_ROM)), 0)
    for sc in (s, h):
        g, o = GpuScene(cuda_ctx, sc), oracle.OracleScene(sc)
        rays = np.concatenate([o.camera_rays(abi.RNG_PCG32, 0), random_rays(rng, 5000, (0, 0, 0), (2, 2, 2))])
        got, ref = gpu_trace(g, rays), o.trace(rays, brute_force=True)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
        assert (got[:, 1].view(np.int32) >= 0).sum() > 100
        r = o.render(params(2, seed=3))
        a = g.render(2, seed=3)["accum"].cpu().numpy()
        assert np.isfinite(a).all()
        assert_bit_identical("spheres / curves only", a, r["accum"])
        g.close()


def test_degenerate_triangles(cuda_ctx):
    """Zero-area triangles (repeated and collinear vertices) next to regular
    ones: never hit, never fault, the regular ones still hit exactly."""
    rng = np.random.default_rng(6)
    p = rng.uniform(-1, 1, (60, 3)).astype(np.float32)
    idx = rng.integers(0, 60, (80, 3))
    idx[:20, 1] = idx[:20, 0]                           # a repeated vertex
    p[40:50], p[50:60] = p[30:40] * 0.5, p[30:40] * 0.25  # three points on a line
    idx[20:30] = np.stack([np.arange(30, 40), np.arange(40, 50), np.arange(50, 60)], 1)
    s = bare_scene(env=(0.5, 0.5, 0.5))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(scenes.Mesh(p, idx.astype(np.uint32))), 0)
    g, o = GpuScene(cuda_ctx, s), oracle.OracleScene(s)
    rays = random_rays(rng, 20000, (0, 0, 0), (1.2, 1.2, 1.2))
    got, ref = gpu_trace(g, rays), o.trace(rays, brute_force=True)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    ids = got[:, 1].view(np.int32)
    assert not np.isin(ids, np.arange(30)).any()
    assert (ids >= 30).sum() > 1000
    assert np.isfinite(g.render(2)["accum"].cpu().numpy()).all()
    g.close()


def test_geometry_far_from_the_origin(cuda_ctx):
    """The Cornell box moved 3e4 units away (camera with it): hits stay
    bit-identical to brute force where the box padding must absorb rounding
    at large coordinates."""
    t = np.array([1.0e4, -2.0e4, 3.0e4])
    sc = scenes.cornell_box(24, 24)
    for inst in sc.instances:
        inst["to_world"] = scenes.translate(*t) @ np.asarray(inst["to_world"], np.float64)
    sc.camera = scenes.camera(40.0, 1.0, scenes.look_at_to_world(tuple(t + [0.0, 1.0, 3.8]), tuple(t + [0.0, 1.0, 0.0])))
    g, o = GpuScene(cuda_ctx, sc), oracle.OracleScene(sc)
    rng = np.random.default_rng(8)
    rays = np.concatenate([o.camera_rays(abi.RNG_PCG32, 0), random_rays(rng, 20000, t + [0, 1, 0], (0.99, 0.99, 0.99))])
    got, ref = gpu_trace(g, rays), o.trace(rays, brute_force=True)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert (got[:, 1].view(np.int32) >= 0).mean() > 0.75  # the box is open towards the camera
    g.close()


def test_zero_samples_leave_the_buffers_alone(cuda_ctx):
    g = GpuScene(cuda_ctx, scenes.cornell_box(8, 8))
    b = g.alloc_buffers()
    for v in b.values():
        v.fill_(7.0)
    g.render(0, buffers=b)
    torch.cuda.synchronize()
    assert all(bool((v == 7.0).all()) for v in b.values())
    g.close()


@pytest.mark.parametrize("fast_build", [False, True])
def test_single_primitive_scene(cuda_ctx, fast_build):
    """One sphere: the tree is a single leaf under either builder."""
    s = bare_scene(env=(0.2, 0.2, 0.2))
    s.add_instance(abi.SHAPE_SPHERE, s.add_sphere((0.1, -0.2, 0.0), 0.8), 0)
    g = GpuScene(cuda_ctx, s, bvh_flags=abi.BVH_FAST_BUILD if fast_build else 0)
    o = oracle.OracleScene(s)
    rays = np.concatenate([o.camera_rays(abi.RNG_PCG32, 0), random_rays(np.random.default_rng(2), 2000, (0, 0, 0),
                                                                        (1.5, 1.5, 1.5))])
    assert np.array_equal(gpu_trace(g, rays).view(np.uint32), o.trace(rays, brute_force=True).view(np.uint32))
    g.close()


def test_coincident_primitives(cuda_ctx):
    """3,000 copies of one triangle next to a few ordinary ones: clustering
    finds one mutual pair per pass among equal boxes, so the build must fall
    back to the radix tree within its pass limit; hits stay exact (equal t
    breaks to the lowest primitive id on both sides)."""
    rng = np.random.default_rng(12)
    tri = np.array([[-0.5, -0.5, 0.0], [0.5, -0.5, 0.0], [0.0, 0.5, 0.0]], np.float32)
    extra = rng.uniform(-1.5, 1.5, (30, 3)).astype(np.float32)
    pos = np.concatenate([np.tile(tri, (3000, 1)), extra])
    idx = np.concatenate([np.arange(9000).reshape(-1, 3), 9000 + rng.integers(0, 30, (10, 3))])
    s = bare_scene(env=(0.5, 0.5, 0.5))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(scenes.Mesh(pos, idx.astype(np.uint32))), 0)
    g, o = GpuScene(cuda_ctx, s), oracle.OracleScene(s)
    assert g.bvh_stats().builder == abi.BVH_BUILDER_RADIX
    rays = np.concatenate([o.camera_rays(abi.RNG_PCG32, 0), random_rays(rng, 3000, (0, 0, 0), (1.0, 1.0, 1.0))])
    got, ref = gpu_trace(g, rays), o.trace(rays, brute_force=True)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert (got[:, 1].view(np.int32) == 0).sum() > 50  # the lowest id of the stack of copies
    g.close()


def test_too_many_primitives_are_refused(cuda_ctx):
    """Instances that add up to more than 2^27 - 1 primitives (the leaf items
    on the traversal stack hold 27-bit primitive slots) are refused with
    PT_ERR_UNSUPPORTED before anything is allocated on the device; the same
    mesh under fewer instances uploads."""
    n = 1 << 20
    rng = np.random.default_rng(3)
    tris = rng.uniform(-1, 1, (n, 1, 3)) + rng.uniform(-0.01, 0.01, (n, 3, 3))
    s = bare_scene()
    m = s.add_mesh(scenes.Mesh(tris.reshape(-1, 3).astype(np.float32), np.arange(3 * n, dtype=np.uint32).reshape(n, 3)))
    for _ in range(abi.MAX_PRIMITIVES // n + 1):
        s.add_instance(abi.SHAPE_MESH, m, 0)
    with pytest.raises(abi.PtError) as e:
        GpuScene(cuda_ctx, s)
    assert e.value.status == abi.PT_ERR_UNSUPPORTED and str(abi.MAX_PRIMITIVES) in str(e.value)
    s.instances = s.instances[:2]
    g = GpuScene(cuda_ctx, s)
    assert g.bvh_stats().num_nodes > 0
    g.close()


def test_oversized_films_and_waves_are_refused(cuda_ctx):
    """Path slots and pixel indices are 32-bit: a film of 2^31 pixels or more
    is refused at upload, a wave of 2^31 path slots or more (frames x pixels)
    at render time, both before any device allocation."""
    s = bare_scene(env=(0.5, 0.5, 0.5))
    s.width, s.height = 65536, 32768
    with pytest.raises(abi.PtError) as e:
        GpuScene(cuda_ctx, s)
    assert e.value.status == abi.PT_ERR_UNSUPPORTED and "2^31" in str(e.value)
    g = GpuScene(cuda_ctx, bare_scene(64, 64, env=(0.5, 0.5, 0.5)))
    frames = (1 << 31) // (64 * 64)
    with pytest.raises(abi.PtError) as e:
        g.render(frames, wave_spp=frames)
    assert "2^31 - 1 path slots" in str(e.value)
    out = g.render(4, wave_spp=2)["accum"].cpu().numpy()
    assert np.allclose(out[:, :3], 0.5)
    g.close()
