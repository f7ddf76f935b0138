"""Traversal parity: pt_trace_rays (closest and any hit, BVH widths 2/4/8 --
8 as compressed nodes -- with and without top levels in shared memory,
origins inside and far outside the scene) against the oracle's
brute-force intersector.  Hit primitive ids, distances and barycentrics must
be bit-identical: both sides run the same watertight triangle test with
explicitly rounded FP32 operations and the (t, id) tie-break."""
import numpy as np
import pytest
import torch

import oracle
from pupiloptixlab_gb300 import abi, scenes
from pupiloptixlab_gb300.api import GpuScene

pytestmark = pytest.mark.gpu


def rays_inside(rng, n, center, half, tmax=1e16):
    o = rng.uniform(-1, 1, (n, 3)) * half + center
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = o, 1e-3, d, tmax
    return r


def gpu_trace(g, rays, anyhit=False):
    return g.trace(torch.from_numpy(np.ascontiguousarray(rays)).cuda(), anyhit=anyhit).cpu().numpy()


def assert_hits_equal(got, ref):
    gid, rid = got[:, 1].view(np.int32), ref[:, 1].view(np.int32)
    bad = np.nonzero(gid != rid)[0]
    assert bad.size == 0, f"{bad.size} prim id mismatches, first {bad[:5]}: gpu {gid[bad[:5]]} ref {rid[bad[:5]]}"
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), "t/u/v differ"


@pytest.mark.parametrize("width", [2, 4, 8])
@pytest.mark.parametrize("smem_nodes", [0, 21])
def test_cornell_primary_and_random_rays(cuda_ctx, width, smem_nodes):
    sc = scenes.cornell_box(64, 64)
    o = oracle.OracleScene(sc, bvh=False)
    g = GpuScene(cuda_ctx, sc, bvh_width=width, max_leaf=2, smem_nodes=smem_nodes)
    rng = np.random.default_rng(width)
    rays = np.concatenate([o.camera_rays(abi.RNG_PCG32, 0), o.camera_rays(abi.RNG_REF_LCG, 5),
                           rays_inside(rng, 20000, (0, 1, 0), (0.99, 0.99, 0.99))])
    assert_hits_equal(gpu_trace(g, rays), o.trace(rays, brute_force=True))


@pytest.mark.parametrize("width", [2, 4, 8])
def test_any_hit_matches_brute_force(cuda_ctx, width):
    sc = scenes.material_spheres(48, 32)
    o = oracle.OracleScene(sc, bvh=False)
    g = GpuScene(cuda_ctx, sc, bvh_width=width)
    rng = np.random.default_rng(11)
    rays = rays_inside(rng, 30000, (0, 2, 0), (7, 2, 3))
    rays[:, 7] = rng.uniform(0.01, 12.0, rays.shape[0])  # bounded shadow segments
    got = gpu_trace(g, rays, anyhit=True)
    ref = o.trace(rays, anyhit=True, brute_force=True)
    assert np.array_equal(got[:, 0], ref[:, 0])
    assert 0.05 < got[:, 0].mean() < 0.95


def test_spheres_and_meshes_closest_hit(cuda_ctx):
    sc = scenes.material_spheres(96, 64)
    o = oracle.OracleScene(sc, bvh=False)
    g = GpuScene(cuda_ctx, sc, bvh_width=4)
    rng = np.random.default_rng(3)
    rays = np.concatenate([o.camera_rays(abi.RNG_PCG32, 1), rays_inside(rng, 20000, (0, 2, 0), (7, 3, 4))])
    got = gpu_trace(g, rays)
    ref = o.trace(rays, brute_force=True)
    assert_hits_equal(got, ref)
    nt, ns = o.num_prims()
    assert (got[:, 1].view(np.int32) >= nt).any(), "no sphere was hit"


@pytest.mark.parametrize("max_leaf", [1, 4, 8, 15])
def test_leaf_sizes(cuda_ctx, max_leaf):
    sc = scenes.icosphere_field(64, 36, num_instances=12, subdivisions=3)
    o = oracle.OracleScene(sc, bvh=False)
    g = GpuScene(cuda_ctx, sc, bvh_width=4, max_leaf=max_leaf)
    rays = o.camera_rays(abi.RNG_PCG32, 0)
    assert_hits_equal(gpu_trace(g, rays), o.trace(rays, brute_force=True))


@pytest.mark.parametrize("width", [2, 4, 8])
@pytest.mark.parametrize("fast_build", [False, True])
def test_both_tree_builders(cuda_ctx, width, fast_build):
    """PLOC clustering and the radix tree (PT_BVH_FAST_BUILD) give the same
    hits for every width; the stats name the builder that ran."""
    sc = scenes.icosphere_field(48, 32, num_instances=20, subdivisions=3, seed=5)
    o = oracle.OracleScene(sc, bvh=False)
    g = GpuScene(cuda_ctx, sc, bvh_width=width, bvh_flags=abi.BVH_FAST_BUILD if fast_build else 0)
    st = g.bvh_stats()
    if fast_build:
        assert st.builder == abi.BVH_BUILDER_RADIX
    elif width < 8:  # a PLOC BVH8 deeper than the stack covers falls back to the radix tree
        assert st.builder == abi.BVH_BUILDER_PLOC
    rng = np.random.default_rng(width + 10 * fast_build)
    rays = np.concatenate([o.camera_rays(abi.RNG_PCG32, 0), rays_inside(rng, 10000, (0, 1, 0), (8, 2, 5))])
    assert_hits_equal(gpu_trace(g, rays), o.trace(rays, brute_force=True))
    rays[:, 7] = rng.uniform(0.05, 6.0, rays.shape[0])
    assert np.array_equal(gpu_trace(g, rays, anyhit=True)[:, 0], o.trace(rays, anyhit=True, brute_force=True)[:, 0])
    g.close()


@pytest.mark.parametrize("width", [2, 4, 8])
def test_far_origins(cuda_ctx, width):
    """Origins far outside the scene's magnitude, where the traversal leaves
    the padded fused-multiply-add slab form for the rounded-difference one
    (for compressed 8-wide nodes: each bound decoded as in the build)."""
    sc = scenes.cornell_box(16, 16)
    o = oracle.OracleScene(sc, bvh=False)
    g = GpuScene(cuda_ctx, sc, bvh_width=width)
    rng = np.random.default_rng(40 + width)
    target = rays_inside(rng, 20000, (0, 1, 0), (0.9, 0.9, 0.9))
    d = rng.normal(size=(target.shape[0], 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dist = rng.uniform(50.0, 5e3, (target.shape[0], 1))
    rays = target.copy()
    rays[:, 0:3] = target[:, 0:3] - d * dist
    rays[:, 4:7] = d
    assert_hits_equal(gpu_trace(g, rays), o.trace(rays, brute_force=True))
    assert (gpu_trace(g, rays)[:, 1].view(np.int32) >= 0).mean() > 0.5


@pytest.mark.parametrize("width", [4, 8])
def test_full_size_scene_primary_rays(cuda_ctx, width):
    """Icosphere-field geometry (1,032,192 triangles + 4 spheres) at 1920x1080:
    every 16th primary ray against the oracle's BVH2 (itself equal to brute
    force, tests/test_oracle_host.py) and 192 rays against brute force."""
    sc = scenes.icosphere_field()
    o = oracle.OracleScene(sc, bvh=True)
    g = GpuScene(cuda_ctx, sc, bvh_width=width)
    st = g.bvh_stats()
    assert st.num_prims == 1032196 and st.num_nodes > 1000
    rays = o.camera_rays(abi.RNG_PCG32, 0)[::16]
    got = gpu_trace(g, rays)
    assert_hits_equal(got, o.trace(rays))
    few = rays[:: max(1, rays.shape[0] // 192)][:192]
    assert_hits_equal(gpu_trace(g, few), o.trace(few, brute_force=True))


def test_empty_and_degenerate_inputs(cuda_ctx):
    sc = scenes.cornell_box(8, 8)
    g = GpuScene(cuda_ctx, sc)
    empty = torch.zeros(0, 8, device="cuda")
    assert g.trace(empty).shape == (0, 4)
    r = np.zeros((3, 8), np.float32)
    r[0, 4:7] = (0, 1, 0)   # from the origin straight up: hits the ceiling
    r[0, 7] = 1e16
    r[1, 4:7] = (0, 1, 0)   # same ray, tmax before the ceiling: miss
    r[1, 7] = 1.0
    r[2, 4:7] = (1, 0, 0)   # along the floor plane (parallel to two walls' slabs)
    r[2, 0:3] = (0, 1e-3, 0)
    r[2, 7] = 1e16
    for row in r:
        row[3] = 1e-4
    o = oracle.OracleScene(sc, bvh=False)
    assert_hits_equal(gpu_trace(g, r), o.trace(r, brute_force=True))
