"""Curve (hair) primitives on the GPU against the oracle: the four curve
types (linear, quadratic and cubic B-spline, Catmull-Rom), tapered and
constant radii, under an instance transform.

* traversal: closest-hit ids, distances and curve parameters bit-identical
  to the oracle's brute force (same round-cone pieces, same explicitly
  rounded FP32 arithmetic), any hit identical, for BVH widths 2, 4, 8;
* whole path: same-stream renders agree per pixel (as for triangle scenes),
  the normal AOV (the reference's SurfaceNormal at the primary hit) matches;
* the image does not depend on the BVH width, and a curve scene rendered in
  a multi-scene launch equals its serial render."""
import numpy as np
import pytest
import torch

import oracle
from pupiloptixlab_gb300 import abi, scenes
from pupiloptixlab_gb300.api import GpuScene, render_batch
from _parity import assert_bit_identical

pytestmark = pytest.mark.gpu

TYPES = [abi.CURVE_LINEAR, abi.CURVE_QUADRATIC_BSPLINE, abi.CURVE_CUBIC_BSPLINE, abi.CURVE_CATMULL_ROM]


def random_rays(rng, n, center, half, tmax=1e16):
    o = rng.uniform(-1, 1, (n, 3)) * half + center
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = o, 1e-3, d, tmax
    return r


def gpu_trace(g, rays, anyhit=False):
    return g.trace(torch.from_numpy(np.ascontiguousarray(rays)).cuda(), anyhit=anyhit).cpu().numpy()


@pytest.mark.parametrize("ctype", TYPES)
@pytest.mark.parametrize("width", [2, 4, 8])
def test_trace_matches_brute_force(cuda_ctx, ctype, width):
    sc = scenes.hair_scene(64, 48, curve_type=ctype, num_strands=300, tapered=(ctype % 2 == 1))
    o = oracle.OracleScene(sc, bvh=False)
    g = GpuScene(cuda_ctx, sc, bvh_width=width)
    assert g.num_curves() == o.num_curves()
    rng = np.random.default_rng(ctype * 10 + width)
    rays = np.concatenate([o.camera_rays(abi.RNG_PCG32, 0), random_rays(rng, 30000, (0, 1.6, 0), (1.8, 1.2, 1.8))])
    got, ref = gpu_trace(g, rays), o.trace(rays, brute_force=True)
    gid, rid = got[:, 1].view(np.int32), ref[:, 1].view(np.int32)
    bad = np.nonzero(gid != rid)[0]
    assert bad.size == 0, f"{bad.size} id mismatches, first {bad[:5]}: gpu {gid[bad[:5]]} ref {rid[bad[:5]]}"
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), "t/u differ"
    nt, ns = o.num_prims()
    assert (gid >= nt + ns).sum() > 1000, "too few curve hits"
    rays[:, 7] = rng.uniform(0.02, 4.0, rays.shape[0])
    assert np.array_equal(gpu_trace(g, rays, anyhit=True)[:, 0], o.trace(rays, anyhit=True, brute_force=True)[:, 0])
    g.close()


@pytest.mark.parametrize("ctype", TYPES)
def test_same_stream_render(cuda_ctx, ctype):
    sc = scenes.hair_scene(64, 48, curve_type=ctype, num_strands=400, tapered=ctype == abi.CURVE_CUBIC_BSPLINE)
    o = oracle.OracleScene(sc)
    g = GpuScene(cuda_ctx, sc)
    p = abi.RenderParams(spp=4, max_depth=0, seed=5, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32)
    ref = o.render(p)
    got = {k: v.cpu().numpy() for k, v in g.render(4, seed=5).items()}
    torch.cuda.synchronize()
    assert np.isfinite(got["accum"]).all()
    assert_bit_identical(f"hair type {ctype}", got["accum"], ref["accum"])
    assert np.array_equal(got["albedo"], ref["albedo"])
    assert np.array_equal(got["normal"].view(np.uint32), ref["normal"].view(np.uint32))
    # the primary hits of some pixels are curves
    rays = o.camera_rays(abi.RNG_PCG32, 5 + 3)
    nt, ns = o.num_prims()
    assert (o.trace(rays)[:, 1].view(np.int32) >= nt + ns).sum() > 100
    g.close()


def test_bvh_width_does_not_change_the_image(cuda_ctx):
    sc = scenes.hair_scene(48, 36, curve_type=abi.CURVE_CATMULL_ROM, num_strands=300)
    imgs = []
    for w in (2, 4, 8):
        g = GpuScene(cuda_ctx, sc, bvh_width=w)
        imgs.append(g.render(8, seed=2)["accum"].cpu().numpy())
        g.close()
    for im in imgs[1:]:
        assert np.array_equal(im.view(np.uint32), imgs[0].view(np.uint32))


def test_curves_in_a_multi_scene_launch(cuda_ctx):
    a = GpuScene(cuda_ctx, scenes.hair_scene(40, 30, curve_type=abi.CURVE_CUBIC_BSPLINE, num_strands=250))
    b = GpuScene(cuda_ctx, scenes.material_spheres(48, 32))
    c = GpuScene(cuda_ctx, scenes.hair_scene(32, 24, curve_type=abi.CURVE_LINEAR, num_strands=150, seed=3))
    serial = [g.render(6, seed=4)["accum"].cpu().numpy() for g in (a, b, c)]
    batch = [o["accum"].cpu().numpy() for o in render_batch(cuda_ctx, [a, b, c], 6, seed=4)]
    for s_, b_ in zip(serial, batch):
        assert np.array_equal(s_.view(np.uint32), b_.view(np.uint32))
    for g in (a, b, c):
        g.close()


def test_invalid_curves_are_rejected(cuda_ctx):
    sc = scenes.hair_scene(16, 16, num_strands=4)
    sc.curves[0].segments[-1] = sc.curves[0].positions.shape[0]  # control points past the end
    with pytest.raises(abi.PtError):
        GpuScene(cuda_ctx, sc)
    sc = scenes.hair_scene(16, 16, num_strands=4)
    sc.curves[0].radii[3] = -0.1
    with pytest.raises(abi.PtError):
        GpuScene(cuda_ctx, sc)
    sc = scenes.hair_scene(16, 16, num_strands=4)
    inst = [i for i in sc.instances if i["shape_type"] == abi.SHAPE_CURVES][0]
    inst["radiance"] = (1.0, 1.0, 1.0)
    with pytest.raises(abi.PtError):
        GpuScene(cuda_ctx, sc)
