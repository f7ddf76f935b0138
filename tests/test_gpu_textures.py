"""Bitmap textures (cuda::Texture, framework/cuda/texture.h:33-57, as a float4
CUDA texture object) and the importance-sampled environment map
(EnvMapEmitter, framework/render/emitter/env.h) on the GPU against the oracle.

The kernels fetch texels through the texture unit; the oracle restates the
fetch on the CPU (oracle/tex_fetch.h).  The two agree to a few units in the
last place of the filter weights, so paths that read a texture are compared
with a tolerance: same random streams, >= 90 % of pixels within 1e-3
(relative) at 4 spp; converged images (512 spp, independent streams) differ
by no more than the noise between two GPU seeds, mean radiance within 1 %."""
import numpy as np
import pytest
import torch

import oracle
from pupiloptixlab_gb300 import abi, scenes
from pupiloptixlab_gb300.api import GpuScene

pytestmark = pytest.mark.gpu


def textured_scene(width=48, height=32, env_map=True, filter=abi.TEX_FILTER_LINEAR, address=abi.TEX_ADDRESS_WRAP):
    rng = np.random.default_rng(5)
    s = scenes.Scene(width, height, 5, name="textured")
    tex = rng.uniform(0.05, 0.9, (16, 24, 4)).astype(np.float32)
    tex[..., 3] = 1.0
    floor = s.add_material(scenes.diffuse(0.5))
    s.materials[floor].tex[0] = scenes.bitmap(tex, address=address, filter=filter, uv_scale=3.0)
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(scenes.grid(4, 4, 6.0, 0.0)), floor)
    base = scenes.icosphere(2)
    ball = s.add_mesh(scenes.displaced_icosphere(1, 0.0, 2, base))
    plastic = s.add_material(scenes.plastic((0.6, 0.3, 0.2), 1.5, 1.0))
    s.materials[plastic].tex[0] = scenes.bitmap(tex[::-1].copy(), filter=filter)
    s.add_instance(abi.SHAPE_MESH, ball, plastic, scenes.translate(-1.0, 1.0, 0.0))
    s.add_instance(abi.SHAPE_MESH, ball, s.add_material(scenes.rough_conductor(0.2)), scenes.translate(1.2, 1.0, 0.5))
    if env_map:
        env = rng.uniform(0.1, 0.6, (24, 48, 4)).astype(np.float32)
        env[4:7, 30:34, :3] = [[20.0, 16.0, 12.0]]
        env[..., 3] = 1.0
        s.env = scenes.EnvMap(env, scale=1.2, to_world=scenes.rotate_y(40.0))
    else:
        s.env = (0.4, 0.45, 0.5)
        light = s.add_material(scenes.diffuse(0.0))
        s.add_instance(abi.SHAPE_SPHERE, s.add_sphere((0.0, 0.0, 0.0), 0.5), light, scenes.translate(0.0, 4.0, 1.0),
                       radiance=(10.0, 9.0, 8.0))
    s.camera = scenes.camera(40.0, width / height, scenes.look_at_to_world((0.0, 3.0, 7.0), (0.0, 0.8, 0.0)))
    return s


def _close(a, b, rel=1e-3):
    return np.all(np.abs(a - b) <= rel * np.maximum(1.0, np.abs(b)), axis=1)


@pytest.mark.parametrize("env_map,filter", [(True, abi.TEX_FILTER_LINEAR), (False, abi.TEX_FILTER_POINT),
                                            (False, abi.TEX_FILTER_LINEAR)])
def test_same_stream_agreement(cuda_ctx, env_map, filter):
    sc = textured_scene(env_map=env_map, filter=filter)
    o = oracle.OracleScene(sc)
    g = GpuScene(cuda_ctx, sc)
    p = abi.RenderParams(spp=4, max_depth=0, seed=3, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32)
    ref = o.render(p)
    got = g.render(4, seed=3)
    torch.cuda.synchronize()
    acc = got["accum"].cpu().numpy()[:, :3]
    assert np.isfinite(acc).all()
    ok = _close(acc, ref["accum"][:, :3])
    assert ok.mean() >= 0.90, ok.mean()
    # the albedo AOV reads the bitmap at the primary hit
    alb = got["albedo"].cpu().numpy()
    assert _close(alb, ref["albedo"], 2e-3).mean() >= 0.97
    g.close()


def test_converged_env_map_render(cuda_ctx):
    """Independent random streams: the GPU-oracle difference must look like
    the noise between two GPU renders with different seeds, and the mean
    radiance must agree to 1 % (no bias)."""
    sc = textured_scene(env_map=True)
    o = oracle.OracleScene(sc)
    g = GpuScene(cuda_ctx, sc)
    p = abi.RenderParams(spp=512, max_depth=0, seed=100, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32)
    ref = o.render(p)["accum"][:, :3].astype(np.float64)
    a = g.render(512, seed=7)["accum"].cpu().numpy()[:, :3].astype(np.float64)
    b = g.render(512, seed=20000)["accum"].cpu().numpy()[:, :3].astype(np.float64)
    noise = float(np.sqrt(np.mean((a - b) ** 2)))
    err = float(np.sqrt(np.mean((a - ref) ** 2)))
    assert err <= 1.3 * noise + 1e-4, (err, noise)
    assert abs(a.mean() - ref.mean()) <= 0.01 * ref.mean()
    g.close()


def test_env_map_rejects_bad_input(cuda_ctx):
    sc = textured_scene(env_map=True)
    sc.env = scenes.EnvMap(np.zeros((1, 8, 4), np.float32))
    with pytest.raises(abi.PtError):
        GpuScene(cuda_ctx, sc)


def test_textured_area_emitters(cuda_ctx):
    """Area emitters whose radiance is a texture (checkerboard on a quad and a
    sphere, and a bitmap on a sphere; framework/render/emitter/area.h:17-45,
    sphere.h:14-42): NEE samples read the texture at the sampled point's
    texture coordinates, hits read it at the hit's, selection weights follow
    GetWeight.  Without the bitmap light the image is bit-identical to the
    oracle; with it, within the texture-fetch tolerance above."""
    from _parity import assert_bit_identical

    import test_oracle_emitters_cpu as te
    s, _ = te.emitter_scene(48, 32)
    s.instances[2]["radiance"] = scenes.checkerboard((6.0, 1.0, 1.0), (1.0, 1.0, 6.0), uv_scale=3.0)  # the bitmap light
    p = abi.RenderParams(spp=4, max_depth=0, seed=3, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32)
    for rng in (abi.RNG_PCG32, abi.RNG_REF_LCG):
        p.rng = rng
        ref = oracle.OracleScene(s).render(p)
        g = GpuScene(cuda_ctx, s)
        got = g.render(4, seed=3, rng=rng)
        torch.cuda.synchronize()
        assert_bit_identical(f"checkerboard lights rng {rng}", got["accum"].cpu().numpy(), ref["accum"])
        g.close()
    s, _ = te.emitter_scene(48, 32)  # with the bitmap sphere light
    ref = oracle.OracleScene(s).render(p)
    g = GpuScene(cuda_ctx, s)
    acc = g.render(4, seed=3, rng=p.rng)["accum"].cpu().numpy()[:, :3]
    assert np.isfinite(acc).all() and acc.mean() > 0.01
    ok = _close(acc, ref["accum"][:, :3])
    assert ok.mean() >= 0.90, ok.mean()
    g.close()
