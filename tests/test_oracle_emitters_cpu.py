"""Textured area-emitter radiance in the oracle (AreaEmitter with a
checkerboard or bitmap radiance texture, framework/render/emitter/area.h:17-45,
sphere.h:14-42): the selection weights follow GetWeight
(framework/world/emitter.cpp:77-101), restated here in numpy, and a textured
light renders finite, non-black images whose brightness follows the
texture."""
import numpy as np

import oracle
from pupiloptixlab_gb300 import abi, scenes


def get_weight(kind, c0=None, c1=None, px=None):
    """GetWeight of the reference: max channel of an RGB value; the mean of the
    two patches' max channels; for a bitmap, pixels i * w + j for i < w, j < h
    (the last pixel where that runs past the array), max channel, mean."""
    mx = lambda v: (v[0] if v[0] > v[2] else v[2]) if v[0] > v[1] else (v[1] if v[1] > v[2] else v[2])  # noqa: E731
    if kind == "rgb":
        return np.float32(mx(c0))
    if kind == "checker":
        return np.float32((np.float32(mx(c0)) + np.float32(mx(c1))) * np.float32(0.5))
    h, w = px.shape[:2]
    flat = px.reshape(-1, 4)
    s = np.float32(0.0)
    for i in range(w):
        for j in range(h):
            q = min(i * w + j, w * h - 1)
            s = np.float32(s + np.float32(mx(flat[q])))
    return np.float32(s / np.float32(np.float32(1.0) * w * h))


def emitter_scene(w=24, h=16):
    rng = np.random.default_rng(3)
    px = rng.uniform(0.0, 6.0, (6, 10, 4)).astype(np.float32)  # wider than high: the clamped read is used
    px[..., 3] = 1.0
    s = scenes.Scene(w, h, 4, name="textured_lights")
    floor = s.add_material(scenes.diffuse(0.6))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(scenes.grid(4, 4, 6.0, 0.0)), floor)
    black = s.add_material(scenes.diffuse(0.0))
    checker = scenes.checkerboard((9.0, 4.0, 2.0), (1.0, 2.0, 7.0), uv_scale=4.0)
    quad = scenes.quad((-0.5, 2.5, -0.5), (-0.5, 2.5, 0.5), (0.5, 2.5, 0.5), (0.5, 2.5, -0.5), (0, -1, 0))
    s.add_instance(abi.SHAPE_MESH, s.add_mesh(quad), black, radiance=checker)
    s.add_instance(abi.SHAPE_SPHERE, s.add_sphere((0.0, 0.0, 0.0), 0.4), black, scenes.translate(1.5, 1.5, 0.0),
                   radiance=scenes.bitmap(px))
    s.add_instance(abi.SHAPE_SPHERE, s.add_sphere((0.0, 0.0, 0.0), 0.3), black, scenes.translate(-1.5, 1.2, 0.5),
                   radiance=(3.0, 5.0, 4.0))
    s.camera = scenes.camera(45.0, w / h, scenes.look_at_to_world((0.0, 2.0, 6.0), (0.0, 1.0, 0.0)))
    return s, px


def test_selection_probabilities_follow_get_weight(ptlib):
    s, px = emitter_scene()
    o = oracle.OracleScene(s, bvh=False)
    table = o.emitter_table()
    assert table.shape[0] == 4  # two quad triangles, two spheres
    w_checker = get_weight("checker", (9.0, 4.0, 2.0), (1.0, 2.0, 7.0))
    w_bitmap = get_weight("bitmap", px=px)
    w_rgb = get_weight("rgb", (3.0, 5.0, 4.0))
    tri_area = np.float32(0.5)
    a1 = np.float32(4 * np.float32(np.pi) * np.float32(0.4) * np.float32(0.4))
    a2 = np.float32(4 * np.float32(np.pi) * np.float32(0.3) * np.float32(0.3))
    weights = np.array([w_checker * tri_area, w_checker * tri_area, w_bitmap * a1, w_rgb * a2], np.float64)
    expect = weights / weights.sum()
    assert np.allclose(table[:, 1], expect, rtol=2e-6, atol=0)
    # the bitmap's weight is not its plain mean (the reference's index arithmetic)
    assert abs(w_bitmap - px[..., :3].max(axis=2).mean()) > 1e-3


def test_textured_lights_render(ptlib):
    s, _ = emitter_scene()
    o = oracle.OracleScene(s, bvh=False)
    out = o.render(abi.RenderParams(spp=8, max_depth=0, seed=1, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32))
    img = out["accum"][:, :3]
    assert np.isfinite(img).all() and img.mean() > 0.01
    # a dimmer checkerboard on the quad light darkens the image
    s2, _ = emitter_scene()
    s2.instances[1]["radiance"] = scenes.checkerboard((0.1, 0.1, 0.1), (0.1, 0.1, 0.1), uv_scale=4.0)
    img2 = oracle.OracleScene(s2, bvh=False).render(
        abi.RenderParams(spp=8, max_depth=0, seed=1, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32))["accum"][:, :3]
    assert img2.mean() < img.mean()
