"""Host-side checks of the oracle and the scene generators: the BVH2 used
for large scenes returns exactly the brute-force answer, random streams and
PCG32 match published values, the procedural scenes are deterministic."""
import numpy as np
import pytest

import oracle
from pupiloptixlab_gb300 import abi, scenes


def random_rays(rng, n, lo, hi, origin_box=None):
    o = rng.uniform(lo, hi, (n, 3)) if origin_box is None else rng.uniform(*origin_box, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = 1e-4
    r[:, 4:7] = d
    r[:, 7] = 1e16
    return r


def test_pcg32_published_values():
    # pcg32-demo (pcg-random.org): pcg32_srandom(42, 54), first six outputs
    want = [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]
    assert list(oracle.pcg32_raw(42, 54, 6)) == want


def test_pcg32_float_stream_is_top_24_bits():
    raw = oracle.pcg32_raw(123, 7, 32)
    f = oracle.rng_stream(1, 123, 7, 32)
    assert np.array_equal(f, (raw >> 8).astype(np.float32) / np.float32(16777216.0))


@pytest.mark.parametrize("make", [lambda: scenes.cornell_box(32, 32),
                                  lambda: scenes.material_spheres(32, 24)])
def test_bvh2_equals_brute_force(ptlib, make):
    sc = make()
    o = oracle.OracleScene(sc, bvh=True)
    rng = np.random.default_rng(5)
    rays = random_rays(rng, 4000, -2.0, 2.0)
    rays[:, 1] += 1.0
    cam = o.camera_rays(abi.RNG_PCG32, 3)
    rays = np.concatenate([rays, cam])
    a = o.trace(rays, brute_force=True)
    b = o.trace(rays, brute_force=False)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert (a[:, 1].view(np.int32) >= 0).mean() > 0.3
    sa = o.trace(rays, anyhit=True, brute_force=True)
    sb = o.trace(rays, anyhit=True, brute_force=False)
    assert np.array_equal(sa[:, 0], sb[:, 0])


def test_bvh2_equals_brute_force_on_icosphere_field(ptlib):
    sc = scenes.icosphere_field(64, 36, num_instances=6, subdivisions=2)
    o = oracle.OracleScene(sc, bvh=True)
    rng = np.random.default_rng(9)
    rays = random_rays(rng, 1500, -12.0, 12.0)
    rays[:, 1] += 10.0
    rays = np.concatenate([rays, o.camera_rays(abi.RNG_REF_LCG, 0)])
    a = o.trace(rays, brute_force=True)
    b = o.trace(rays, brute_force=False)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_procedural_scenes_are_deterministic(ptlib):
    a = scenes.icosphere_field(32, 18, num_instances=4, subdivisions=2, seed=3)
    b = scenes.icosphere_field(32, 18, num_instances=4, subdivisions=2, seed=3)
    for ma, mb in zip(a.meshes, b.meshes):
        assert np.array_equal(ma.positions, mb.positions) and np.array_equal(ma.indices, mb.indices)
    full = scenes.icosphere(4)
    assert full[1].shape[0] == 5120


def test_cornell_box_layout(ptlib):
    sc = scenes.cornell_box()
    assert sc.num_triangles == 10 + 24 + 2
    o = oracle.OracleScene(sc)
    table = o.emitter_table()
    assert table.shape[0] == 2  # the light quad's two triangles, no environment
    assert np.allclose(table[:, 1].sum(), 1.0, atol=1e-6)


def test_oracle_render_is_energy_plausible(ptlib):
    sc = scenes.cornell_box(24, 24)
    o = oracle.OracleScene(sc)
    p = abi.RenderParams(spp=8, max_depth=0, seed=0, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32)
    out = o.render(p)
    img = out["accum"][:, :3]
    assert np.isfinite(img).all() and img.min() >= 0
    assert 0.01 < img.mean() < 5.0  # a 0.25 x 0.25 light over a 2 x 2 box: mean about 0.05
    assert np.all(out["accum"][:, 3] == 1.0)


def test_accumulation_equals_frame_by_frame(ptlib):
    """spp frames in one call == spp calls of one frame with increasing seed
    and sample count (PTPass::OnRun, pt_pass.cpp:39-57)."""
    sc = scenes.cornell_box(12, 12)
    o = oracle.OracleScene(sc)
    one = o.render(abi.RenderParams(spp=4, seed=10, sample_cnt=0, accumulate=1, rng=abi.RNG_REF_LCG))["accum"]
    acc = np.zeros((144, 4), np.float32)
    for f in range(4):
        acc = o.render(abi.RenderParams(spp=1, seed=10 + f, sample_cnt=f, accumulate=1, rng=abi.RNG_REF_LCG),
                       accum=acc)["accum"]
    assert np.array_equal(one, acc)


def test_render_does_not_depend_on_threads_or_pixel_subsets(ptlib):
    """The CPU baseline renders strided pixel subsets on all host cores: every
    pixel's result is the same whatever the thread count, and a subset render
    writes exactly the full render's values at its pixels (and nothing else)."""
    import oracle
    from pupiloptixlab_gb300 import abi, scenes
    o = oracle.OracleScene(scenes.cornell_box(24, 16))
    p = abi.RenderParams(spp=2, max_depth=4, seed=3, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32)
    one = o.render(p, threads=1)
    many = o.render(p, threads=4)
    for k in one:
        assert np.array_equal(one[k].view(np.uint32), many[k].view(np.uint32)), k
    px = np.arange(5, 24 * 16, 7, dtype=np.uint32)
    sub = o.render(p, pixels=px, threads=3)
    assert np.array_equal(sub["accum"][px].view(np.uint32), one["accum"][px].view(np.uint32))
    rest = np.setdiff1d(np.arange(24 * 16), px)
    assert not sub["accum"][rest].any()
