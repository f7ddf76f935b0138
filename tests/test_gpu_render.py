"""Whole-path parity: pt_render against the oracle's restatement of the
reference integrator (example/path_tracer/main.cu:38-197) on identical
scenes, seeds and per-pixel random streams (reference LCG and PCG32).

* same-stream check: with identical random numbers every pixel is
  bit-identical (shared trigonometry, no FMA contraction on either side);
* converged check: 4096-spp images agree within RMSE 1e-3;
* invariances that must hold bit for bit on the GPU: BVH width, wave size,
  splitting one call into several calls with continuing sample counts."""
import numpy as np
import pytest
import torch

import oracle
from pupiloptixlab_gb300 import abi, scenes
from pupiloptixlab_gb300.api import GpuScene
from _parity import assert_bit_identical

pytestmark = pytest.mark.gpu


def params(spp, seed=0, cnt=0, rng=abi.RNG_PCG32, accumulate=1, max_depth=0):
    return abi.RenderParams(spp=spp, max_depth=max_depth, seed=seed, sample_cnt=cnt, accumulate=accumulate, rng=rng)


def gpu_render(g, spp, **kw):
    out = g.render(spp, **kw)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def rmse(a, b):
    return float(np.sqrt(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)))


@pytest.mark.parametrize("rng", [abi.RNG_REF_LCG, abi.RNG_PCG32])
@pytest.mark.parametrize("make", [lambda: scenes.cornell_box(48, 48), lambda: scenes.material_spheres(64, 40)],
                         ids=["cornell", "materials"])
def test_same_stream_per_pixel(cuda_ctx, rng, make):
    sc = make()
    o = oracle.OracleScene(sc)
    g = GpuScene(cuda_ctx, sc)
    spp = 4
    ref = o.render(params(spp, seed=3, rng=rng))
    got = gpu_render(g, spp, seed=3, rng=rng)
    assert_bit_identical(f"{sc.name} {rng}", got["accum"], ref["accum"])
    assert np.all(got["accum"][:, 3] == 1.0)
    # AOVs of the last frame
    for k in ("frame", "albedo", "normal", "test"):
        assert np.array_equal(got[k].view(np.uint32), ref[k].view(np.uint32)), k


@pytest.mark.parametrize("make,spp", [(lambda: scenes.cornell_box(40, 40), 4096),
                                      (lambda: scenes.material_spheres(48, 32), 4096)],
                         ids=["cornell", "materials"])
def test_converged_rmse(cuda_ctx, make, spp):
    sc = make()
    o = oracle.OracleScene(sc)
    g = GpuScene(cuda_ctx, sc)
    ref = o.render(params(spp, rng=abi.RNG_PCG32))["accum"][:, :3]
    got = gpu_render(g, spp, rng=abi.RNG_PCG32)["accum"][:, :3]
    assert np.isfinite(got).all()
    assert rmse(got, ref) <= 1e-3, rmse(got, ref)


def test_bvh_width_and_wave_size_do_not_change_the_image(cuda_ctx):
    sc = scenes.material_spheres(40, 24)
    imgs = []
    for width, wave in ((2, 0), (4, 0), (8, 0), (4, 1), (4, 3)):
        g = GpuScene(cuda_ctx, sc, bvh_width=width)
        imgs.append(gpu_render(g, 7, seed=1, wave_spp=wave)["accum"])
    for im in imgs[1:]:
        assert np.array_equal(im.view(np.uint32), imgs[0].view(np.uint32))


def test_split_calls_equal_one_call(cuda_ctx):
    """PTPass::OnRun accumulates one frame per call (pt_pass.cpp:39-57)."""
    sc = scenes.cornell_box(24, 24)
    g = GpuScene(cuda_ctx, sc)
    one = gpu_render(g, 6, seed=20, rng=abi.RNG_REF_LCG)["accum"]
    buf = g.alloc_buffers()
    for f in range(0, 6, 2):
        g.render(2, seed=20 + f, sample_cnt=f, rng=abi.RNG_REF_LCG, buffers=buf)
    torch.cuda.synchronize()
    assert np.array_equal(buf["accum"].cpu().numpy(), one)


def test_no_accumulation_and_depth_override(cuda_ctx):
    sc = scenes.cornell_box(16, 16)
    o = oracle.OracleScene(sc)
    g = GpuScene(cuda_ctx, sc)
    for md in (1, 2, 3):
        ref = o.render(params(3, seed=9, accumulate=0, max_depth=md, rng=abi.RNG_REF_LCG))["accum"]
        got = gpu_render(g, 3, seed=9, accumulate=False, max_depth=md, rng=abi.RNG_REF_LCG)["accum"]
        assert_bit_identical(f"no accumulation, depth {md}", got, ref)


def test_icosphere_field_reduced(cuda_ctx):
    """The icosphere-field scene (all 7 materials, env + sphere lights, depth 8) at
    reduced resolution: bit-identical to the oracle, and counters."""
    sc = scenes.icosphere_field(96, 54)
    o = oracle.OracleScene(sc)
    g = GpuScene(cuda_ctx, sc)
    ref = o.render(params(8, seed=0))["accum"]
    got = gpu_render(g, 8, seed=0, flags=abi.RENDER_COUNTERS)["accum"]
    assert_bit_identical("icosphere field 96x54 8 spp", got, ref)
    st = g.render_stats()
    assert st.samples == 96 * 54 * 8
    assert st.extension_rays >= st.samples
    assert st.nodes_visited > st.extension_rays
    assert st.overflow == 0


def test_material_sort_and_graph_do_not_change_the_image(cuda_ctx):
    """Binning hits by material and CUDA-graph replay only reorder work; dropping
    non-finite samples changes nothing in an image that has none."""
    sc = scenes.material_spheres(48, 32)
    g = GpuScene(cuda_ctx, sc)
    ref = gpu_render(g, 5, seed=2, flags=abi.RENDER_NO_GRAPH)["accum"]
    for flags in (0, abi.RENDER_NO_MATERIAL_SORT, abi.RENDER_NO_MATERIAL_SORT | abi.RENDER_NO_GRAPH,
                  abi.RENDER_KERNEL_TIMING | abi.RENDER_COUNTERS, abi.RENDER_DROP_NONFINITE):
        got = gpu_render(g, 5, seed=2, flags=flags)["accum"]
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), flags
    # the instantiated graph is updated in place by later calls with other parameters
    a = gpu_render(g, 3, seed=7)["accum"]
    b = gpu_render(g, 3, seed=7, flags=abi.RENDER_NO_GRAPH)["accum"]
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_autotune_picks_a_configuration_and_keeps_the_image(cuda_ctx):
    sc = scenes.material_spheres(64, 40)
    g = GpuScene(cuda_ctx, sc)
    before = gpu_render(g, 4, seed=1)["accum"]
    r = g.autotune(spp=2)
    assert r.bvh_width in (2, 4, 8) and r.block_size in (64, 128, 256)
    assert r.wave_paths in (16 << 20, 32 << 20, 64 << 20, 128 << 20)
    assert r.trials >= 10 and r.msamples_per_s > 0
    assert g.bvh_stats().width == r.bvh_width
    after = gpu_render(g, 4, seed=1)["accum"]
    assert np.array_equal(after.view(np.uint32), before.view(np.uint32))


def test_nonfinite_samples_are_counted_dropped_or_reported(cuda_ctx):
    """A material whose reflectance is NaN poisons the paths that bounce off
    it: the samples are counted, PT_RENDER_DROP_NONFINITE accumulates them as
    zero, PT_RENDER_CHECK_FINITE turns the render into PT_ERR_NAN."""
    sc = scenes.cornell_box(24, 24)
    sc.materials[0].tex[0].color0[:] = [float("nan")] * 3
    g = GpuScene(cuda_ctx, sc)
    out = gpu_render(g, 2, seed=1)
    st = g.render_stats()
    assert st.nonfinite_samples > 0 and not np.isfinite(out["accum"]).all()
    out = gpu_render(g, 2, seed=1, flags=abi.RENDER_DROP_NONFINITE)
    assert g.render_stats().nonfinite_samples == st.nonfinite_samples
    assert np.isfinite(out["accum"]).all()
    with pytest.raises(abi.PtError) as e:
        g.render(2, seed=1, flags=abi.RENDER_CHECK_FINITE)
    assert e.value.status == 5 and "PT_ERR_NAN" in str(e.value)
    g.close()
    clean = GpuScene(cuda_ctx, scenes.cornell_box(24, 24))
    gpu_render(clean, 2, seed=1, flags=abi.RENDER_CHECK_FINITE)
    assert clean.render_stats().nonfinite_samples == 0
    clean.close()
