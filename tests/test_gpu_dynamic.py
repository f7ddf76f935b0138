"""Animated vertices: pt_scene_update_all_vertices + refit / rebuild.  Hits
after either must equal brute force on the moved geometry, bit for bit."""
import copy

import numpy as np
import pytest
import torch

import oracle
from pupiloptixlab_gb300 import abi, scenes
from pupiloptixlab_gb300.api import GpuScene
from _parity import assert_bit_identical

pytestmark = pytest.mark.gpu


def jittered(sc, sigma, seed):
    rng = np.random.default_rng(seed)
    out = copy.copy(sc)
    out.meshes = [scenes.Mesh(m.positions + rng.normal(0.0, sigma, m.positions.shape).astype(np.float32), m.indices,
                              m.normals, m.texcoords) for m in sc.meshes]
    return out


def all_positions(sc):
    return np.concatenate([m.positions for m in sc.meshes]).astype(np.float32)


@pytest.mark.parametrize("on_device,width", [(True, 4), (False, 4), (True, 8)])
def test_update_refit_rebuild_match_brute_force(cuda_ctx, on_device, width):
    """Width 8: the refit recompresses the 8-wide nodes the traversal reads."""
    sc = scenes.icosphere_field(64, 36, num_instances=10, subdivisions=3)
    g = GpuScene(cuda_ctx, sc, bvh_width=width)
    sah0 = g.bvh_stats().sah_cost
    moved = jittered(sc, 0.02, 5)
    pos = all_positions(moved)
    g.update_all_vertices(torch.from_numpy(pos).cuda() if on_device else pos)
    o = oracle.OracleScene(moved, bvh=False)
    rays = o.camera_rays(abi.RNG_PCG32, 0)
    ref = o.trace(rays, brute_force=True)
    refit = g.refit()
    got = g.trace(torch.from_numpy(rays).cuda()).cpu().numpy()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert refit.sah_cost > 0 and refit.build_ms > 0
    rebuilt = g.build_bvh(width=width)
    got2 = g.trace(torch.from_numpy(rays).cuda()).cpu().numpy()
    assert np.array_equal(got2.view(np.uint32), ref.view(np.uint32))
    # refitting a small jitter keeps the tree close to a rebuild
    assert refit.sah_cost >= 0.9 * rebuilt.sah_cost
    assert abs(rebuilt.sah_cost - sah0) / sah0 < 0.2


def test_render_after_update_matches_oracle(cuda_ctx):
    sc = scenes.cornell_box(32, 32)
    g = GpuScene(cuda_ctx, sc)
    moved = jittered(sc, 0.01, 9)
    g.update_all_vertices(torch.from_numpy(all_positions(moved)).cuda())
    g.refit()
    out = g.render(4, seed=0, rng=abi.RNG_PCG32)
    torch.cuda.synchronize()
    got = out["accum"].cpu().numpy()
    ref = oracle.OracleScene(moved).render(abi.RenderParams(spp=4, seed=0, accumulate=1, rng=abi.RNG_PCG32))["accum"]
    assert_bit_identical("cornell after vertex update + refit", got, ref)
