"""pt_render_batch: several scenes of different sizes, resolutions and
materials in one launch per bounce.  Every path keeps its scene-local pixel
index and random stream and every hit is decided by the exact primitive test,
so each scene's image must be bit-identical to rendering it alone with
pt_render and the same parameters."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _scenes():
    from pupiloptixlab_gb300 import scenes
    return [scenes.cornell_box(64, 48, max_depth=5), scenes.material_spheres(40, 24, max_depth=5),
            scenes.icosphere_field(56, 32, max_depth=5, num_instances=12, subdivisions=3, seed=4),
            scenes.cornell_box(16, 16, max_depth=5)]


@pytest.mark.parametrize("flags,width", [(0, 4), ("nosort", 4), ("nograph", 4), (0, 8)])
def test_batch_equals_serial_renders(cuda_ctx, flags, width):
    """Width 8: the merged BVH is compressed after rebasing, as each scene's own."""
    from pupiloptixlab_gb300 import abi
    from pupiloptixlab_gb300.api import GpuScene, render_batch, render_batch_stats
    fl = {0: 0, "nosort": abi.RENDER_NO_MATERIAL_SORT, "nograph": abi.RENDER_NO_GRAPH}[flags]
    gs = [GpuScene(cuda_ctx, sc, bvh_width=width) for sc in _scenes()]
    serial = [g.render(spp=3, seed=11, max_depth=5, flags=fl) for g in gs]
    batched = render_batch(cuda_ctx, gs, spp=3, seed=11, max_depth=5, flags=fl)
    torch.cuda.synchronize()
    for k, (a, b) in enumerate(zip(serial, batched)):
        for key in ("accum", "albedo", "normal", "test"):
            x = a[key].cpu().numpy().view(np.uint32)
            y = b[key].cpu().numpy().view(np.uint32)
            assert np.array_equal(x, y), (k, key, int((x != y).sum()))
    st = render_batch_stats(cuda_ctx)
    assert st.samples == 3 * sum(g.width * g.height for g in gs)
    for g in gs:
        g.close()


def test_batch_accumulates_across_calls(cuda_ctx):
    """Two batched calls of 2 spp (sample_cnt 0 then 2, seeds 0 then 2) equal
    one 4-spp call, as pt_render's frame-by-frame accumulation does."""
    from pupiloptixlab_gb300.api import GpuScene, render_batch
    gs = [GpuScene(cuda_ctx, sc) for sc in _scenes()[:2]]
    one = render_batch(cuda_ctx, gs, spp=4, seed=0, max_depth=5)
    two = render_batch(cuda_ctx, gs, spp=2, seed=0, max_depth=5)
    two = render_batch(cuda_ctx, gs, spp=2, seed=2, sample_cnt=2, max_depth=5, buffers=two)
    torch.cuda.synchronize()
    for a, b in zip(one, two):
        assert np.array_equal(a["accum"].cpu().numpy().view(np.uint32), b["accum"].cpu().numpy().view(np.uint32))
    for g in gs:
        g.close()


def test_batch_rejects_mixed_bvh_widths(cuda_ctx):
    from pupiloptixlab_gb300 import abi
    from pupiloptixlab_gb300.api import GpuScene, render_batch
    a = GpuScene(cuda_ctx, _scenes()[0], bvh_width=4)
    b = GpuScene(cuda_ctx, _scenes()[1], bvh_width=2)
    with pytest.raises(abi.PtError):
        render_batch(cuda_ctx, [a, b], spp=1)
    a.close()
    b.close()
