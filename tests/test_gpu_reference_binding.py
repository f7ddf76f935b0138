"""The reference-side WavefrontPTPass (pupiloptixlab_gb300/host/
reference_binding/) end to end on the GPU: tests/scenes/box.xml built in the
reference's data model is put into a World, the SceneLoad event hands it to
the pass (ToPtSceneDesc, pt_scene_upload, pt_bvh_build, BufferManager
buffers), and 8 OnRun calls accumulate 8 frames into "final result".  The
image equals pt_render of the library's own XML loading of the same file
over 8 frames in the reference's random streams; the two scene builds differ
only in the last bits of a few instance transforms (float vs double
composition), so a few paths may diverge: at least 99 % of the pixels agree
within 1e-4, the rest stay close."""
import subprocess
from pathlib import Path

import numpy as np
import pytest
import torch

from pupiloptixlab_gb300 import abi, build
from pupiloptixlab_gb300.api import GpuScene
from _parity import compare
from test_reference_binding_cpu import compile_driver

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_reference_side_pass_renders_like_pt_render(cuda_ctx, tmp_path):
    if not build.HOST_LIB.exists():
        build.build_host()
    from pupiloptixlab_gb300 import host_api
    drv = compile_driver(tmp_path / "box_driver")
    out = tmp_path / "frame.f32"
    r = subprocess.run([str(drv), "run", "8", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "8 frames"
    img = np.fromfile(out, np.float32).reshape(-1, 4)
    g = GpuScene(cuda_ctx, host_api.XmlScene(str(ROOT / "tests" / "scenes" / "box.xml")))
    ref = g.render(8, seed=0, rng=abi.RNG_REF_LCG)["frame"]
    torch.cuda.synchronize()
    ref = ref.cpu().numpy()
    same, close = compare("reference-side WavefrontPTPass, box.xml, 8 frames", img, ref)
    assert np.isfinite(img).all() and img[:, :3].mean() > 0.02
    assert close.mean() >= 0.99
    assert np.abs(img - ref).mean() < 1e-3
