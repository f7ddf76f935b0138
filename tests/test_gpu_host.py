"""The C++ host layer on the GPU: System + WavefrontPTPass (one frame per
OnRun, as PTPass) over scenes loaded by the C++ mitsuba-style loader."""
import subprocess
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle
from pupiloptixlab_gb300 import abi, build
from pupiloptixlab_gb300.api import GpuScene
from _parity import assert_bit_identical

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent / "scenes"


@pytest.fixture(scope="module")
def host(ptlib):
    if not build.HOST_LIB.exists():
        build.build_host()
    from pupiloptixlab_gb300 import host_api
    return host_api


@pytest.mark.parametrize("name", ["box.xml", "materials.xml"])
def test_pass_equals_c_abi_render(cuda_ctx, host, name):
    """8 frames of WavefrontPTPass::OnRun == one pt_render of 8 frames."""
    path = str(HERE / name)
    img = host.run_scene(path, 8, rng=abi.RNG_REF_LCG)
    xs = host.XmlScene(path)
    g = GpuScene(cuda_ctx, xs)
    out = g.render(8, rng=abi.RNG_REF_LCG)
    torch.cuda.synchronize()
    assert np.array_equal(img.view(np.uint32), out["frame"].cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("name", ["box.xml", "materials.xml"])
def test_pass_matches_oracle(cuda_ctx, host, name):
    path = str(HERE / name)
    img = host.run_scene(path, 4, rng=abi.RNG_PCG32)
    o = oracle.OracleScene(host.XmlScene(path))
    ref = o.render(abi.RenderParams(spp=4, seed=0, accumulate=1, rng=abi.RNG_PCG32))["frame"]
    assert_bit_identical(f"WavefrontPTPass {name}", img, ref)


def test_cli_writes_pfm(host, tmp_path):
    out = tmp_path / "box.pfm"
    r = subprocess.run([str(build.HOST_CLI), str(HERE / "box.xml"), str(out), "4"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    data = out.read_bytes()
    assert data.startswith(b"PF\n48 48\n-1.0\n")
    px = np.frombuffer(data[len(b"PF\n48 48\n-1.0\n"):], np.float32).reshape(-1, 3)
    assert px.shape[0] == 48 * 48 and np.isfinite(px).all() and px.mean() > 0
