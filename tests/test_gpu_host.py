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


def test_progress_file_resumes_the_frame_sequence(cuda_ctx, host, tmp_path):
    """Progressive resume: 4 frames, SaveProgress, a new System and pass,
    LoadProgress, 4 more frames == 8 frames in one go, bit for bit."""
    path = str(HERE / "box.xml")
    full = host.run_scene_ex(path, 8, rng=abi.RNG_PCG32)
    save = str(tmp_path / "box.ptprogress")
    host.run_scene_ex(path, 4, rng=abi.RNG_PCG32, save_to=save)
    cont = host.run_scene_ex(path, 4, rng=abi.RNG_PCG32, resume_from=save)
    assert np.array_equal(cont.view(np.uint32), full.view(np.uint32))
    # a progress file of another film size is refused
    with pytest.raises(abi.PtError) as e:
        host.run_scene_ex(str(HERE / "materials.xml"), 1, resume_from=save)
    assert "film" in str(e.value)


def _mesh_positions(d):
    import ctypes as C
    return [np.ctypeslib.as_array(C.cast(d.meshes[i].positions, C.POINTER(C.c_float)),
                                  shape=(d.meshes[i].num_vertices, 3)) for i in range(d.num_meshes)]


def test_world_events_reach_the_pass(cuda_ctx, host):
    """EWorldEvent::RenderInstanceUpdate (new vertices, refit) and
    EWorldEvent::CameraChange reach the WavefrontPTPass through the event
    lists; each restarts accumulation, so the frames after the change equal a
    fresh render of the changed scene."""
    from pupiloptixlab_gb300 import scenes
    path = str(HERE / "box.xml")
    rng = np.random.default_rng(4)
    xs = host.XmlScene(path)
    pos = _mesh_positions(xs.desc())
    jit = np.concatenate([p + rng.normal(0, 0.01, p.shape).astype(np.float32) for p in pos]).astype(np.float32)
    got = host.run_scene_ex(path, 5, rng=abi.RNG_PCG32, change_after=3, positions=jit)
    moved = host.XmlScene(path)
    off = 0
    for p in _mesh_positions(moved.desc()):
        p[:] = jit[off:off + p.shape[0]]
        off += p.shape[0]
    g = GpuScene(cuda_ctx, moved)
    ref = g.render(2, seed=0, rng=abi.RNG_PCG32)["frame"].cpu().numpy()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    g.close()
    cam = scenes.camera(30.0, 1.0, scenes.look_at_to_world((0.3, 1.2, 3.5), (0.0, 0.9, 0.0)))
    got = host.run_scene_ex(path, 4, rng=abi.RNG_PCG32, change_after=1, camera=cam)
    g = GpuScene(cuda_ctx, host.XmlScene(path))
    g.set_camera(cam)
    ref = g.render(3, seed=0, rng=abi.RNG_PCG32)["frame"].cpu().numpy()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
