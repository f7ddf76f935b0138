"""bench.py's bookkeeping that needs no GPU: the workload string follows the
options, and the committed DRAM-traffic capture is attached to the roofline
only at the configuration it was captured on."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def _parse(monkeypatch, *argv):
    monkeypatch.setattr(sys, "argv", ["bench.py", *argv])
    return bench.parse()


def test_default_run_is_the_captured_configuration(monkeypatch):
    a = _parse(monkeypatch)
    assert a.at_capture_config
    w = bench.headline_workload(a)
    assert w.startswith("1M-triangle") and "200 x 5120" in w and "1920x1080, 64 spp, max depth 8" in w
    t = bench.committed_traffic("headline")
    assert t and t["dram_bytes_per_launch"] > 0 and t["passes"] == 1
    assert bench.committed_traffic("hair")["dram_bytes_per_launch"] > 0


def test_other_configurations_get_no_committed_traffic(monkeypatch):
    for argv in (["--spp", "2"], ["--width", "1280"], ["--bvh-width", "8"], ["--bvh-fast-build"], ["--smem-nodes", "5"],
                 ["--wave-spp", "16"], ["--no-material-sort"], ["--autotune"], ["--instances", "800"]):
        a = _parse(monkeypatch, *argv)
        assert not a.at_capture_config, argv
    a = _parse(monkeypatch, "--spp", "2", "--instances", "800")
    assert bench.headline_workload(a).startswith("4M-triangle") and "2 spp" in bench.headline_workload(a)


def test_timing_options_keep_the_captured_configuration(monkeypatch):
    a = _parse(monkeypatch, "--steps", "1", "--warmup", "1", "--no-cpu-baseline", "--no-e2e")
    assert a.at_capture_config
    a = _parse(monkeypatch, "--workload", "hair")
    assert a.at_capture_config
