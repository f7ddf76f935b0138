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
    assert t and t["dram_bytes_per_ray"] > 0 and "--spp 2" in t["command"]


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


def test_reference_arm_never_loads_the_library_under_test():
    """`bench.py --impl reference` times the CPU restatement alone: the
    process maps the oracle library and not libpt_gb300.so (its camera comes
    from the oracle's own camera arithmetic)."""
    import json
    import subprocess
    code = (
        "import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--instances', '2', '--width', '48', "
        "'--height', '27', '--steps', '1', '--warmup', '0']\n"
        "import bench; bench.main()\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'pt': 'libpt_gb300' in maps, 'oracle': 'liboracle' in maps}))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.strip().splitlines() if x.startswith("{")]
    line, maps = lines[0], lines[-1]
    assert line["impl"] == "reference" and line["value"] > 0
    assert maps == {"pt": False, "oracle": True}
