"""Build recipe for the native parts of the package.

``build_library()`` compiles ``csrc/`` into ``_build/libpt_gb300.so``: the CUDA
translation units with nvcc for sm_103a only, the host translation unit with
g++, in parallel, then links them with nvcc.  ``build_oracle()`` runs
``make`` in ``oracle/`` (the CPU checker used by the tests) and, when the
PupilOptixLab source tree is present, its ``ref`` target.

Host code is built with ``-ffp-contract=off``: the scene flattening must
produce the same bits on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libpt_gb300.so"
ORACLE = ROOT / "oracle"
# The PupilOptixLab source tree (only for the oracle's reference-compiled
# known-answer library): $PUPIL_REFERENCE_DIR if set, else a `reference`
# directory beside this repository; absent on machines that only run the tests.
REFERENCE_TREE = Path(os.environ.get("PUPIL_REFERENCE_DIR") or (ROOT.parent / "reference"))

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "-I", str(ROOT / "include")]
# Per-file extra flags.  The shading code is compiled without FMA contraction
# so that its arithmetic follows the reference's operation order exactly.
CU_SOURCES = {
    "pt_bvh.cu": [],
    "pt_render.cu": ["-fmad=false"],
    "pt_conv.cu": [],
    "pt_denoise.cu": [],
}
CPP_SOURCES = ["pt_scene.cpp"]
# C++ host layer above the C-ABI (Pass / System / scene loader): its own
# library, linked against libpt_gb300.so, plus the pupil_pt command-line tool.
HOST = PKG / "host"
HOST_SOURCES = ["xml.cpp", "image.cpp", "inflate.cpp", "jpeg.cpp", "hair.cpp", "scene.cpp", "pass.cpp", "host_capi.cpp"]
HOST_LIB = BUILD / "libpupil_host.so"
HOST_CLI = BUILD / "pupil_pt"


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "pt_api.h"]
    jobs = []
    objs = []
    for src, extra in CU_SOURCES.items():
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append([nvcc] + NVCC_COMMON + extra + ["-c", str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I", _cuda_include(), "-I", str(ROOT / "include"), "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + GENCODE + ["-shared", "-o", str(LIB)] + [str(o) for o in objs])
    return LIB


def _cuda_lib_dir() -> str:
    root = Path(_nvcc()).resolve().parent.parent
    for cand in (root / "lib64", root / "lib", root / "targets" / "sbsa-linux" / "lib",
                 root / "targets" / "x86_64-linux" / "lib"):
        if (cand / "libcudart.so").exists():
            return str(cand)
    return str(root / "lib64")


def build_host(force: bool = False) -> Path:
    """libpupil_host.so and pupil_pt (g++ only; they see nothing but pt_api.h)."""
    BUILD.mkdir(exist_ok=True)
    srcs = [HOST / f for f in HOST_SOURCES]
    deps = srcs + sorted(HOST.glob("*.h")) + [ROOT / "include" / "pt_api.h", LIB]
    common = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", str(ROOT / "include"),
              "-I", str(HOST), "-I", _cuda_include()]
    links = ["-L", str(BUILD), "-lpt_gb300", "-L", _cuda_lib_dir(), "-lcudart", "-Wl,-rpath,$ORIGIN",
             "-Wl,-rpath," + _cuda_lib_dir()]
    if force or _stale(HOST_LIB, deps):
        _run(["g++"] + common + ["-shared", "-o", str(HOST_LIB)] + [str(x) for x in srcs] + links)
    if force or _stale(HOST_CLI, [HOST / "pt_main.cpp", HOST_LIB]):
        _run(["g++"] + common + ["-o", str(HOST_CLI), str(HOST / "pt_main.cpp"), "-L", str(BUILD), "-lpupil_host"]
             + links)
    return HOST_LIB


def build_oracle(verbose: bool = False) -> None:
    _run(["make", "-C", str(ORACLE), "-s", "all"])
    if (REFERENCE_TREE / "framework").is_dir():
        _run(["make", "-C", str(ORACLE), "-s", "ref", f"REF_DIR={REFERENCE_TREE}", f"CUDA_INC={_cuda_include()}"])


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
    build_host(force="--force" in sys.argv)
    build_oracle(verbose=True)
    print(LIB)
