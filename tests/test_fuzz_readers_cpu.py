"""Mutation test of the host layer's file readers (tests/fuzz/readers_fuzz.cpp):
PNG, JPEG, OpenEXR (RLE / ZIPS / ZIP), Radiance HDR, PFM, OBJ, HAIR and the
reference's own mitsuba XML scenes, each seed mutated a few hundred times and
read back by a build of the readers with AddressSanitizer and
UndefinedBehaviorSanitizer.  A mutated file may be accepted or refused; an
out-of-bounds access, an overflow or an exception escaping a reader fails the
test.  Seeds come from the encoders of tests/test_host_loader.py."""
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

import test_host_loader as T

HERE = Path(__file__).resolve().parent
HOST = HERE.parent / "pupiloptixlab_gb300" / "host"
SOURCES = [HERE / "fuzz" / "readers_fuzz.cpp"] + [HOST / f for f in
                                                   ("scene.cpp", "xml.cpp", "hair.cpp", "image.cpp", "inflate.cpp",
                                                    "jpeg.cpp")]
ITERATIONS = 300


def _seeds(d: Path):
    rng = np.random.default_rng(9)
    out = []

    def put(name, data):
        (d / name).write_bytes(data)
        out.append(d / name)

    for i, (ct, depth, il) in enumerate([(2, 8, False), (6, 16, True), (0, 4, True), (3, 8, False)]):
        chans = {0: 1, 2: 3, 3: 1, 6: 4}[ct]
        pal = trns = None
        if ct == 3:
            pal, trns = rng.integers(0, 256, (256, 3)), rng.integers(0, 256, 128)
            s = rng.integers(0, 256, (9, 11, 1))
        else:
            s = rng.integers(0, 1 << depth, (9, 11, chans))
        put(f"p{i}.png", T._png_bytes(s, ct, depth, il, pal, trns))
    img = rng.random((7, 9, 4)).astype(np.float32)
    for c in (1, 2, 3):
        put(f"e{c}.exr", T._exr_bytes(img, c, c == 2))
    src = rng.integers(0, 256, (17, 21, 3)).astype(np.uint8)
    put("j0.jpg", T._jpeg_bytes(src, False, 3, 0, False)[0])
    put("j1.jpg", T._jpeg_bytes(src, True, 3, 2, False)[0])
    put("g.jpg", T._jpeg_bytes(src[..., 1], False, 3, 0, True)[0])
    px = rng.integers(0, 256, (4, 12, 4)).astype(np.uint8)
    put("a.hdr", b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 4 +X 12\n" + px.tobytes())
    rle = b"".join(b"\x02\x02" + struct.pack(">H", 12) + b"".join(bytes([12]) + bytes(rng.integers(0, 256, 12).tolist())
                                                                  for _ in range(4)) for _ in range(4))
    put("b.hdr", b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 4 +X 12\n" + rle)
    put("c.pfm", b"PF\n7 5\n-1.0\n" + rng.random((5, 7, 3)).astype("<f4").tobytes())
    T._write_hair(d / "h.hair", [rng.random((n, 3)).astype(np.float32) for n in (4, 6, 3)])
    out.append(d / "h.hair")
    put("t.obj", (HERE / "scenes" / "tetra.obj").read_bytes())
    for name in ("cornellbox", "mis", "material_test"):
        put(f"{name}.xml", (HERE / "golden" / "ref_scenes" / f"{name}.xml").read_bytes())
    return out


def _compile(tmp: Path, sanitize: bool) -> Path:
    exe = tmp / "readers_fuzz"
    flags = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-O1", "-g"] if sanitize else ["-O2"]
    cmd = ["g++", "-std=c++17", *flags, f"-I{HOST}", f"-I{HERE.parent / 'include'}", *map(str, SOURCES), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    if r.returncode != 0:
        return None
    return exe


def test_readers_survive_mutated_files(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = _compile(tmp_path, sanitize=True) or _compile(tmp_path, sanitize=False)
    assert exe is not None, "the fuzz driver does not compile"
    seeds = _seeds(tmp_path)
    env = {"ASAN_OPTIONS": "detect_leaks=0", "PATH": "/usr/bin:/bin"}
    r = subprocess.run([str(exe), str(ITERATIONS), *map(str, seeds)], capture_output=True, text=True, timeout=600,
                       env=env)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert r.stdout.count("mutations accepted") == len(seeds)
