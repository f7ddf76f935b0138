"""Copy the reference's own sample scenes (PupilOptixLab data/static/*.xml) into
tests/golden/ref_scenes/ as test fixtures, byte for byte.

They are the only scenes the reference ships and the only way it checks its
renderer (by eye, in its GUI): cornellbox, default, denoised_scene,
material_test (all seven materials), mis (Veach-style rough-conductor plates)
and restir_test.  They name no external assets.  The tests load them with the
library's XML loader and render them on the GPU against the oracle, on
machines that do not hold the reference tree.  Run once where the tree is
present:

    python tests/golden/make_ref_scenes.py      # $PUPIL_REFERENCE_DIR or ../reference
"""
from __future__ import annotations

import hashlib
import shutil
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from pupiloptixlab_gb300.build import REFERENCE_TREE  # noqa: E402

NAMES = ["cornellbox", "default", "denoised_scene", "material_test", "mis", "restir_test"]
OUT = Path(__file__).resolve().parent / "ref_scenes"


def main() -> None:
    src = REFERENCE_TREE / "data" / "static"
    OUT.mkdir(exist_ok=True)
    lines = []
    for n in NAMES:
        shutil.copyfile(src / f"{n}.xml", OUT / f"{n}.xml")
        digest = hashlib.sha256((OUT / f"{n}.xml").read_bytes()).hexdigest()
        lines.append(f"{digest}  {n}.xml")
    (OUT / "SHA256SUMS").write_text("\n".join(lines) + "\n")
    print(f"copied {len(NAMES)} scenes from {src}")


if __name__ == "__main__":
    main()
