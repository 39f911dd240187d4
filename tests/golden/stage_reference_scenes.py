"""Stages the reference's larger scene data (the living room: room.json, its
152 BSON meshes and the JPEG textures, about 50 MB) into
tests/golden/reference_scenes/, a git-ignored folder that still travels with
the repository snapshot to the GPU machine. The small Cornell scene
(cbox.json, its OBJ/MTL source and 8 meshes) is committed under
tests/golden/cbox/ instead.

The files are the reference project's own data (Apache-2.0, see its
LICENSE), copied unchanged. Usage:

    python tests/golden/stage_reference_scenes.py <reference checkout>

or with AQUA_REFERENCE_DIR set. Tests that need these files skip when the
folder is absent.
"""
from __future__ import annotations

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEST = os.path.join(HERE, "reference_scenes")


def main(ref: str) -> None:
    src = os.path.join(ref, "scenes")
    if not os.path.isdir(src):
        sys.exit(f"no scenes folder under {ref}")
    os.makedirs(DEST, exist_ok=True)
    n = 0
    for name in sorted(os.listdir(src)):
        if name == "room.json" or name == "living_room.mtl" or (name.startswith("living_room_") and name.endswith(".mesh")):
            shutil.copyfile(os.path.join(src, name), os.path.join(DEST, name))
            n += 1
    tex = os.path.join(src, "textures")
    if os.path.isdir(tex):
        os.makedirs(os.path.join(DEST, "textures"), exist_ok=True)
        for name in sorted(os.listdir(tex)):
            shutil.copyfile(os.path.join(tex, name), os.path.join(DEST, "textures", name))
            n += 1
    print(f"staged {n} files into {DEST}")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AQUA_REFERENCE_DIR")
    if not ref:
        sys.exit(__doc__)
    main(ref)
