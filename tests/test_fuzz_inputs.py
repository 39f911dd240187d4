"""Malformed inputs to the host-side parsers: JPEG bytes, BSON `.mesh` files,
scene JSON and OBJ/MTL text, each mutated many times from a valid file
(bytes overwritten, truncated, duplicated or deleted; seeded). Every call
must come back with a status (success or an error code and message); none
may crash, hang or exhaust memory. The mutations run in a child process with
a 6 GB address-space limit, so a crash fails the test instead of ending the
session, and a header that asks for an enormous image has to fail cleanly
(AQUA_ERR_OOM or a refusal) rather than take the machine's memory. No GPU
needed."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import json, os, random, resource, sys
import numpy as np
resource.setrlimit(resource.RLIMIT_AS, (6 << 30, 6 << 30))
ROOT, KIND, SEED, N, TMP = sys.argv[1], sys.argv[2], int(sys.argv[3]), int(sys.argv[4]), sys.argv[5]
sys.path[:0] = [os.path.join(ROOT, "aqua-engine_gb300"), os.path.join(ROOT, "tests")]
import aqua
ctx = aqua.Context(device=-2)
rng = random.Random(SEED)


def mutate(b):
    b = bytearray(b)
    for _ in range(rng.randint(1, 3)):
        if not b:
            break
        k = rng.randrange(4)
        i = rng.randrange(len(b))
        if k == 0:
            for _ in range(rng.randint(1, 8)):
                b[rng.randrange(len(b))] = rng.randrange(256)
        elif k == 1:
            del b[i:]
        elif k == 2:
            b[i:i] = b[i:i + rng.randint(1, 64)]
        else:
            del b[i:i + rng.randint(1, 64)]
    return bytes(b)


ok = err = 0
if KIND == "jpeg":
    from test_jpeg import encode, synthetic_image
    seeds = [encode(synthetic_image(40, 56, 3))[0],
             encode(synthetic_image(33, 17, 4), sampling=(2, 2), restart=2)[0],
             encode(synthetic_image(24, 24, 5), progressive=True)[0],
             encode(synthetic_image(16, 40, 6), grey=True)[0]]
    for k in range(N):
        data = mutate(seeds[k % len(seeds)])
        try:
            ctx.decode_jpeg(data)
            ok += 1
        except aqua.AquaError:
            err += 1
else:
    from test_loaders import principled, scene_json, write_mesh
    mesh = os.path.join(TMP, "m.mesh")
    write_mesh(mesh, [[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1], [0, 1, 0]],
               [[0, 1, 2], [0, 2, 3], [0, 1, 4]], uvs=[[0, 0], [1, 0], [1, 1], [0, 1], [0.5, 0.5]])
    good_mesh = open(mesh, "rb").read()
    scene = os.path.join(TMP, "s.json")
    good_scene = json.dumps(scene_json([("m.mesh", "w")], {"w": principled(metallic=0.5)}), indent=1).encode()
    objp = os.path.join(TMP, "a.obj")
    good_obj = (b"mtllib a.mtl\no box\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\n"
                b"vn 0 0 1\nusemtl red\nf 1/1/1 2/2/1 3/3/1 4/1/1\ng second\nf -1 -2 -3\n")
    good_mtl = b"newmtl red\nKd 0.8 0.1 0.1\nKe 0 0 0\nnewmtl lamp\nKd 0 0 0\nKe 5 5 5\n"
    for k in range(N):
        open(mesh, "wb").write(good_mesh)
        open(scene, "wb").write(good_scene)
        if KIND == "mesh":
            open(mesh, "wb").write(mutate(good_mesh))
        elif KIND == "scene":
            open(scene, "wb").write(mutate(good_scene))
        if KIND in ("mesh", "scene"):
            try:
                s = ctx.load_scene(scene, allow_missing=bool(k % 2))
                s.bvh()
                s.free()
                ok += 1
            except aqua.AquaError:
                err += 1
            continue
        open(objp, "wb").write(mutate(good_obj) if k % 2 == 0 else good_obj)
        open(os.path.join(TMP, "a.mtl"), "wb").write(mutate(good_mtl) if k % 2 == 1 else good_mtl)
        out = os.path.join(TMP, "out")
        os.makedirs(out, exist_ok=True)
        try:
            ctx.convert_obj(objp, out, "conv.json", 16, 16)
            ok += 1
        except aqua.AquaError:
            err += 1
print(json.dumps({"ok": ok, "err": err}))
'''


@pytest.mark.parametrize("kind,n", [("jpeg", 6000), ("mesh", 1500), ("scene", 1500), ("obj", 1500)])
def test_mutated_inputs_return_a_status(built, tmp_path, kind, n):
    # seed 3: its JPEG sequence reaches, at mutation 4533, a Huffman table
    # that overran the decoder's lookup table before that was fixed
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, kind, "3", str(n), str(tmp_path)],
                       capture_output=True, text=True, timeout=240)
    assert r.returncode == 0, f"child died (rc {r.returncode}):\n{r.stderr[-2000:]}"
    counts = json.loads(r.stdout.strip().splitlines()[-1])
    assert counts["ok"] + counts["err"] == n
    # the mutations reach both outcomes (some survive, some are refused)
    assert counts["err"] > 0
