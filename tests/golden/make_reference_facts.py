"""Writes reference_facts.json: numbers read from the reference's own data
files (the only checkable facts it ships; it has no tests or golden images).

Run in a container where the reference tree is mounted (path as argv[1]);
the JSON it writes is committed so the tests never read the reference.
Sources: scenes/cbox.json, scenes/room.json, scenes/integrator.json,
scenes/*.mesh (BSON), scenes/CornellBox-Original.mtl.
"""
from __future__ import annotations

import json
import os
import struct
import sys


def bson(b: bytes, off: int = 0):
    n = struct.unpack_from("<i", b, off)[0]
    end, off, out = off + n - 1, off + 4, {}
    while off < end:
        t = b[off]
        off += 1
        k = b[off:b.index(b"\0", off)].decode()
        off += len(k) + 1
        if t == 0x01:
            v = struct.unpack_from("<d", b, off)[0]; off += 8
        elif t == 0x02:
            ln = struct.unpack_from("<i", b, off)[0]; v = b[off + 4:off + 3 + ln].decode(); off += 4 + ln
        elif t in (0x03, 0x04):
            ln = struct.unpack_from("<i", b, off)[0]; v = bson(b, off); off += ln
            if t == 0x04:
                v = [v[str(i)] for i in range(len(v))]
        elif t == 0x12:
            v = struct.unpack_from("<q", b, off)[0]; off += 8
        elif t == 0x10:
            v = struct.unpack_from("<i", b, off)[0]; off += 4
        else:
            raise ValueError(f"bson type {t:#x}")
        out[k] = v
    return out


def main(ref: str):
    sc = os.path.join(ref, "scenes")
    facts = {}
    for name in ("cbox", "room"):
        d = json.load(open(os.path.join(sc, f"{name}.json")))
        tris, meshes, missing = 0, 0, []
        for s in d["shapes"]:
            f = os.path.join(sc, s["Mesh"][0])
            if not os.path.exists(f):
                missing.append(s["Mesh"][0])
                continue
            m = bson(open(f, "rb").read())
            tris += len(m["indices"])
            meshes += 1
        cam = d["camera"]["Perspective"]
        facts[name] = {"shapes": len(d["shapes"]), "named_bsdfs": len(d["named_bsdfs"]), "meshes_present": meshes,
                       "triangles_present": tris, "missing_meshes": missing, "res": cam["res"], "fov": cam["fov"],
                       "translate": cam["transform"]["translate"],
                       "lights": [l["Point"]["pos"] for l in d["lights"]],
                       "image_textures": sum(1 for b in d["named_bsdfs"].values()
                                             if "Image" in b["Principled"]["color"])}
    cb = json.load(open(os.path.join(sc, "cbox.json")))
    facts["cbox"]["srgb"] = {n: b["Principled"]["color"]["Srgb"] for n, b in cb["named_bsdfs"].items()}
    facts["cbox"]["metallic"] = {n: b["Principled"]["metallic"]["Float"] for n, b in cb["named_bsdfs"].items()}
    facts["cbox"]["roughness"] = {n: b["Principled"]["roughness"]["Float"] for n, b in cb["named_bsdfs"].items()}
    kd = {}
    cur = None
    for ln in open(os.path.join(sc, "CornellBox-Original.mtl")):
        p = ln.split()
        if p and p[0] == "newmtl":
            cur = p[1]
        elif p and p[0] in ("Kd", "Ke") and cur:
            kd.setdefault(cur, {})[p[0]] = [float(x) for x in p[1:4]]
    facts["mtl"] = kd
    facts["integrator"] = json.load(open(os.path.join(sc, "integrator.json")))
    short = bson(open(os.path.join(sc, "CornellBox-Original_shortBox_5.mesh"), "rb").read())
    facts["shortBox_mesh"] = {"vertices": len(short["vertices"]), "triangles": len(short["indices"]),
                              "first_vertex": short["vertices"][0], "first_index": short["indices"][0]}
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_facts.json")
    json.dump(facts, open(out, "w"), indent=1, sort_keys=True)
    print(out)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AQUA_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_reference_facts.py <reference checkout> (or set AQUA_REFERENCE_DIR)")
    main(ref)
