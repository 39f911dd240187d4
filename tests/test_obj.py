"""OBJ/MTL conversion (the role of the reference's tobj-based conversion,
Cargo.toml:23) and the film writers.

Parity: converting scenes/CornellBox-Original.obj must reproduce the
reference's own converted meshes (scenes/CornellBox-Original_*.mesh: same
file names, mesh names, vertices bit for bit, indices) and the colours of
scenes/cbox.json; the converted scene must load into the same triangles as
cbox.json. Synthetic files cover the OBJ forms the Cornell file does not use.
"""
from __future__ import annotations

import json
import os
import struct
import sys

import numpy as np
import pytest

import aqua

from conftest import reference_scene

REF_SCENES = os.path.dirname(reference_scene("cbox.json") or "")
ROOM = reference_scene("room.json")
need_ref = pytest.mark.skipif(not REF_SCENES, reason="reference Cornell scene not found")
need_room = pytest.mark.skipif(ROOM is None, reason="reference living-room scene not staged")


def read_bson(b: bytes):
    """Minimal BSON reader (document, array, string, double, int32, int64)."""
    def doc(p):
        n = struct.unpack_from("<i", b, p)[0]
        end, p, out = p + n - 1, p + 4, []
        while p < end:
            t = b[p]
            k_end = b.index(b"\0", p + 1)
            key, p = b[p + 1:k_end].decode(), k_end + 1
            if t == 0x01:
                v, p = struct.unpack_from("<d", b, p)[0], p + 8
            elif t == 0x02:
                ln = struct.unpack_from("<i", b, p)[0]
                v, p = b[p + 4:p + 4 + ln - 1].decode(), p + 4 + ln
            elif t == 0x10:
                v, p = struct.unpack_from("<i", b, p)[0], p + 4
            elif t == 0x12:
                v, p = struct.unpack_from("<q", b, p)[0], p + 8
            elif t in (0x03, 0x04):
                ln = struct.unpack_from("<i", b, p)[0]
                v = doc(p)
                v = [x for _, x in v] if t == 0x04 else dict(v)
                p += ln
            else:
                raise ValueError(t)
            out.append((key, v))
        return out
    return dict(doc(0))


@pytest.fixture(scope="module")
def ctx():
    c = aqua.Context(device=-2)  # AQUA_DEVICE_HOST_ONLY
    yield c
    c.close()


@need_ref
def test_cornell_obj_reproduces_the_reference_meshes(ctx, tmp_path):
    meshes, tris = ctx.convert_obj(os.path.join(REF_SCENES, "CornellBox-Original.obj"), str(tmp_path), "cbox.json",
                                   512, 512)
    assert (meshes, tris) == (8, 36)
    ref_files = sorted(f for f in os.listdir(REF_SCENES) if f.startswith("CornellBox-Original_") and f.endswith(".mesh"))
    ours = sorted(f for f in os.listdir(tmp_path) if f.endswith(".mesh"))
    assert ours == ref_files
    for f in ref_files:
        a = read_bson(open(os.path.join(REF_SCENES, f), "rb").read())
        b = read_bson(open(os.path.join(tmp_path, f), "rb").read())
        assert a["name"] == b["name"], f
        assert np.array_equal(np.array(a["vertices"]), np.array(b["vertices"])), f  # float32 positions, exactly
        assert np.array_equal(np.array(a["indices"]), np.array(b["indices"])), f
        assert a["texcoords"] == b["texcoords"] == [], f
        na, nb = np.array(a["normals"]), np.array(b["normals"])
        assert na.shape == nb.shape and np.all(np.sum(na * nb, axis=1) > 0.999), f


@need_ref
def test_cornell_obj_materials_match_cbox_json(ctx, tmp_path):
    ctx.convert_obj(os.path.join(REF_SCENES, "CornellBox-Original.obj"), str(tmp_path), "cbox.json", 512, 512)
    ours = json.load(open(tmp_path / "cbox.json"))["named_bsdfs"]
    ref = json.load(open(os.path.join(REF_SCENES, "cbox.json")))["named_bsdfs"]
    assert set(ours) == set(ref)
    for name, b in ref.items():
        p, q = b["Principled"], ours[name]["Principled"]
        np.testing.assert_allclose(q["color"]["Srgb"], p["color"]["Srgb"], atol=1e-6)  # reference stores float32
        assert q["roughness"]["Float"] == pytest.approx(0.4)
        assert q["specular"]["Float"] == 0.0
    # The MTL's Ke becomes the light's emission (CornellBox-Original.mtl: Ke 17 12 4).
    assert ours["light"]["Principled"]["emission"]["Float3"] == [17.0, 12.0, 4.0]


@need_ref
def test_converted_scene_loads_the_same_triangles(ctx, tmp_path):
    ctx.convert_obj(os.path.join(REF_SCENES, "CornellBox-Original.obj"), str(tmp_path), "cbox.json", 512, 512)
    a = ctx.load_scene(os.path.join(REF_SCENES, "cbox.json"))
    b = ctx.load_scene(str(tmp_path / "cbox.json"))
    va, vb = a.triangles()[0], b.triangles()[0]
    assert va.shape == vb.shape == (36, 9)
    assert sorted(map(tuple, va.tolist())) == sorted(map(tuple, vb.tolist()))
    assert b.info().num_lights == 2  # the emissive light quad: two triangle lights
    a.free()
    b.free()


def write(path, text):
    with open(path, "w") as f:
        f.write(text)


def test_synthetic_obj_forms(ctx, tmp_path):
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import test_jpeg

    data, _ = test_jpeg.encode(test_jpeg.synthetic_image(16, 24, 2))
    (tmp_path / "tex").mkdir()
    open(tmp_path / "tex" / "checker.jpg", "wb").write(data)
    write(tmp_path / "m.mtl", "newmtl red\n Kd 0.5 0.1 0.1\nnewmtl img\n Kd 1 1 1\n map_Kd -s 1 1 1 tex\\checker.jpg\n"
                              "newmtl glow\n Ke 2 2 2\n")
    write(tmp_path / "m.obj", "\n".join([
        "mtllib m.mtl",
        "v 0 0 0", "v 1 0 0", "v 1 1 0", "v 0 1 0", "v 0 0 1",
        "vt 0 0", "vt 1 0", "vt 1 1", "vt 0 1",
        "vn 0 0 1",
        "o quad",
        "usemtl img",
        "f 1/1/1 2/2/1 3/3/1 4/4/1",     # quad with v/vt/vn -> 2 triangles, 4 vertices
        "usemtl red",                     # material change inside the object: another mesh
        "f -5//-1 -3//-1 -1//-1",         # relative indices, v//vn
        "g pent",
        "usemtl glow",
        "f 1 2 3 4 5",                    # pentagon -> 3 triangles, computed normals
    ]) + "\n")
    meshes, tris = ctx.convert_obj(str(tmp_path / "m.obj"), str(tmp_path), "m.json", 64, 32)
    assert (meshes, tris) == (3, 6)
    files = sorted(f for f in os.listdir(tmp_path) if f.endswith(".mesh"))
    assert files == ["m_pent_2.mesh", "m_quad_0.mesh", "m_quad_1.mesh"]
    q = read_bson(open(tmp_path / "m_quad_0.mesh", "rb").read())
    assert q["name"] == "quad" and len(q["vertices"]) == 4 and q["indices"] == [[0, 1, 2], [0, 2, 3]]
    assert q["texcoords"] == [[0, 0], [1, 0], [1, 1], [0, 1]] and all(n == [0, 0, 1] for n in q["normals"])
    r = read_bson(open(tmp_path / "m_quad_1.mesh", "rb").read())
    assert r["vertices"] == [[0, 0, 0], [1, 1, 0], [0, 0, 1]] and r["texcoords"] == []
    p = read_bson(open(tmp_path / "m_pent_2.mesh", "rb").read())
    assert len(p["indices"]) == 3 and all(abs(np.linalg.norm(n) - 1) < 1e-12 for n in p["normals"])
    s = ctx.load_scene(str(tmp_path / "m.json"))
    i = s.info()
    assert (i.num_triangles, i.num_meshes, i.num_textures, i.width, i.height) == (6, 3, 1, 64, 32)
    assert i.num_lights == 3  # the glowing pentagon's triangles
    mats = {tuple(np.round(m.base_color, 4)): m for m in s.materials()}
    assert any(m.base_texture == 0 for m in mats.values())
    s.free()


def test_obj_errors(ctx, tmp_path):
    with pytest.raises(aqua.AquaError) as e:
        ctx.convert_obj(str(tmp_path / "missing.obj"), str(tmp_path))
    assert e.value.status == aqua.ERR_IO
    write(tmp_path / "bad.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 7\n")
    with pytest.raises(aqua.AquaError) as e:
        ctx.convert_obj(str(tmp_path / "bad.obj"), str(tmp_path))
    assert e.value.status == aqua.ERR_PARSE and "out of range" in str(e.value)
    write(tmp_path / "two.obj", "v 0 0 0\nv 1 0 0\nf 1 2\n")
    with pytest.raises(aqua.AquaError) as e:
        ctx.convert_obj(str(tmp_path / "two.obj"), str(tmp_path))
    assert e.value.status == aqua.ERR_PARSE
    # A number made of bytes that are not UTF-8: the message quotes it with
    # those bytes escaped, so the C string aqua_last_error returns is UTF-8.
    (tmp_path / "bytes.obj").write_bytes(b"v 0 0 \x89\xff\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    st = ctx.lib.aqua_convert_obj(ctx.handle, str(tmp_path / "bytes.obj").encode(), str(tmp_path).encode(),
                                  b"s.json", 8, 8, None, None)
    assert st == aqua.ERR_PARSE
    raw = ctx.lib.aqua_last_error(ctx.handle)
    msg = raw.decode("utf-8")  # strict: must not raise
    assert "bad number" in msg and "\\x89\\xff" in msg
    # strtod reads "nan" and "inf"; a vertex must be a finite number
    write(tmp_path / "nan.obj", "v 0 0 nan\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    with pytest.raises(aqua.AquaError) as e:
        ctx.convert_obj(str(tmp_path / "nan.obj"), str(tmp_path))
    assert e.value.status == aqua.ERR_PARSE and "bad number" in str(e.value)


def test_write_image_pfm_and_ppm(ctx, tmp_path):
    w, h = 5, 3
    rgb = np.linspace(0, 1.5, w * h * 3, dtype=np.float32).reshape(h, w, 3)
    rgb[0, 0] = [0.0, 0.5, 1.0]
    ctx.write_image(str(tmp_path / "a.pfm"), rgb, w, h)
    b = open(tmp_path / "a.pfm", "rb").read()
    head = b"PF\n5 3\n-1.0\n"
    assert b.startswith(head)
    back = np.frombuffer(b[len(head):], "<f4").reshape(h, w, 3)[::-1]  # PFM rows run bottom to top
    assert np.array_equal(back, rgb)
    ctx.write_image(str(tmp_path / "a.ppm"), rgb, w, h)
    b = open(tmp_path / "a.ppm", "rb").read()
    head = b"P6\n5 3\n255\n"
    px = np.frombuffer(b[len(head):], np.uint8).reshape(h, w, 3)
    assert list(px[0, 0]) == [0, 188, 255]  # sRGB(0.5) = 0.7354 -> 188
    assert px[-1, -1].tolist() == [255, 255, 255]  # clamped
    with pytest.raises(aqua.AquaError) as e:
        ctx.write_image(str(tmp_path / "a.png"), rgb, w, h)
    assert e.value.status == aqua.ERR_INVALID_ARG
