"""The full `Principled` model on the GPU against the FP64 oracle.

The reference's scenes/cbox.json with its materials edited so that every
lobe the loader reads is non-zero somewhere (scenes/cbox.json:3-62 lists
them; both reference scenes leave them at 0): a glass tallBox
(transmission 1, ior 1.5), a clearcoated, sheened shortBox, a tinted
specular back wall, a sheen-only left wall and a partly transmissive floor.
Sample-matched (same seed, same random numbers per bounce) through the
wavefront (sorted and unsorted shading), the persistent kernel and a batch
job; each must meet the relMSE 1e-3 bar, with ray counts within 2e-3.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np
import pytest

from conftest import reference_scene

pytestmark = pytest.mark.gpu

TOL = 1e-3
RAYS = 2e-3

EDITS = {
    "tallBox": dict(transmission=1.0, ior=1.5, roughness=0.15, metallic=0.0, color=[0.9, 0.95, 1.0]),
    "shortBox": dict(clearcoat=1.0, clearcoat_roughness=0.1, sheen=0.5, sheen_tint=0.5, roughness=0.5,
                     specular=0.5, color=[0.7, 0.2, 0.15]),
    "backWall": dict(specular=0.6, specular_tint=1.0, roughness=0.3),
    "leftWall": dict(sheen=1.0, sheen_tint=1.0),
    "floor": dict(transmission=0.3, roughness=0.6, metallic=0.1),
}


def principled_scene(tmp_path) -> str:
    src = reference_scene("cbox.json")
    d = json.load(open(src))
    for name, kw in EDITS.items():
        p = d["named_bsdfs"][name]["Principled"]
        for k, v in kw.items():
            if k == "color":
                p["color"] = {"Float3": v}
            else:
                p[k] = {"Float": v}
    base = os.path.dirname(src)
    for shape in d["shapes"]:
        shape["Mesh"][0] = os.path.join(base, shape["Mesh"][0])
    d["camera"]["Perspective"]["res"] = [128, 128]
    out = tmp_path / "cbox_principled.json"
    out.write_text(json.dumps(d))
    return str(out)


@pytest.fixture(scope="module")
def scene(gpu_ctx, tmp_path_factory):
    s = gpu_ctx.load_scene(principled_scene(tmp_path_factory.mktemp("principled")))
    mats = {round(m.transmission, 3): m for m in s.materials()}
    assert 1.0 in mats and abs(mats[1.0].ior - 1.5) < 1e-6
    yield s
    s.free()


@pytest.fixture(scope="module")
def reference(scene):
    import pyoracle

    o = pyoracle.OracleScene.from_aqua(scene)
    return o.render(64, 8, seed=31, precision=64)


def check(img, st, ref, ost):
    import pyoracle

    err = pyoracle.rel_mse(img, ref)
    assert err < TOL, err
    assert img.mean() > 0.01
    if st is not None:
        assert st.paths == int(ost[0])
        assert abs(st.ext_rays - ost[1]) / ost[1] < RAYS
        assert abs(st.shadow_rays - ost[2]) / ost[2] < RAYS


@pytest.mark.parametrize("sort", [1, 0])
def test_wavefront(gpu_ctx, scene, reference, sort):
    cfg = gpu_ctx.integrator(spp=64, max_depth=8, rr_depth=3, seed=31)
    img, st = gpu_ctx.render(scene, cfg, tuning=gpu_ctx.tuning(sort_by_material=sort))
    check(img, st, *reference)


def test_persistent_kernel(gpu_ctx, scene, reference):
    import aqua

    cfg = gpu_ctx.integrator(spp=64, max_depth=8, rr_depth=3, seed=31)
    img, st = gpu_ctx.render(scene, cfg, tuning=gpu_ctx.tuning(kernel=aqua.KERNEL_PERSISTENT))
    check(img, st, *reference)


def test_batch_job(gpu_ctx, scene, reference):
    torch = pytest.importorskip("torch")
    b = torch.full((128 * 128 * 3,), -1.0, dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    st, _ = gpu_ctx.render_batch([(scene, 128, 128, 64, 8, 31, b.data_ptr())])
    check(b.cpu().numpy().reshape(128, 128, 3), None, *reference)


def test_noalloc(gpu_ctx, scene, reference):
    import aqua
    torch = pytest.importorskip("torch")

    out = torch.zeros(128 * 128 * 3, dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    cfg = gpu_ctx.integrator(spp=64, max_depth=8, rr_depth=3, seed=31)
    st = aqua.Stats()
    assert gpu_ctx.lib.aqua_render_noalloc(gpu_ctx.handle, scene.handle, ctypes.byref(cfg),
                                           ctypes.c_void_p(out.data_ptr()), ctypes.byref(st)) == aqua.OK
    check(out.cpu().numpy().reshape(128, 128, 3), st, *reference)
