"""aqua_render_noalloc: the render entry point for callers that may not let
a library allocate device memory (engines that own every device byte through
their own arena, hosts that cannot afford the device-wide synchronisation of
cudaMalloc/cudaFree). It runs on a fixed static scratch array instead of a
per-context workspace.

The test calls it through the C ABI twice in a row (different seeds, spp and
image sizes, so a leftover of the first call would show in the second) and
compares each image with the one aqua_render returns for the same inputs,
within the tests' image tolerance (relMSE 1e-3; the two are in fact
bit-identical, because every pixel's samples run in the same order whatever
the slot count). It also checks that the call allocated no workspace and that
an image above the fixed limit is refused before any device work. A 512x512
image (262,144 pixels over 65,536 path slots, so each slot owns four pixels)
is compared with the FP64 oracle at the same seed and with aqua_render, and
depth limits outside [0, 250] are refused like aqua_render refuses them. The
file is
named so that pytest collects it last, and it builds its own context so it
passes alone in a fresh process as well as after the other tests.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-3  # relMSE, as in the other image tests


def rel_mse(x, r):
    x = x.astype(np.float64)
    r = r.astype(np.float64)
    return float(np.mean((x - r) ** 2 / (r * r + 1e-2)))


def test_noalloc_matches_render_on_two_calls():
    torch = pytest.importorskip("torch")
    import aqua

    with aqua.Context(device=0) as ctx:
        lib = ctx.lib
        assert lib.aqua_render_noalloc_max_pixels() == 1 << 19
        scene = ctx.procedural(2, seed=0, width=160, height=120)
        noalloc_images = []
        for seed, spp, (w, h) in [(1, 16, (160, 120)), (2, 8, (96, 64))]:
            scene.set_resolution(w, h)
            cfg = ctx.integrator(spp=spp, max_depth=8, rr_depth=3, seed=seed)
            out = torch.full((h * w * 3,), -1.0, dtype=torch.float32, device="cuda:0")
            torch.cuda.synchronize()
            st = aqua.Stats()
            status = lib.aqua_render_noalloc(ctx.handle, scene.handle, ctypes.byref(cfg),
                                             ctypes.c_void_p(out.data_ptr()), ctypes.byref(st))
            assert status == aqua.OK, lib.aqua_last_error(ctx.handle)
            assert st.paths == w * h * spp
            # No per-context workspace was allocated by the no-allocation calls.
            assert ctx.workspace_bytes() == 0
            noalloc_images.append((cfg, out.cpu().numpy().reshape(h, w, 3)))
        for (cfg, img), (w, h) in zip(noalloc_images, [(160, 120), (96, 64)]):
            scene.set_resolution(w, h)
            # The existing entry point, with one path slot per pixel like the
            # no-allocation variant (no sample replicas).
            ref, _ = ctx.render(scene, cfg, tuning=ctx.tuning(replicas=1))
            assert np.isfinite(img).all()
            assert rel_mse(img, ref) < TOL
            assert np.array_equal(img, ref)
        scene.free()


def test_noalloc_refuses_images_above_the_limit():
    torch = pytest.importorskip("torch")
    import aqua

    with aqua.Context(device=0) as ctx:
        scene = ctx.procedural(1, seed=0, width=1024, height=1024)  # 2^20 pixels > 2^19
        cfg = ctx.integrator(spp=1, max_depth=2, seed=0)
        out = torch.zeros(16, dtype=torch.float32, device="cuda:0")
        status = ctx.lib.aqua_render_noalloc(ctx.handle, scene.handle, ctypes.byref(cfg),
                                             ctypes.c_void_p(out.data_ptr()), None)
        assert status == aqua.ERR_INVALID_ARG
        assert b"scratch limit" in ctx.lib.aqua_last_error(ctx.handle)
        scene.free()


def test_noalloc_several_pixels_per_slot_against_the_oracle():
    """512x512 = 2^18 pixels on 2^16 slots: slot s runs pixels s, s + 2^16,
    s + 2^17 and s + 3 * 2^16 in turn. Sample-matched (same seed, same PCG32
    stream per pixel) against the FP64 oracle, and bit-equal to aqua_render
    with one replica."""
    torch = pytest.importorskip("torch")
    import aqua
    import pyoracle

    w = h = 512
    spp = 2
    with aqua.Context(device=0) as ctx:
        lib = ctx.lib
        scene = ctx.procedural(2, seed=0, width=w, height=h)
        cfg = ctx.integrator(spp=spp, max_depth=8, rr_depth=3, seed=5)
        out = torch.full((h * w * 3,), -1.0, dtype=torch.float32, device="cuda:0")
        torch.cuda.synchronize()
        st = aqua.Stats()
        status = lib.aqua_render_noalloc(ctx.handle, scene.handle, ctypes.byref(cfg),
                                         ctypes.c_void_p(out.data_ptr()), ctypes.byref(st))
        assert status == aqua.OK, lib.aqua_last_error(ctx.handle)
        assert st.paths == w * h * spp
        img = out.cpu().numpy().reshape(h, w, 3)
        assert np.isfinite(img).all()
        o = pyoracle.OracleScene.from_aqua(scene)
        ref, ost = o.render(spp, 8, seed=5, precision=64)
        assert rel_mse(img, ref) < TOL
        assert abs(st.ext_rays - ost[1]) / ost[1] < 2e-3
        assert abs(st.shadow_rays - ost[2]) / ost[2] < 2e-3
        again, _ = ctx.render(scene, cfg, tuning=ctx.tuning(replicas=1))
        assert np.array_equal(img, again)
        scene.free()


@pytest.mark.parametrize("max_depth,rr_depth", [(251, 3), (-1, 3), (8, -1), (8, 251)])
def test_noalloc_refuses_depths_out_of_range(max_depth, rr_depth):
    torch = pytest.importorskip("torch")
    import aqua

    with aqua.Context(device=0) as ctx:
        scene = ctx.procedural(1, seed=0, width=16, height=16)
        cfg = ctx.integrator(spp=1, max_depth=max_depth, rr_depth=rr_depth, seed=0)
        out = torch.zeros(16 * 16 * 3, dtype=torch.float32, device="cuda:0")
        status = ctx.lib.aqua_render_noalloc(ctx.handle, scene.handle, ctypes.byref(cfg),
                                             ctypes.c_void_p(out.data_ptr()), None)
        assert status == aqua.ERR_INVALID_ARG
        assert b"_depth must be in [0, 250]" in ctx.lib.aqua_last_error(ctx.handle)
        # aqua_render refuses the same settings.
        with pytest.raises(aqua.AquaError):
            ctx.render(scene, cfg)
        scene.free()
