"""Image parity on the GPU: the wavefront renderer against the FP64 oracle.

relMSE = mean over pixels and channels of (x - r)^2 / (r^2 + 1e-2).
Sample-matched tests use the same seed on both sides (same PCG32 stream per
pixel, same random numbers per bounce), so the images agree far below the
1e-3 bar; the converged test uses independent seeds and high spp.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-3  # relMSE bar against the FP64 oracle


def rel_mse(x, r):
    import pyoracle

    return pyoracle.rel_mse(x, r)


@pytest.mark.parametrize("config,depth", [(1, 5), (2, 8)])
def test_cornell_sample_matched(gpu_ctx, config, depth):
    import pyoracle

    s = gpu_ctx.procedural(config, seed=0, width=48, height=48)
    o = pyoracle.OracleScene.from_aqua(s)
    cfg = gpu_ctx.integrator(spp=128, max_depth=depth, rr_depth=3, seed=11)
    img, st = gpu_ctx.render(s, cfg)
    ref, ost = o.render(128, depth, seed=11, precision=64)
    err = rel_mse(img, ref)
    assert err < TOL, err
    assert st.paths == 48 * 48 * 128 == int(ost[0])
    # Same random numbers: ray counts agree to within rare FP32/FP64 divergences.
    assert abs(st.ext_rays - ost[1]) / ost[1] < 2e-3
    assert abs(st.shadow_rays - ost[2]) / ost[2] < 2e-3
    s.free()


def test_cornell_converged_independent_seeds(gpu_ctx):
    import pyoracle

    s = gpu_ctx.procedural(2, seed=0, width=24, height=24)
    o = pyoracle.OracleScene.from_aqua(s)
    cfg = gpu_ctx.integrator(spp=16384, max_depth=8, rr_depth=3, seed=101)
    img, _ = gpu_ctx.render(s, cfg)
    ref, _ = o.render(16384, 8, seed=202, precision=64)
    err = rel_mse(img, ref)
    assert err < TOL, err
    s.free()


def test_interior_textured_sample_matched(gpu_ctx):
    import pyoracle

    s = gpu_ctx.procedural(3, seed=0, width=64, height=36)
    o = pyoracle.OracleScene.from_aqua(s)
    cfg = gpu_ctx.integrator(spp=16, max_depth=8, rr_depth=3, seed=3)
    img, st = gpu_ctx.render(s, cfg)
    ref, _ = o.render(16, 8, seed=3, precision=64)
    err = rel_mse(img, ref)
    assert err < TOL, err
    assert img.mean() > 0.01
    s.free()


def test_launch_shape_does_not_change_the_image(gpu_ctx):
    s = gpu_ctx.procedural(2, seed=0, width=40, height=30)
    cfg = gpu_ctx.integrator(spp=32, max_depth=8, rr_depth=3, seed=9)
    base, _ = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(replicas=1))
    for kw in [dict(slots=1000), dict(slots=37), dict(sort_by_material=0), dict(block_trace=64, block_shade=32),
               dict(slots=333, sort_by_material=1, blocks_per_sm=2)]:
        img, _ = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(replicas=1, **kw))
        assert np.array_equal(img.view(np.uint32), base.view(np.uint32)), kw
    s.free()


def test_sample_replicas(gpu_ctx):
    """Small images run several slots per pixel, each on its own film copy:
    deterministic for a given replica count, equal up to summation order
    across counts, and the default for images below 2^24 pixels."""
    import pyoracle

    s = gpu_ctx.procedural(2, seed=0, width=40, height=30)
    cfg = gpu_ctx.integrator(spp=32, max_depth=8, rr_depth=3, seed=9)
    one, st1 = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(replicas=1))
    four, st4 = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(replicas=4))
    again, _ = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(replicas=4, sort_by_material=0, block_trace=64))
    auto, sta = gpu_ctx.render(s, cfg)
    assert np.array_equal(four, again)
    np.testing.assert_allclose(four, one, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(auto, one, rtol=1e-5, atol=1e-6)
    assert st1.paths == st4.paths == sta.paths == 40 * 30 * 32
    # fewer iterations: the same work spread over more slots
    assert sta.iterations < st1.iterations
    o = pyoracle.OracleScene.from_aqua(s)
    ref, _ = o.render(32, 8, seed=9, precision=64)
    assert pyoracle.rel_mse(auto, ref) < TOL
    s.free()


def test_depth_zero_sees_only_emitters(gpu_ctx):
    import pyoracle

    s = gpu_ctx.procedural(1, seed=0, width=64, height=64)
    cfg = gpu_ctx.integrator(spp=4, max_depth=0, rr_depth=3, seed=1)
    img, st = gpu_ctx.render(s, cfg)
    assert st.shadow_rays == 0
    lit = img.max(axis=2) > 0
    assert 0 < lit.mean() < 0.05  # only the ceiling light is visible
    o = pyoracle.OracleScene.from_aqua(s)
    ref, _ = o.render(4, 0, seed=1, precision=64)
    assert rel_mse(img, ref) < TOL
    s.free()


def test_progressive_accumulation_matches_one_call(gpu_ctx):
    import aqua

    s = gpu_ctx.procedural(2, seed=0, width=32, height=32)
    full, _ = gpu_ctx.render(s, gpu_ctx.integrator(spp=16, max_depth=8, seed=4))
    acc = np.zeros_like(full)
    for off in range(0, 16, 4):
        gpu_ctx.render(s, gpu_ctx.integrator(spp=4, max_depth=8, seed=4, spp_offset=off), out=acc,
                       flags=aqua.RENDER_ACCUMULATE)
    np.testing.assert_allclose(acc / 16, full, rtol=1e-5, atol=1e-6)
    s.free()


def test_invalid_arguments_raise(gpu_ctx):
    import aqua

    s = gpu_ctx.procedural(1, seed=0, width=8, height=8)
    with pytest.raises(aqua.AquaError) as e:
        gpu_ctx.render(s, gpu_ctx.integrator(spp=0))
    assert e.value.status == aqua.ERR_INVALID_ARG
    with pytest.raises(aqua.AquaError) as e:
        gpu_ctx.render(s, gpu_ctx.integrator(spp=1), tuning=gpu_ctx.tuning(block_trace=100))
    assert e.value.status == aqua.ERR_INVALID_ARG
    s.free()


@pytest.mark.parametrize("config", [2, 3])
def test_persistent_kernel_matches_wavefront(gpu_ctx, config):
    """The persistent kernel (one launch, a path per lane regenerated in
    place) renders the same image as the wavefront: same random numbers per
    sample and bounce, contributions summed per pixel in the same order, so
    only the per-pixel film summation (one sum vs film += per event) differs.
    Ray counts are equal."""
    import aqua
    import pyoracle

    s = gpu_ctx.procedural(config, seed=0, width=64, height=48)
    cfg = gpu_ctx.integrator(spp=32, max_depth=8, rr_depth=3, seed=5)
    wf, sw = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(kernel=aqua.KERNEL_WAVEFRONT))
    pk, sp = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(kernel=aqua.KERNEL_PERSISTENT))
    np.testing.assert_allclose(pk, wf, rtol=1e-5, atol=1e-6)
    assert sp.paths == sw.paths == 64 * 48 * 32
    assert (sp.ext_rays, sp.shadow_rays) == (sw.ext_rays, sw.shadow_rays)
    assert sp.total_launches == 1 and sp.iterations == 0
    again, _ = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(kernel=aqua.KERNEL_PERSISTENT, block_trace=256,
                                                            blocks_per_sm=2))
    assert np.array_equal(again, pk)  # the launch shape does not change the image
    # Flags the persistent kernel does not serve run on the wavefront.
    _, sc = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(kernel=aqua.KERNEL_PERSISTENT), flags=aqua.RENDER_COUNT)
    assert sc.node_visits > 0 and sc.iterations > 0
    o = pyoracle.OracleScene.from_aqua(s)
    ref, _ = o.render(32, 8, seed=5, precision=64)
    assert pyoracle.rel_mse(pk, ref) < TOL
    s.free()


def test_autotune_picks_a_kernel(gpu_ctx):
    import aqua

    s = gpu_ctx.procedural(2, seed=0, width=96, height=64)
    cfg = gpu_ctx.integrator(spp=64, max_depth=8, rr_depth=3, seed=3)
    t = gpu_ctx.autotune(s, cfg)
    assert t.kernel in (aqua.KERNEL_WAVEFRONT, aqua.KERNEL_PERSISTENT)
    img, st = gpu_ctx.render(s, cfg, tuning=t)
    ref, _ = gpu_ctx.render(s, cfg)
    np.testing.assert_allclose(img, ref, rtol=1e-5, atol=1e-6)
    with pytest.raises(aqua.AquaError) as e:
        gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(kernel=7))
    assert e.value.status == aqua.ERR_INVALID_ARG
    s.free()


def smooth_sphere_scene(tmp_path, with_normals=True):
    """A UV sphere with vertex normals on a flat floor, lit by an emissive
    quad and a point light, written as BSON meshes + scene JSON."""
    import json
    import os
    import sys

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import test_loaders as tl

    nu, nv, r, c = 24, 12, 0.5, np.array([0.0, 0.55, 0.0])
    verts, nrms, idx = [], [], []
    for j in range(nv + 1):
        th = np.pi * j / nv
        for i in range(nu):
            ph = 2 * np.pi * i / nu
            d = np.array([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)])
            verts.append(c + r * d)
            nrms.append(d)
    for j in range(nv):
        for i in range(nu):
            a, b = j * nu + i, j * nu + (i + 1) % nu
            idx += [[a, a + nu, b], [b, a + nu, b + nu]]
    tl.write_mesh(tmp_path / "sphere.mesh", verts, idx, normals=nrms if with_normals else False)
    tl.write_mesh(tmp_path / "floor.mesh", [[-3, 0, -3], [3, 0, -3], [3, 0, 3], [-3, 0, 3]], [[0, 2, 1], [0, 3, 2]],
                  normals=False)
    tl.write_mesh(tmp_path / "lamp.mesh", [[-0.4, 2.2, -0.4], [0.4, 2.2, -0.4], [0.4, 2.2, 0.4], [-0.4, 2.2, 0.4]],
                  [[0, 1, 2], [0, 2, 3]], normals=False)
    bsdfs = {"ball": tl.principled({"Float3": [0.7, 0.4, 0.2]}, metallic=0.0, roughness=0.3, specular=0.5),
             "floor": tl.principled({"Float3": [0.5, 0.5, 0.5]}),
             "lamp": tl.principled({"Float3": [0.0, 0.0, 0.0]}, emission=8.0)}
    js = tl.scene_json([("sphere.mesh", "ball"), ("floor.mesh", "floor"), ("lamp.mesh", "lamp")], bsdfs,
                       lights=[{"Point": {"pos": [1.5, 1.5, 1.5], "emission": {"Float3": [3.0, 3.0, 3.0]}}}],
                       res=(48, 36))
    path = tmp_path / ("smooth.json" if with_normals else "flat.json")
    path.write_text(json.dumps(js))
    return str(path)


def test_shading_normals_sample_matched(gpu_ctx, tmp_path):
    """Interpolated vertex normals against the FP64 oracle (same seeds): the
    shading frame and the NEE cosine use them, the geometric normal guards
    against light leaks; a faceted copy of the scene renders differently."""
    import aqua
    import pyoracle

    s = gpu_ctx.load_scene(smooth_sphere_scene(tmp_path))
    assert s.normals() is not None
    cfg = gpu_ctx.integrator(spp=64, max_depth=5, rr_depth=3, seed=21)
    img, st = gpu_ctx.render(s, cfg)
    o = pyoracle.OracleScene.from_aqua(s)
    ref, ost = o.render(64, 5, seed=21, precision=64)
    assert rel_mse(img, ref) < TOL
    assert abs(st.ext_rays - ost[1]) / ost[1] < 5e-3
    assert abs(st.shadow_rays - ost[2]) / ost[2] < 5e-3
    pk, _ = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning(kernel=aqua.KERNEL_PERSISTENT))
    np.testing.assert_allclose(pk, img, rtol=1e-5, atol=1e-6)
    f = gpu_ctx.load_scene(smooth_sphere_scene(tmp_path, with_normals=False))
    assert f.normals() is None
    flat, _ = gpu_ctx.render(f, cfg)
    assert rel_mse(flat, img) > 1e-4  # same seeds: the whole difference is the normals
    s.free()
    f.free()


def test_stats_and_stage_timing(gpu_ctx):
    import aqua

    s = gpu_ctx.procedural(2, seed=0, width=64, height=64)
    img, st = gpu_ctx.render(s, gpu_ctx.integrator(spp=8, max_depth=8, seed=2),
                             flags=aqua.RENDER_STAGE_TIMING | aqua.RENDER_COUNT)
    assert st.paths == 64 * 64 * 8
    assert st.trace_ms > 0 and st.shade_ms > 0 and st.shadow_ms > 0
    assert st.device_ms >= st.trace_ms
    assert st.node_visits > st.ext_rays and st.tri_tests > 0
    s.free()


def test_chained_launches_match_event_separated_ones(gpu_ctx):
    """The wavefront stages are chained by programmatic dependent launch;
    stage timing records events between the launches of every 8th iteration,
    which separates those launches. The image is the same bit for bit."""
    import aqua

    s = gpu_ctx.procedural(2, seed=0, width=256, height=256)
    cfg = gpu_ctx.integrator(spp=64, max_depth=8, rr_depth=3, seed=4)
    tune = gpu_ctx.tuning(replicas=1)
    chained, st = gpu_ctx.render(s, cfg, tuning=tune)
    timed, st2 = gpu_ctx.render(s, cfg, tuning=tune, flags=aqua.RENDER_STAGE_TIMING)
    assert st.iterations > 100 and st2.iterations == st.iterations
    assert np.array_equal(chained.view(np.uint32), timed.view(np.uint32))
    s.free()


def test_allocation_failure_is_reported():
    import aqua

    # The first device allocation of this context (the scene image) fails.
    with aqua.Context(device=0, fail_alloc_after=1) as c:
        with pytest.raises(aqua.AquaError) as e:
            c.procedural(1, seed=0, width=8, height=8)
        assert e.value.status == aqua.ERR_OOM and "fail_alloc_after" in e.value.message
    # The second one (the render workspace) fails; the context stays usable.
    with aqua.Context(device=0, fail_alloc_after=2) as c:
        s = c.procedural(1, seed=0, width=8, height=8)
        with pytest.raises(aqua.AquaError) as e:
            c.render(s, c.integrator(spp=1))
        assert e.value.status == aqua.ERR_OOM
        s.free()


def test_row_subset_equals_rows_of_the_full_image(gpu_ctx):
    """With row_step > 1 only every row_step-th row is rendered, and each
    pixel keeps its full-image random-number stream: the rows equal the same
    rows of a full render bit for bit (one slot per pixel on both sides)."""
    import aqua

    s = gpu_ctx.procedural(3, seed=0, width=96, height=54)
    cfg = gpu_ctx.integrator(spp=8, max_depth=8, rr_depth=3, seed=4)
    one = gpu_ctx.tuning(replicas=1)
    full, _ = gpu_ctx.render(s, cfg, tuning=one)
    for begin, step in [(0, 2), (3, 7), (5, 16)]:
        rows = np.arange(begin, 54, step)
        sub = gpu_ctx.integrator(spp=8, max_depth=8, rr_depth=3, seed=4, row_begin=begin, row_step=step)
        out = np.zeros((len(rows), 96, 3), np.float32)
        img, st = gpu_ctx.render(s, sub, tuning=one, out=out)
        assert st.paths == len(rows) * 96 * 8
        assert np.array_equal(img, full[rows])
        auto, _ = gpu_ctx.render(s, sub, out=np.zeros_like(out))  # sample replicas on the small film
        np.testing.assert_allclose(auto, full[rows], rtol=1e-5, atol=1e-6)
    bad = gpu_ctx.integrator(spp=1, max_depth=2, row_begin=4, row_step=3)
    with pytest.raises(aqua.AquaError):
        gpu_ctx.render(s, bad)
    s.free()
