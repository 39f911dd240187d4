"""Traversal parity on the GPU: aqua_trace against the CPU oracle.

The oracle walks the same flattened BVH with the same FP32 operations, so
closest-hit ids, distances, barycentrics and the per-ray work counters must
be bit-identical; the FP64 brute force checks the answers themselves.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from conftest import random_rays

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cornell(gpu_ctx):
    import pyoracle

    s = gpu_ctx.procedural(2, seed=0, width=64, height=64)
    yield s, pyoracle.OracleScene.from_aqua(s)
    s.free()


@pytest.fixture(scope="module")
def interior(gpu_ctx):
    import pyoracle

    s = gpu_ctx.procedural(3, seed=0, width=96, height=54)
    yield s, pyoracle.OracleScene.from_aqua(s)
    s.free()


def camera_rays(orc, w, h):
    """Pinhole rays through pixel centres of the scene camera."""
    c = orc.s.cam
    th = np.tan(0.5 * np.radians(c.fov_deg))
    ys, xs = np.mgrid[0:h, 0:w]
    sx = (2 * (xs + 0.5) / w - 1) * th * (w / h)
    sy = (1 - 2 * (ys + 0.5) / h) * th
    R, U, B = np.array(c.right), np.array(c.up), np.array(c.back)
    d = sx[..., None] * R + sy[..., None] * U - B
    rays = np.zeros((w * h, 8), np.float32)
    rays[:, 0:3] = np.array(c.pos)
    rays[:, 4:7] = d.reshape(-1, 3)
    rays[:, 7] = np.inf
    return rays


def assert_bit_exact(ctx, scene, orc, rays, any_hit=False):
    """Both device traversals against the FP32 CPU walk: the counting one
    visits in the canonical order (work counts must match too), the fast one
    postpones leaves warp-wide (results must match)."""
    ot, ou, ov, oprim, ocnt = orc.trace_bvh_f32(rays, any_hit=any_hit)
    for count in (True, False):
        t, u, v, prim, cnt = ctx.trace(scene, rays, any_hit=any_hit, count=count)
        assert np.array_equal(prim, oprim), f"{int((prim != oprim).sum())} ids differ (count={count})"
        assert np.array_equal(t.view(np.uint32), ot.view(np.uint32))
        assert np.array_equal(u.view(np.uint32), ou.view(np.uint32))
        assert np.array_equal(v.view(np.uint32), ov.view(np.uint32))
        if count:
            assert cnt.node_visits == int(ocnt[:, 0].sum())
            assert cnt.tri_tests == int(ocnt[:, 1].sum())
    return prim, t


def test_cornell_random_rays_bit_exact(gpu_ctx, cornell):
    s, o = cornell
    rays = random_rays(200_000, -0.6, 1.1, seed=1)
    prim, t = assert_bit_exact(gpu_ctx, s, o, rays)
    assert 0.2 < (prim >= 0).mean() < 0.9


def test_cornell_camera_rays_bit_exact(gpu_ctx, cornell):
    s, o = cornell
    rays = camera_rays(o, 256, 256)
    prim, _ = assert_bit_exact(gpu_ctx, s, o, rays)
    assert (prim >= 0).mean() > 0.7


def test_cornell_against_fp64_brute_force(gpu_ctx, cornell):
    s, o = cornell
    rays = random_rays(50_000, -0.6, 1.1, seed=2)
    t, _, _, prim, _ = gpu_ctx.trace(s, rays)
    td, _, _, pd = o.trace_brute_f64(rays)
    assert np.array_equal(prim >= 0, pd >= 0)
    hit = prim >= 0
    # Same closest surface: distance within 1e-5 of the scene scale (1) or of t.
    assert np.all(np.abs(t[hit] - td[hit]) <= 1e-5 * np.maximum(td[hit], 1.0))
    # Different ids only where two triangles overlap at the same distance
    # (box bottoms lying on the floor).
    diff = hit & (prim != pd)
    assert diff.mean() < 0.01
    assert np.all(np.abs(t[diff] - td[diff]) <= 1e-5 * np.maximum(td[diff], 1.0))


def test_any_hit_matches_oracle(gpu_ctx, cornell):
    s, o = cornell
    rays = random_rays(100_000, -0.6, 1.1, seed=3)
    rays[:, 7] = np.random.default_rng(3).uniform(0.05, 2.0, rays.shape[0])
    prim, _ = assert_bit_exact(gpu_ctx, s, o, rays, any_hit=True)
    _, _, _, bprim = o.trace_brute_f32(rays, any_hit=True)
    assert np.array_equal(prim, bprim)
    assert set(np.unique(prim)) <= {-1, 1}


def test_axis_aligned_and_interval_edges(gpu_ctx, cornell):
    s, o = cornell
    rng = np.random.default_rng(4)
    n = 30_000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-0.4, 0.9, (n, 3))
    axis = rng.integers(0, 3, n)
    sign = rng.choice([-1.0, 1.0], n)
    rays[np.arange(n), 4 + axis] = sign  # exactly axis-aligned directions
    rays[:, 3] = rng.choice([0.0, 0.1, 0.5], n)
    rays[:, 7] = rng.choice([np.inf, 0.3, 0.05], n)
    rays[:100, 3], rays[:100, 7] = 1.0, 0.5  # empty interval
    prim, _ = assert_bit_exact(gpu_ctx, s, o, rays)
    assert np.all(prim[:100] == -1)


def test_interior_million_triangles_bit_exact(gpu_ctx, interior):
    s, o = interior
    info = s.info()
    assert info.num_triangles > 1_000_000
    rays = random_rays(100_000, -9.0, 3.9, seed=5)
    rays[:, 1] = np.random.default_rng(5).uniform(0.05, 3.9, rays.shape[0])
    assert_bit_exact(gpu_ctx, s, o, rays)
    rays = camera_rays(o, 192, 108)
    prim, _ = assert_bit_exact(gpu_ctx, s, o, rays)
    assert (prim >= 0).mean() > 0.99  # closed room


def test_zero_rays_and_empty_scene(gpu_ctx, tmp_path):
    scene_json = {"named_bsdfs": {}, "camera": {"Perspective": {"res": [8, 8], "fov": 40.0, "lens_radius": 0.0,
                                                                  "focal": 1.0}},
                  "lights": [], "shapes": []}
    p = tmp_path / "empty.json"
    p.write_text(json.dumps(scene_json))
    s = gpu_ctx.load_scene(str(p))
    assert s.info().num_triangles == 0
    rays = random_rays(1000, -1, 1, seed=6)
    t, u, v, prim, _ = gpu_ctx.trace(s, rays)
    assert np.all(prim == -1)
    t, u, v, prim, _ = gpu_ctx.trace(s, rays[:0])
    assert prim.shape == (0,)
    s.free()


def test_device_pointer_path(gpu_ctx, cornell):
    torch = pytest.importorskip("torch")
    import aqua
    import ctypes

    s, o = cornell
    rays = random_rays(10_000, -0.6, 1.1, seed=8)
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.zeros((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = gpu_ctx.lib.aqua_trace(gpu_ctx.handle, s.handle, ctypes.c_void_p(d_rays.data_ptr()), rays.shape[0],
                                ctypes.c_void_p(d_hits.data_ptr()), aqua.TRACE_DEVICE_PTRS, None)
    assert st == 0
    h = d_hits.cpu().numpy()
    ot, _, _, oprim, _ = o.trace_bvh_f32(rays)
    assert np.array_equal(h[:, 3].view(np.int32), oprim)
    assert np.array_equal(h[:, 0], ot)


@pytest.mark.parametrize("kind", ["coincident", "chain", "cloud"])
def test_degenerate_triangle_sets_bit_exact(gpu_ctx, tmp_path, kind):
    """Ties and degenerate trees: 37 coincident triangles (every hit a tie,
    broken by the smaller scene index), a chain of thin triangles whose sizes
    span six decades, a dense random cloud. Closest and any hit, both device
    traversals against the oracle's walk."""
    import pyoracle
    from test_bvh_structure import aimed_rays, soup
    from test_loaders import principled, scene_json, write_mesh

    rng = np.random.default_rng(11)
    v = soup(kind, rng)
    verts = v.reshape(-1, 3)
    idx = np.arange(verts.shape[0]).reshape(-1, 3)
    write_mesh(tmp_path / "m.mesh", verts.tolist(), idx.tolist(), normals=False)
    p = tmp_path / "s.json"
    p.write_text(json.dumps(scene_json([("m.mesh", "w")], {"w": principled()})))
    s = gpu_ctx.load_scene(str(p))
    o = pyoracle.OracleScene.from_aqua(s)
    rays = aimed_rays(v.astype(np.float32), 20_000, rng)
    prim, _ = assert_bit_exact(gpu_ctx, s, o, rays)
    assert np.mean(prim >= 0) > 0.5
    if kind == "coincident":
        assert set(prim[prim >= 0].tolist()) == {0}
    assert_bit_exact(gpu_ctx, s, o, rays, any_hit=True)
    s.free()


def test_node_formats_give_identical_hits_and_images(gpu_ctx):
    """The interior walked through its full-precision and its quantized nodes:
    every closest and any hit identical bit for bit (decoded boxes contain
    the true ones, and culling never depends on a box's slack), so images
    are identical too; the quantized walk counts match the oracle's."""
    import aqua
    import pyoracle
    from conftest import random_rays

    s = gpu_ctx.procedural(3, seed=0, width=64, height=36)
    s.set_bvh_format(aqua.BVH_QUANTIZED)
    assert s.info().bvh_format == aqua.BVH_QUANTIZED
    rays = random_rays(20000, -9.0, 3.9, seed=9)
    tq, uq, vq, pq, cq = gpu_ctx.trace(s, rays, count=True)
    oq = pyoracle.OracleScene.from_aqua(s).trace_bvh_f32(rays)
    assert np.array_equal(pq, oq[3]) and np.array_equal(tq.view(np.uint32), oq[0].view(np.uint32))
    assert cq.node_visits == int(oq[4][:, 0].sum()) and cq.tri_tests == int(oq[4][:, 1].sum())
    cfg = gpu_ctx.integrator(spp=8, max_depth=8, rr_depth=3, seed=6)
    img_q, _ = gpu_ctx.render(s, cfg)
    s.set_bvh_format(aqua.BVH_FULL)
    assert s.info().bvh_format == aqua.BVH_FULL
    tf, uf, vf, pf, cf = gpu_ctx.trace(s, rays, count=True)
    assert np.array_equal(pq, pf)
    assert np.array_equal(tq.view(np.uint32), tf.view(np.uint32))
    assert np.array_equal(uq.view(np.uint32), uf.view(np.uint32))
    assert cq.node_visits >= cf.node_visits
    img_f, _ = gpu_ctx.render(s, cfg)
    assert np.array_equal(img_q, img_f)
    s.free()
