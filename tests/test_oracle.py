"""The CPU oracle itself, on CPU: known answers (PCG32, sRGB), the BVH walk
against brute force, FP32 vs FP64 path tracing, and the network's analytic
gradient against finite differences."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

import pyoracle
from conftest import random_rays, reference_scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FACTS = json.load(open(os.path.join(GOLDEN, "reference_facts.json")))


def test_pcg32_known_answer():
    # pcg32_srandom(42, 54), first six outputs of the PCG reference demo.
    assert [hex(v) for v in pyoracle.pcg32_sequence(42, 54, 6)] == [
        "0xa15c02b7", "0x7b47f409", "0xba1d3330", "0x83d2f293", "0xbfa4784b", "0xcbed606e"]


def test_srgb_decode_matches_reference_mtl():
    # cbox.json Srgb colours decode to CornellBox-Original.mtl Kd values.
    for name, srgb in FACTS["cbox"]["srgb"].items():
        lin = [pyoracle.srgb_to_linear(c) for c in srgb]
        np.testing.assert_allclose(lin, FACTS["mtl"][name]["Kd"], atol=1.5e-3)


@pytest.fixture(scope="module")
def cornell_orc(host_ctx):
    s = host_ctx.procedural(2, seed=0, width=32, height=32)
    yield pyoracle.OracleScene.from_aqua(s)
    s.free()


@pytest.fixture(scope="module")
def interior_orc(host_ctx):
    s = host_ctx.procedural(3, seed=0, width=32, height=18)
    yield pyoracle.OracleScene.from_aqua(s)
    s.free()


def test_bvh_walk_equals_brute_force_cornell(cornell_orc):
    rays = random_rays(50_000, -0.6, 1.1, seed=1)
    t, u, v, p, cnt = cornell_orc.trace_bvh_f32(rays)
    tb, ub, vb, pb = cornell_orc.trace_brute_f32(rays)
    assert np.array_equal(p, pb)
    assert np.array_equal(t.view(np.uint32), tb.view(np.uint32))
    assert np.array_equal(u.view(np.uint32), ub.view(np.uint32))
    assert (cnt[:, 0] >= 1).all()


def test_bvh_walk_equals_brute_force_interior(interior_orc):
    rays = random_rays(300, -9.0, 3.9, seed=2)
    t, u, v, p, _ = interior_orc.trace_bvh_f32(rays)
    tb, ub, vb, pb = interior_orc.trace_brute_f32(rays)
    assert np.array_equal(p, pb)
    assert np.array_equal(t.view(np.uint32), tb.view(np.uint32))


def test_fp32_render_tracks_fp64(cornell_orc):
    a, sa = cornell_orc.render(32, 8, seed=3, precision=64)
    b, sb = cornell_orc.render(32, 8, seed=3, precision=32)
    assert pyoracle.rel_mse(b, a) < 1e-4
    assert sa[0] == sb[0] == 32 * 32 * 32


def test_render_is_deterministic_and_pixel_range(cornell_orc):
    a, _ = cornell_orc.render(8, 5, seed=9, precision=64)
    b, _ = cornell_orc.render(8, 5, seed=9, precision=64, pixel_begin=100, pixel_end=200)
    flat_a, flat_b = a.reshape(-1, 3), b.reshape(-1, 3)
    assert np.array_equal(flat_a[100:200], flat_b[100:200])
    assert not flat_b[:100].any() and not flat_b[200:].any()


def _rand_net(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    w = (rng.uniform(-1, 1, pyoracle.NRC_PARAMS) * np.sqrt(6 / 64) * scale).astype(np.float32)
    return w


def test_mlp_gradient_matches_finite_differences():
    rng = np.random.default_rng(4)
    w = _rand_net(1)
    x = rng.uniform(-1, 1, (6, 64)).astype(np.float32)
    t = rng.uniform(0, 2, (6, 3)).astype(np.float32)
    g, loss = pyoracle.mlp_grad(w, x, t, emulate_bf16=False)
    # The loss with its denominator frozen at the current outputs.
    y0 = pyoracle.mlp_forward_f64(w, x)
    den = y0 ** 2 + 0.01

    def frozen_loss(wp):
        y = pyoracle.mlp_forward_f64(wp, x)
        return float(np.mean((y - t) ** 2 / den))

    assert abs(frozen_loss(w) - loss) < 1e-6 * max(loss, 1)
    idx = np.concatenate([rng.integers(0, 5 * 4096, 40), 5 * 4096 + rng.integers(0, 192, 10)])
    for i in idx:
        h = 2e-3 * max(abs(float(w[i])), 1e-2)
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        h_eff = float(wp[i]) - float(wm[i])  # exact step after float32 rounding
        fd = (frozen_loss(wp) - frozen_loss(wm)) / h_eff
        assert abs(fd - g[i]) <= 2e-3 * abs(g[i]) + 1e-7, (i, fd, g[i])


def test_mlp_bf16_emulation_is_close_to_fp64():
    rng = np.random.default_rng(5)
    w = _rand_net(2)
    x = rng.uniform(-1, 1, (256, 64)).astype(np.float32)
    y64 = pyoracle.mlp_forward(w, x, emulate_bf16=False)
    y16 = pyoracle.mlp_forward(w, x, emulate_bf16=True)
    assert np.abs(y16 - y64).max() < 0.05 * (np.abs(y64).max() + 1e-3)


def test_encoding_shape_and_ranges():
    rng = np.random.default_rng(6)
    raw = np.zeros((500, 16), np.float32)
    raw[:, 0:3] = rng.uniform(-2, 2, (500, 3))
    for sl in (slice(3, 6), slice(6, 9)):
        v = rng.normal(size=(500, 3))
        raw[:, sl] = v / np.linalg.norm(v, axis=1, keepdims=True)
    raw[:, 9] = rng.uniform(0, 1, 500)
    raw[:, 10:16] = rng.uniform(0, 1, (500, 6))
    x = pyoracle.nrc_encode(raw, [-2, -2, -2], [2, 2, 2])
    assert x.shape == (500, 64)
    assert np.all(np.abs(x[:, :48]) <= 1.0)
    assert np.all((x[:, 48:58] > 0) & (x[:, 48:58] <= 1.0))  # one-blob bins
    np.testing.assert_allclose(x[:, 58], raw[:, 9], rtol=1e-7)
    np.testing.assert_array_equal(x[:, 59:62], raw[:, 10:13])
    lum = 0.2126 * raw[:, 13] + 0.7152 * raw[:, 14] + 0.0722 * raw[:, 15]
    np.testing.assert_allclose(x[:, 62], lum, rtol=1e-6)
    assert np.all(x[:, 63] == 1.0)
    # sin^2 + cos^2 = 1 for every position octave
    np.testing.assert_allclose(x[:, 0:48:2] ** 2 + x[:, 1:48:2] ** 2, 1.0, atol=1e-6)


@pytest.mark.skipif(reference_scene("room.json") is None, reason="reference living-room scene not staged")
def test_bvh_walk_equals_brute_force_reference_room(host_ctx):
    """The reference's own living-room geometry (room.json, 394,269 triangles
    from 152 BSON meshes): the four-wide BVH walk finds exactly the brute-force
    closest hits for rays from the camera and from random points inside the
    room, closest and any hit."""
    s = host_ctx.load_scene(reference_scene("room.json"), allow_missing=True)
    o = pyoracle.OracleScene.from_aqua(s)
    verts = s.triangles()[0].reshape(-1, 3)
    lo, hi = verts.min(0), verts.max(0)
    rng = np.random.default_rng(4)
    rays = np.zeros((400, 8), np.float32)
    rays[:200, 0:3] = np.array(s.camera().pos)
    rays[200:, 0:3] = lo + rng.uniform(0.05, 0.95, (200, 3)) * (hi - lo)
    rays[:, 4:7] = rng.normal(size=(400, 3))
    rays[:, 7] = np.inf
    t, u, v, p, _ = o.trace_bvh_f32(rays)
    tb, ub, vb, pb = o.trace_brute_f32(rays)
    assert np.array_equal(p, pb)
    assert np.array_equal(t.view(np.uint32), tb.view(np.uint32))
    assert np.mean(p >= 0) > 0.5
    occ = o.trace_bvh_f32(rays, any_hit=True)[3]
    assert np.array_equal(occ >= 0, pb >= 0)
    s.free()


def test_render_pixel_list_equals_full_render(cornell_orc):
    """The pixel-list render (every k-th row, used for uniform row samples of
    large images) gives each pixel exactly what the full render gives it."""
    full, st = cornell_orc.render(8, 8, seed=3, precision=32)
    rows = [0, 5, 17, 31]
    part, pst = cornell_orc.render_rows(rows, 8, 8, seed=3, precision=32)
    assert np.array_equal(part, full[rows])
    assert 0 < pst[0] == 8 * 32 * len(rows) < st[0]
    with pytest.raises(RuntimeError):
        cornell_orc.render_pixels([32 * 32], 1, 1)


def test_quantized_walk_equals_brute_force_interior(host_ctx):
    """The interior with quantized nodes: the oracle decodes them and its
    walk still equals brute force, closest and any hit."""
    import aqua

    s = host_ctx.procedural(3, seed=0, width=32, height=18)
    s.set_bvh_format(aqua.BVH_QUANTIZED)
    assert s.info().bvh_format == aqua.BVH_QUANTIZED
    o = pyoracle.OracleScene.from_aqua(s)
    rays = random_rays(400, -9.0, 3.9, seed=5)
    t, u, v, p, _ = o.trace_bvh_f32(rays)
    tb, ub, vb, pb = o.trace_brute_f32(rays)
    assert np.array_equal(p, pb)
    assert np.array_equal(t.view(np.uint32), tb.view(np.uint32))
    occ = o.trace_bvh_f32(rays, any_hit=True)[3]
    assert np.array_equal(occ >= 0, pb >= 0)
    s.free()
