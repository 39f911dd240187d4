"""The four-wide BVH as the library exports it (aqua_scene_export_bvh),
checked structurally on the CPU: every node is reached once from the root and
only forward, every triangle sits in exactly one leaf, each slot's box holds
what lies under it, empty slots are boxes no ray can enter with a leaf of no
triangles behind them, and the deepest traversal stack fits the kernels'
96 entries. Scenes: the procedural ones and triangle sets built to stress
the builder (one triangle, coincident triangles, a long thin chain, a dense
random cloud). No GPU needed."""
from __future__ import annotations

import json

import numpy as np
import pytest

from test_loaders import principled, scene_json, write_mesh

STACK_SLOTS = 96


def check_tree(scene):
    nodes, order = scene.bvh()
    info = scene.info()
    ntri = info.num_triangles
    verts = scene.triangles()[0].reshape(-1, 3, 3)
    n = nodes.shape[0]
    assert n == info.num_bvh_nodes >= 1
    lo = np.stack([nodes[:, 0:4], nodes[:, 8:12], nodes[:, 16:20]], axis=-1)   # [node, slot, axis]
    hi = np.stack([nodes[:, 4:8], nodes[:, 12:16], nodes[:, 20:24]], axis=-1)
    link = nodes[:, 24:28].copy().view(np.int32)
    count = nodes[:, 28:32].copy().view(np.int32)

    # Slots: real ones first, empty ones (+inf box, link ~0, count 0) after.
    empty = (link == -1) & np.all(np.isposinf(lo), axis=2) & np.all(np.isposinf(hi), axis=2)
    real = ~empty
    nreal = real.sum(axis=1)
    assert np.all(nreal >= 2), "every node has at least two children"
    np.testing.assert_array_equal(real, np.arange(4)[None, :] < nreal[:, None])
    assert np.all(count[empty] == 0)
    assert np.all(lo[real] <= hi[real]), "inverted box"

    # Inner links: forward, each node but the root reached exactly once.
    inner = real & (link >= 0)
    par, slot = np.nonzero(inner)
    child = link[inner].astype(np.int64)
    assert np.all(child > par) and np.all(child < n), "links point forward"
    reached = np.bincount(child, minlength=n)
    assert reached[0] == 0 and np.all(reached[1:] == 1)
    # A child's slot boxes lie inside the slot box that points at it.
    clo = np.where(real[:, :, None], lo, np.inf).min(axis=1)
    chi = np.where(real[:, :, None], hi, -np.inf).max(axis=1)
    assert np.all(clo[child] >= lo[par, slot]) and np.all(chi[child] <= hi[par, slot])

    # Depth and stack bound (parents precede children).
    parent = np.full(n, -1, np.int64)
    parent[child] = par
    need = np.zeros(n, np.int64)
    depth = np.ones(n, np.int64)
    for k in range(1, n):
        q = parent[k]
        need[k] = need[q] + nreal[q] - 1
        depth[k] = depth[q] + 1
    max_stack = int((need + nreal - 1).max())
    assert max_stack < STACK_SLOTS
    assert info.bvh_depth == int(depth.max())

    # Leaves: the triangles of every leaf slot, each triangle in one leaf,
    # inside the slot's box.
    leaf = real & (link < 0)
    code = ~link[leaf]
    first, cnt = (code >> 3).astype(np.int64), (code & 7).astype(np.int64)
    np.testing.assert_array_equal(cnt, count[leaf])
    assert np.all(first >= 0) and np.all(first + cnt <= ntri)
    starts = np.repeat(first, cnt)
    pos = starts + np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    assert np.all(np.bincount(pos, minlength=ntri) == 1), "every triangle lies in exactly one leaf"
    assert sorted(order.tolist()) == list(range(ntri))
    blo = np.repeat(lo[leaf], cnt, axis=0)[:, None, :]
    bhi = np.repeat(hi[leaf], cnt, axis=0)[:, None, :]
    tv = verts[order[pos]]
    assert np.all(tv >= blo) and np.all(tv <= bhi), "a leaf's triangles lie inside its box"
    assert 1 <= info.max_leaf_size <= 4
    return max_stack


@pytest.mark.parametrize("config", [1, 2])
def test_procedural_trees(host_ctx, config):
    s = host_ctx.procedural(config, seed=0, width=32, height=32)
    check_tree(s)
    s.free()


def test_interior_tree(host_ctx):
    s = host_ctx.procedural(3, seed=0, width=32, height=18)
    assert check_tree(s) < 64
    s.free()


def soup(kind: str, rng):
    if kind == "one":
        v = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float64)
    elif kind == "coincident":  # 37 copies of one triangle: no split separates them
        v = np.repeat(np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float64), 37, axis=0)
    elif kind == "chain":  # thin triangles along a line, sizes spanning 6 decades
        x = np.cumsum(10.0 ** rng.uniform(-6, 0, 500))
        v = np.stack([np.stack([x, np.zeros_like(x), np.zeros_like(x)], 1),
                      np.stack([x + 1e-3, np.zeros_like(x), np.zeros_like(x) + 1e-3], 1),
                      np.stack([x, np.zeros_like(x) + 1e-3, np.zeros_like(x)], 1)], 1)
    else:  # dense random cloud
        c = rng.uniform(-1, 1, (3000, 1, 3))
        v = c + rng.normal(scale=0.02, size=(3000, 3, 3))
    return v


def aimed_rays(v, n, rng):
    """Rays from around the triangles' bounding box towards points on the
    triangles themselves, so that most of them hit."""
    lo, hi = v.reshape(-1, 3).min(0), v.reshape(-1, 3).max(0)
    ext = np.maximum(hi - lo, 1e-3)
    tri = v[rng.integers(0, v.shape[0], n)]
    w = rng.dirichlet(np.ones(3), n)
    target = np.einsum("nk,nka->na", w, tri)
    org = lo - 0.5 * ext + rng.uniform(0, 1, (n, 3)) * 2 * ext
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = org
    rays[:, 4:7] = target - org
    rays[:, 7] = np.inf
    return rays


@pytest.mark.parametrize("kind", ["one", "coincident", "chain", "cloud"])
def test_stress_trees(host_ctx, tmp_path, kind):
    import pyoracle

    rng = np.random.default_rng(7)
    v = soup(kind, rng)
    verts = v.reshape(-1, 3)
    idx = np.arange(verts.shape[0]).reshape(-1, 3)
    write_mesh(tmp_path / "m.mesh", verts.tolist(), idx.tolist(), normals=False)
    p = tmp_path / "s.json"
    p.write_text(json.dumps(scene_json([("m.mesh", "w")], {"w": principled()})))
    s = host_ctx.load_scene(str(p))
    assert s.info().num_triangles == idx.shape[0]
    check_tree(s)
    # The oracle's walk of this tree equals brute force bit for bit
    # (coincident triangles: the smallest scene index wins the tie).
    o = pyoracle.OracleScene.from_aqua(s)
    rays = aimed_rays(v.astype(np.float32), 4000, rng)
    t, u, _, prim, _ = o.trace_bvh_f32(rays)
    tb, ub, _, pb = o.trace_brute_f32(rays)
    np.testing.assert_array_equal(prim, pb)
    np.testing.assert_array_equal(t.view(np.uint32), tb.view(np.uint32))
    np.testing.assert_array_equal(u.view(np.uint32), ub.view(np.uint32))
    assert np.mean(prim >= 0) > 0.5
    occ = o.trace_bvh_f32(rays, any_hit=True)[3]
    np.testing.assert_array_equal(occ >= 0, pb >= 0)
    if kind == "coincident":
        assert set(prim[prim >= 0].tolist()) == {0}
    s.free()


def decode_quantized(q):
    """Planes of the quantized nodes (16 floats each) as the device decodes
    them: fmaf(byte, 2^(e - 127), origin) in float, i.e. the exact sum in
    double rounded once to float."""
    q = np.ascontiguousarray(q, np.float32)
    words = q.view(np.uint32)
    origin = q[:, 0:3].astype(np.float64)
    ex = words[:, 3]
    lo = np.zeros((q.shape[0], 4, 3), np.float32)
    hi = np.zeros_like(lo)
    for a in range(3):
        e = ((ex >> (8 * a)) & 0xFF).astype(np.int64)
        assert np.all((e >= 1) & (e <= 254))
        sc = np.ldexp(1.0, e - 127)
        for k in range(4):
            ql = ((words[:, 8 + 2 * a] >> (8 * k)) & 0xFF).astype(np.float64)
            qh = ((words[:, 9 + 2 * a] >> (8 * k)) & 0xFF).astype(np.float64)
            lo[:, k, a] = (origin[:, a] + ql * sc).astype(np.float32)
            hi[:, k, a] = (origin[:, a] + qh * sc).astype(np.float32)
    return lo, hi, words[:, 4:8].view(np.int32)


@pytest.mark.parametrize("config", [1, 2, 3])
def test_quantized_nodes_contain_the_boxes(host_ctx, config):
    """Every decoded child box of the quantized copy contains the child's
    full-precision box, with the same links, and is at most a few of its
    8-bit steps larger."""
    s = host_ctx.procedural(config, seed=0, width=32, height=18)
    nodes, _ = s.bvh()
    q = s.bvh_quantized()
    assert q.shape == (nodes.shape[0], 16)
    lo = np.stack([nodes[:, 0:4], nodes[:, 8:12], nodes[:, 16:20]], axis=-1)
    hi = np.stack([nodes[:, 4:8], nodes[:, 12:16], nodes[:, 20:24]], axis=-1)
    link = nodes[:, 24:28].copy().view(np.int32)
    qlo, qhi, qlink = decode_quantized(q)
    np.testing.assert_array_equal(qlink, link)
    real = link != -1
    assert np.all(qlo[real] <= lo[real]) and np.all(qhi[real] >= hi[real])
    # Tight: per node and axis the slack is below two steps of the frame.
    ex = q.view(np.uint32)[:, 3]
    for a in range(3):
        step = np.ldexp(1.0, ((ex >> (8 * a)) & 0xFF).astype(np.int64) - 127)[:, None]
        slack = np.maximum(lo[..., a] - qlo[..., a], qhi[..., a] - hi[..., a])
        assert np.all(np.where(real, slack <= 2 * step + 1e-30, True))
    s.free()


@pytest.mark.parametrize("kind", ["chain", "cloud", "coincident"])
def test_quantized_walk_equals_brute_force(host_ctx, tmp_path, kind):
    """With the quantized nodes selected, the oracle's FP32 walk (which
    decodes them as the device does) still finds exactly the brute-force
    closest and any hits; it visits at least as many nodes as the full
    precision walk."""
    import pyoracle
    import aqua

    rng = np.random.default_rng(11)
    v = soup(kind, rng)
    verts = v.reshape(-1, 3)
    idx = np.arange(verts.shape[0]).reshape(-1, 3)
    write_mesh(tmp_path / "m.mesh", verts.tolist(), idx.tolist(), normals=False)
    p = tmp_path / "s.json"
    p.write_text(json.dumps(scene_json([("m.mesh", "w")], {"w": principled()})))
    s = host_ctx.load_scene(str(p))
    rays = aimed_rays(v.astype(np.float32), 4000, rng)
    full = pyoracle.OracleScene.from_aqua(s).trace_bvh_f32(rays)
    s.set_bvh_format(aqua.BVH_QUANTIZED)
    assert s.info().bvh_format == aqua.BVH_QUANTIZED
    o = pyoracle.OracleScene.from_aqua(s)
    t, u, _, prim, cnt = o.trace_bvh_f32(rays)
    tb, ub, _, pb = o.trace_brute_f32(rays)
    np.testing.assert_array_equal(prim, pb)
    np.testing.assert_array_equal(t.view(np.uint32), tb.view(np.uint32))
    np.testing.assert_array_equal(u.view(np.uint32), ub.view(np.uint32))
    occ = o.trace_bvh_f32(rays, any_hit=True)[3]
    np.testing.assert_array_equal(occ >= 0, pb >= 0)
    assert cnt[:, 0].sum() >= full[4][:, 0].sum()
    s.set_bvh_format(aqua.BVH_FULL)
    assert s.info().bvh_format == aqua.BVH_FULL
    s.free()


def test_automatic_node_format(host_ctx):
    """AUTO keeps full-precision nodes below 8 GiB of them (the interior's
    38 MB included); QUANTIZED and FULL switch the same tree's format."""
    import aqua

    big = host_ctx.procedural(3, seed=0, width=16, height=16)
    assert big.info().bvh_format == aqua.BVH_FULL
    n = big.info().num_bvh_nodes
    big.set_bvh_format(aqua.BVH_QUANTIZED)
    assert big.info().bvh_format == aqua.BVH_QUANTIZED and big.info().num_bvh_nodes == n
    big.set_bvh_format(aqua.BVH_AUTO)
    assert big.info().bvh_format == aqua.BVH_FULL
    with pytest.raises(aqua.AquaError):
        big.set_bvh_format(7)
    big.free()
