"""GPU parity at the benchmarked shapes and on the reference's own scenes.

Every test here is sample-matched against the FP64 oracle: the same seed
gives both sides the same PCG32 stream per pixel and the same random numbers
per bounce, so the images agree far below the relMSE 1e-3 bar and the
extension/shadow ray counts agree to within the rare FP32/FP64 divergences
(2e-3 relative).

- The Cornell GGX box at the bench's exact launch shape: 1024 x 1024 pixels,
  2^24 path slots (16 sample replicas per pixel, each with its film copy),
  unsorted shading, default tuning — only the samples per slot are lowered
  (1 instead of 64).
- The synthetic interior at 1920 x 1080 (2,073,600 slots, textures),
  against the FP32 oracle at 1 spp and the FP64 oracle at 32 spp.
- One persistent-kernel batch job per scene of the 64-job serving batch,
  the 4.0M-triangle sphere field included, each against the oracle directly.
- The reference's scenes/cbox.json (Point light, metallic tallBox) through
  the wavefront, the persistent kernel and a batch job, and the reference's
  scenes/room.json (394,269 triangles, JPEG textures, shading normals) when
  its staged copy is present.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import reference_scene

pytestmark = pytest.mark.gpu

TOL = 1e-3     # relMSE bar against the FP64 oracle
RAYS = 2e-3    # relative difference of ray counts


def rel_mse(x, r):
    import pyoracle

    return pyoracle.rel_mse(x, r)


def check_counts(st, ost):
    assert st.paths == int(ost[0])
    assert abs(st.ext_rays - ost[1]) / ost[1] < RAYS, (st.ext_rays, ost[1])
    if ost[2] > 0:
        assert abs(st.shadow_rays - ost[2]) / ost[2] < RAYS, (st.shadow_rays, ost[2])


def test_cornell_ggx_at_bench_shape(gpu_ctx):
    import pyoracle

    s = gpu_ctx.procedural(2, seed=0, width=1024, height=1024)
    cfg = gpu_ctx.integrator(spp=16, max_depth=8, rr_depth=3, seed=1)
    img, st = gpu_ctx.render(s, cfg, tuning=gpu_ctx.tuning())
    # the bench's shape: 16 slots per pixel (2^24 paths in flight)
    assert st.iterations < 64  # one sample per slot: the queue drains within the bounce limit and its tail
    assert gpu_ctx.workspace_bytes() > 2e9  # 2^24 slots of path state and queues
    o = pyoracle.OracleScene.from_aqua(s)
    ref, ost = o.render(16, 8, seed=1, precision=64)
    err = rel_mse(img, ref)
    assert err < TOL, err
    check_counts(st, ost)
    s.free()


def test_interior_1080p_sample_matched(gpu_ctx):
    """1920 x 1080 at 1 spp against the FP32 oracle (the same operations in
    the same precision; the device contracts multiply-adds, the oracle does
    not): all but a few pixels in 10^4 agree to 1e-3 in the relMSE metric's
    scale, and the ray counts agree to 1e-4. Against the FP64 oracle, 1 spp is the wrong
    test: about 2% of the interior's paths take another branch in double
    precision (grazing hits on the displaced planes, offsets of the ray
    origins), which alone gives relMSE ~2e-2 between the oracle's own FP32
    and FP64 images at 1 spp. The FP64 check therefore runs at 32 spp, on
    every 8th row of the 1080p image, where it must meet the 1e-3 bar."""
    import pyoracle

    s = gpu_ctx.procedural(3, seed=0, width=1920, height=1080)
    o = pyoracle.OracleScene.from_aqua(s)
    cfg = gpu_ctx.integrator(spp=1, max_depth=8, rr_depth=3, seed=1)
    img, st = gpu_ctx.render(s, cfg)
    ref32, o32 = o.render(1, 8, seed=1, precision=32)
    assert rel_mse(img, ref32) < 1e-4
    same = np.all(np.abs(img - ref32) <= 1e-3 * np.sqrt(ref32 * ref32 + 1e-2), axis=2)
    assert same.mean() > 0.999, same.mean()
    assert st.paths == int(o32[0])
    assert abs(st.ext_rays - o32[1]) / o32[1] < 1e-4
    assert abs(st.shadow_rays - o32[2]) / o32[2] < 1e-4
    assert img.mean() > 0.01

    cfg = gpu_ctx.integrator(spp=32, max_depth=8, rr_depth=3, seed=2)
    img, _ = gpu_ctx.render(s, cfg)
    rows = np.arange(4, 1080, 8)
    ref, _ = o.render_rows(rows, 32, 8, seed=2, precision=64)
    err = rel_mse(img[rows], ref)
    assert err < TOL, err
    s.free()


# One job per scene of the serving batch (configs 1, 2, 3 and the sphere
# field), each rendered by the persistent kernel in one launch.
BATCH_SPECS = [(1, 96, 96, 32, 5, 11), (2, 96, 96, 32, 8, 12), (3, 128, 72, 8, 8, 13), (5, 96, 96, 8, 8, 14)]


def test_batch_jobs_against_the_oracle(gpu_ctx):
    import pyoracle
    torch = pytest.importorskip("torch")

    scenes = {c: gpu_ctx.procedural(c, seed=0) for c in (1, 2, 3, 5)}
    bufs, jobs = [], []
    for (c, w, h, spp, depth, seed) in BATCH_SPECS:
        b = torch.full((h * w * 3,), -1.0, dtype=torch.float32, device="cuda:0")
        bufs.append(b)
        jobs.append((scenes[c], w, h, spp, depth, seed, b.data_ptr()))
    torch.cuda.synchronize()
    st, _ = gpu_ctx.render_batch(jobs)
    assert st.paths == sum(w * h * spp for (_, w, h, spp, _, _) in BATCH_SPECS)
    for (c, w, h, spp, depth, seed), b in zip(BATCH_SPECS, bufs):
        img = b.cpu().numpy().reshape(h, w, 3)
        o = pyoracle.OracleScene.from_aqua(scenes[c])
        o.set_resolution(w, h)
        ref, _ = o.render(spp, depth, seed=seed, precision=64, rr_depth=3)
        err = rel_mse(img, ref)
        assert err < TOL, (c, err)
        assert img.mean() > 0.005, c
    for s in scenes.values():
        s.free()


@pytest.fixture(scope="module")
def cbox(gpu_ctx):
    path = reference_scene("cbox.json")
    assert path is not None  # committed under tests/golden/cbox
    s = gpu_ctx.load_scene(path)
    yield s
    s.free()


def test_reference_cbox_wavefront(gpu_ctx, cbox):
    """scenes/cbox.json: 36 triangles, one Point light (cbox.json:544-561),
    a metallic 1.0 / roughness 0.1 tallBox (cbox.json:345-356); depth 5 as
    integrator.json:5."""
    import pyoracle

    info = cbox.info()
    assert info.num_lights == 1 and info.num_triangles == 36
    cbox.set_resolution(128, 128)
    cfg = gpu_ctx.integrator(spp=64, max_depth=5, rr_depth=3, seed=21)
    img, st = gpu_ctx.render(cbox, cfg)
    o = pyoracle.OracleScene.from_aqua(cbox)
    ref, ost = o.render(64, 5, seed=21, precision=64)
    err = rel_mse(img, ref)
    assert err < TOL, err
    assert img.mean() > 0.01
    check_counts(st, ost)
    # the metallic box is in view: some pixels are lit only through it
    assert any(m.metallic == 1.0 for m in cbox.materials())


def test_reference_cbox_persistent_and_batch(gpu_ctx, cbox):
    import aqua
    import pyoracle
    torch = pytest.importorskip("torch")

    cbox.set_resolution(96, 96)
    cfg = gpu_ctx.integrator(spp=32, max_depth=5, rr_depth=3, seed=22)
    o = pyoracle.OracleScene.from_aqua(cbox)
    ref, _ = o.render(32, 5, seed=22, precision=64)
    img, _ = gpu_ctx.render(cbox, cfg, tuning=gpu_ctx.tuning(kernel=aqua.KERNEL_PERSISTENT))
    assert rel_mse(img, ref) < TOL
    b = torch.full((96 * 96 * 3,), -1.0, dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    gpu_ctx.render_batch([(cbox, 96, 96, 32, 5, 22, b.data_ptr())])
    assert rel_mse(b.cpu().numpy().reshape(96, 96, 3), ref) < TOL


@pytest.mark.skipif(reference_scene("room.json") is None, reason="reference living-room scene not staged")
def test_reference_room_sample_matched(gpu_ctx):
    """scenes/room.json (fov-120 camera at room.json:2628-2674, 152 meshes
    with vertex normals, 16 JPEG textures; mesh 43 is missing from the
    reference snapshot and is skipped by allow_missing)."""
    import pyoracle

    s = gpu_ctx.load_scene(reference_scene("room.json"), allow_missing=True)
    assert s.info().num_triangles == 394269
    s.set_resolution(320, 180)
    cfg = gpu_ctx.integrator(spp=8, max_depth=5, rr_depth=3, seed=23)
    img, st = gpu_ctx.render(s, cfg)
    o = pyoracle.OracleScene.from_aqua(s)
    ref, ost = o.render(8, 5, seed=23, precision=64)
    err = rel_mse(img, ref)
    assert err < TOL, err
    assert img.mean() > 0.005
    check_counts(st, ost)
    s.free()
