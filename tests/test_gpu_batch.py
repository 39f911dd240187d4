"""Batched rendering on the GPU: many jobs over several scenes in one
persistent launch (replayed from a CUDA graph) must give, job by job, the
image aqua_render gives for the same view, seed and sample count."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes(gpu_ctx):
    out = {c: gpu_ctx.procedural(c, seed=0) for c in (1, 2, 3)}
    yield out
    for s in out.values():
        s.free()


def make_jobs(scenes, specs):
    torch = pytest.importorskip("torch")
    bufs, jobs = [], []
    for (cfg, w, h, spp, depth, seed) in specs:
        b = torch.full((h * w * 3,), -1.0, dtype=torch.float32, device="cuda:0")
        bufs.append(b)
        jobs.append((scenes[cfg], w, h, spp, depth, seed, b.data_ptr()))
    torch.cuda.synchronize()
    return jobs, bufs


SPECS = [(1, 64, 48, 16, 5, 1), (2, 37, 29, 33, 8, 2), (3, 48, 27, 4, 8, 3), (2, 16, 16, 64, 8, 4),
         (1, 1, 1, 7, 3, 5), (3, 20, 30, 2, 2, 6)]


def reference(gpu_ctx, scene, w, h, spp, depth, seed):
    info = scene.info()
    scene.set_resolution(w, h)
    img, _ = gpu_ctx.render(scene, gpu_ctx.integrator(spp=spp, max_depth=depth, rr_depth=3, seed=seed),
                            tuning=gpu_ctx.tuning(replicas=1))
    scene.set_resolution(info.width, info.height)
    return img


def test_batch_matches_single_renders(gpu_ctx, scenes):
    jobs, bufs = make_jobs(scenes, SPECS)
    st, job_ms = gpu_ctx.render_batch(jobs)
    assert st.paths == sum(w * h * spp for (_, w, h, spp, _, _) in SPECS)
    assert np.all(job_ms > 0) and np.all(job_ms <= st.device_ms * 1.05 + 0.05)
    for (cfg, w, h, spp, depth, seed), b in zip(SPECS, bufs):
        img = b.cpu().numpy().reshape(h, w, 3)
        ref = reference(gpu_ctx, scenes[cfg], w, h, spp, depth, seed)
        np.testing.assert_allclose(img, ref, rtol=1e-5, atol=1e-6, err_msg=str((cfg, w, h, spp)))


def test_graph_replay_is_identical(gpu_ctx, scenes):
    jobs, bufs = make_jobs(scenes, SPECS[:3])
    t = gpu_ctx.tuning(use_graph=1, block_trace=64)
    gpu_ctx.render_batch(jobs, t)
    first = [b.cpu().numpy().copy() for b in bufs]
    for b in bufs:
        b.fill_(-1.0)
    st, _ = gpu_ctx.render_batch(jobs, t)  # same jobs: the captured graph is replayed
    for a, b in zip(first, bufs):
        assert np.array_equal(a, b.cpu().numpy())


def test_launch_shapes_agree(gpu_ctx, scenes):
    jobs, bufs = make_jobs(scenes, SPECS[:2])
    outs = []
    for kw in (dict(block_trace=64, blocks_per_sm=1), dict(block_trace=256), dict(use_graph=0)):
        gpu_ctx.render_batch(jobs, gpu_ctx.tuning(**kw))
        outs.append([b.cpu().numpy().copy() for b in bufs])
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert np.array_equal(a, b)


def test_batch_autotuner(gpu_ctx, scenes):
    jobs, _ = make_jobs(scenes, SPECS)
    t = gpu_ctx.autotune_batch(jobs)
    assert t.block_trace in (64, 128, 256) and t.use_graph == 1


def test_single_scene_autotuner(gpu_ctx, scenes):
    s = gpu_ctx.procedural(2, seed=0, width=128, height=96)
    cfg = gpu_ctx.integrator(spp=8, max_depth=8, seed=3)
    t = gpu_ctx.autotune(s, cfg)
    assert t.block_trace in (64, 128) and t.block_shade in (64, 128)
    a, _ = gpu_ctx.render(s, cfg)
    b, _ = gpu_ctx.render(s, cfg, tuning=t)
    assert np.array_equal(a, b)
    s.free()


def test_batch_arguments(gpu_ctx, scenes):
    import aqua
    import ctypes

    st, _ = gpu_ctx.render_batch([])
    assert st.paths == 0
    jobs, _ = make_jobs(scenes, SPECS[:1])
    bad = [(jobs[0][0], 0, 10, 4, 3, 1, jobs[0][6])]
    with pytest.raises(aqua.AquaError) as e:
        gpu_ctx.render_batch(bad)
    assert e.value.status == aqua.ERR_INVALID_ARG
    arr = (aqua.Job * 1)(aqua.Job(None, 4, 4, 1, 1, 0, jobs[0][6]))
    assert gpu_ctx.lib.aqua_render_batch(gpu_ctx.handle, arr, 1, None, None) == aqua.ERR_INVALID_ARG
