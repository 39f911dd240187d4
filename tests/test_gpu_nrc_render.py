"""The cached renderer (radiance cache in the wavefront) on the GPU.

- With a zero network and no training it must equal, bit for bit, the path
  tracer cut after the query vertex's emission.
- With a constant network it must match the FP64 oracle's constant-cache
  estimator on the same random numbers (relMSE < 1e-3).
- Trained online it must converge towards the path-traced reference and beat
  the plain path tracer at equal sample count (the gain of the network).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-3


def constant_weights(rgb):
    """Weights whose output is `rgb` for every input (input 63 is 1)."""
    w = np.zeros(20672, np.float32)
    w[0 * 4096 + 0 * 64 + 63] = 1.0
    for l in range(1, 5):
        w[l * 4096 + 0] = 1.0
    for c in range(3):
        w[5 * 4096 + c * 64 + 0] = rgb[c]
    return w


def nrc_cfg(ctx, **kw):
    import aqua

    base = dict(type=aqua.INTEGRATOR_NRC, spp=1, max_depth=8, rr_depth=3, seed=1, nrc_query_vertex=2,
                nrc_train_samples=0, batch_size=4096, training_iters=0)
    base.update(kw)
    return ctx.integrator(**base)


def rel_mse(x, r):
    import pyoracle

    return pyoracle.rel_mse(x, r)


def test_zero_cache_equals_truncated_path_tracer(gpu_ctx):
    import aqua

    s = gpu_ctx.procedural(2, seed=0, width=48, height=40)
    net = aqua.Nrc(gpu_ctx, seed=1)
    net.set_weights(np.zeros(20672, np.float32))
    img, st = gpu_ctx.render_nrc(s, nrc_cfg(gpu_ctx, spp=8, seed=5), net)
    ref, _ = gpu_ctx.render(s, gpu_ctx.integrator(spp=8, max_depth=1, rr_depth=3, seed=5))
    assert np.array_equal(img, ref)
    assert st.nrc_queries > 0 and st.nrc_train_records == 0
    net.free()
    s.free()


def test_training_paths_keep_the_plain_depth_in_the_image(gpu_ctx):
    """When every path is a training path nothing queries the cache, and
    what the paths gather past max_depth (they run on for their targets)
    must stay out of the image: it equals the plain path tracer's, with the
    same random numbers, bit for bit."""
    import aqua

    s = gpu_ctx.procedural(2, seed=0, width=48, height=40)
    net = aqua.Nrc(gpu_ctx, seed=1)
    tune = gpu_ctx.tuning(replicas=4)
    cfg = nrc_cfg(gpu_ctx, spp=4, seed=5, nrc_query_vertex=aqua.NRC_QUERY_SPREAD, nrc_train_samples=1 << 20)
    img, st = gpu_ctx.render_nrc(s, cfg, net, tuning=tune)
    ref, _ = gpu_ctx.render(s, gpu_ctx.integrator(spp=4, max_depth=8, rr_depth=3, seed=5), tuning=tune)
    assert st.nrc_queries == 0 and st.nrc_train_records > 48 * 40 * 4
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    net.free()
    s.free()


@pytest.mark.parametrize("config", [1, 2])
def test_constant_cache_matches_oracle(gpu_ctx, config):
    import aqua
    import pyoracle

    rgb = [0.25, 0.5, 0.125]  # exact in bf16
    s = gpu_ctx.procedural(config, seed=0, width=40, height=40)
    o = pyoracle.OracleScene.from_aqua(s)
    net = aqua.Nrc(gpu_ctx, seed=1)
    net.set_weights(constant_weights(rgb))
    img, st = gpu_ctx.render_nrc(s, nrc_cfg(gpu_ctx, spp=64, seed=7), net)
    ref, _ = o.render(64, 8, seed=7, precision=64, query_depth=1, cache_rgb=rgb)
    assert rel_mse(img, ref) < TOL
    net.free()
    s.free()


def test_visualize_shows_the_cache(gpu_ctx):
    import aqua

    rgb = [0.25, 0.5, 0.125]
    s = gpu_ctx.procedural(1, seed=0, width=32, height=32)
    net = aqua.Nrc(gpu_ctx, seed=1)
    net.set_weights(constant_weights(rgb))
    img, st = gpu_ctx.render_nrc(s, nrc_cfg(gpu_ctx, spp=2, visualize_cache=1, nrc_train_samples=4096), net)
    # Each pixel averages 2 samples; a sample that hits shows the cache, a
    # miss shows the (black) environment: every pixel is 0, rgb/2 or rgb.
    frac = img[..., 1] / rgb[1]
    assert np.all(np.isin(np.round(frac * 2), [0, 1, 2]))
    np.testing.assert_allclose(img, frac[..., None] * np.array(rgb, np.float32), rtol=1e-6, atol=1e-7)
    assert (frac == 1).mean() > 0.5
    assert st.nrc_train_records == 0
    net.free()
    s.free()


@pytest.fixture(scope="module", params=[(1, 64, 64, 4, 4096, 1024, 150), (3, 160, 90, 1, 16384, 4096, 200)],
                ids=["cornell", "interior"])
def trained(gpu_ctx, request):
    """Online training: Cornell box (Lambert) 64x64 at 4 spp per frame, and
    the 1.15M-triangle interior 160x90 at 1 spp per frame; training paths
    are a few percent of all paths."""
    import aqua

    conf, w, h, spp, tsamp, batch, frames = request.param
    s = gpu_ctx.procedural(conf, seed=0, width=w, height=h)
    net = aqua.Nrc(gpu_ctx, seed=3, learning_rate=1e-2)
    train = lambda seed: nrc_cfg(gpu_ctx, spp=spp, seed=seed, nrc_train_samples=tsamp, batch_size=batch)
    view = nrc_cfg(gpu_ctx, spp=64, visualize_cache=1)
    before, _ = gpu_ctx.render_nrc(s, view, net)
    losses = []
    for f in range(frames):
        _, st = gpu_ctx.render_nrc(s, train(1000 + f), net)
        losses.append(st.nrc_loss)
    after, _ = gpu_ctx.render_nrc(s, view, net)
    ref, _ = gpu_ctx.render(s, gpu_ctx.integrator(spp=8192 if conf == 1 else 4096, max_depth=8, rr_depth=3,
                                                  seed=99))
    yield s, net, losses, ref, before, after, train, spp
    net.free()
    s.free()


def test_online_training_learns(trained):
    s, net, losses, ref, before, after, _, _ = trained
    # Targets are single path samples and the relative loss is normalised by
    # the network's own output, so the loss value is noise-dominated and not
    # a progress measure; it only has to stay finite.
    assert all(np.isfinite(losses))
    # The cache seen at the first hit approximates the reflected radiance
    # there, i.e. the converged image wherever a light is not visible.
    mask = ref.max(axis=2) < 3.0
    e_before = rel_mse(before[mask], ref[mask])
    e_after = rel_mse(after[mask], ref[mask])
    assert e_after < 0.2 * e_before and e_after < 0.1, (e_before, e_after)


def test_cached_render_converges_and_gains(gpu_ctx, trained):
    """What the trained network gains: at equal sample count the cached
    image is closer to the converged reference than the plain one."""
    import aqua

    s, net, losses, ref, _, _, train, spp = trained
    frames = 64 // spp
    acc = np.zeros_like(ref)
    for f in range(frames):
        gpu_ctx.render_nrc(s, train(5000 + f), net, out=acc, flags=aqua.RENDER_ACCUMULATE)
    cached = acc / (frames * spp)
    plain, _ = gpu_ctx.render(s, gpu_ctx.integrator(spp=64, max_depth=8, rr_depth=3, seed=7000))
    e_cached, e_plain = rel_mse(cached, ref), rel_mse(plain, ref)
    assert e_cached < 0.8 * e_plain, (e_cached, e_plain)


def test_path_spread_query_lies_between_the_fixed_cuts(gpu_ctx):
    """AQUA_NRC_QUERY_SPREAD queries where a path's spread exceeds 0.01 of its
    first-hit footprint, at vertex 2 or later. With a zero network every path
    is the path tracer's, with the same random numbers, cut at its query
    vertex: per pixel the image lies between the path tracer cut at vertex 2
    and the uncut path tracer, and the GGX box's glossy hits (small spread)
    make it differ from the vertex-2 cut."""
    import aqua

    s = gpu_ctx.procedural(2, seed=0, width=48, height=40)
    net = aqua.Nrc(gpu_ctx, seed=1)
    net.set_weights(np.zeros(20672, np.float32))
    img, st = gpu_ctx.render_nrc(s, nrc_cfg(gpu_ctx, spp=16, seed=5, nrc_query_vertex=aqua.NRC_QUERY_SPREAD), net)
    cut2, _ = gpu_ctx.render_nrc(s, nrc_cfg(gpu_ctx, spp=16, seed=5, nrc_query_vertex=2), net)
    full, _ = gpu_ctx.render(s, gpu_ctx.integrator(spp=16, max_depth=8, rr_depth=3, seed=5),
                             tuning=gpu_ctx.tuning(replicas=1))
    eps = 1e-5 * (1.0 + full)
    assert np.all(img >= cut2 - eps) and np.all(img <= full + eps)
    assert np.mean(np.abs(img - cut2) > 1e-6) > 0.01
    assert 0 < st.nrc_queries <= 48 * 40 * 16
    net.free()
    s.free()


@pytest.mark.parametrize("config", [2, 3])
def test_path_spread_constant_cache_matches_oracle(gpu_ctx, config):
    """The path-spread query rule against the FP64 oracle's restatement of
    it (query_depth -2), with a constant network: the same vertices query,
    sample for sample (the rule reads the hit distance, the shading normal
    and the previous bounce's pdf, which the oracle computes in double)."""
    import aqua
    import pyoracle

    rgb = [0.25, 0.5, 0.125]  # exact in bf16
    s = gpu_ctx.procedural(config, seed=0, width=40, height=32)
    o = pyoracle.OracleScene.from_aqua(s)
    net = aqua.Nrc(gpu_ctx, seed=1)
    net.set_weights(constant_weights(rgb))
    img, st = gpu_ctx.render_nrc(s, nrc_cfg(gpu_ctx, spp=64, seed=9, nrc_query_vertex=aqua.NRC_QUERY_SPREAD), net)
    ref, _ = o.render(64, 8, seed=9, precision=64, query_depth=-2, cache_rgb=rgb)
    assert rel_mse(img, ref) < TOL
    assert st.nrc_queries > 0
    net.free()
    s.free()
