"""The radiance cache's network on the GPU against the FP64 CPU oracle.

The oracle emulates the device's bf16 storage points (weights, inputs,
activations, gradients), so the remaining differences are FP32 vs FP64
accumulation and the rare bf16 rounding flips they cause. Tolerances:
forward outputs within 1e-2 of the output scale; gradients within 2e-2
relative L2 and cosine > 0.999; Adam bit-close to its closed form.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rand_raw(n, seed):
    rng = np.random.default_rng(seed)
    raw = np.zeros((n, 16), np.float32)
    raw[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    for sl in (slice(3, 6), slice(6, 9)):
        v = rng.normal(size=(n, 3))
        raw[:, sl] = v / np.linalg.norm(v, axis=1, keepdims=True)
    raw[:, 9] = rng.uniform(0, 1, n)
    raw[:, 10:16] = rng.uniform(0, 1, (n, 6))
    return raw


def smooth_target(raw):
    p = raw[:, 0:3]
    return np.stack([1.0 + 0.5 * np.sin(3 * p[:, 0]) * raw[:, 10],
                     0.5 + 0.3 * np.cos(2 * p[:, 1] + p[:, 2]),
                     np.abs(p[:, 2]) * raw[:, 12] + 0.2], axis=1).astype(np.float32)


@pytest.fixture()
def net(gpu_ctx):
    import aqua

    n = aqua.Nrc(gpu_ctx, seed=3, learning_rate=1e-2, bbox_min=[-1, -1, -1], bbox_max=[1, 1, 1])
    yield n
    n.free()


def test_encode_matches_oracle(net):
    import pyoracle

    raw = rand_raw(5000, 1)
    x = net.encode(raw)
    ref = pyoracle.nrc_encode(raw, [-1, -1, -1], [1, 1, 1])
    got = pyoracle.bf16_to_float(x)
    # bf16 keeps 8 significant bits (half-ulp 2^-8 relative); the finest
    # position octave (2^7 pi) turns the FP32 vs FP64 normalised position
    # (~1e-7) into ~5e-5 absolute near sine zero crossings.
    assert np.all(np.abs(got - ref) <= 2 ** -8 * np.abs(ref) + 2e-4)
    assert np.abs(got - ref).mean() < 2e-3


@pytest.mark.parametrize("kernel", ["mma_sync", "tcgen05"])
@pytest.mark.parametrize("rows", [1, 127, 4099])
def test_forward_matches_oracle(gpu_ctx, kernel, rows):
    """Both inference kernels against the bf16-emulating FP64 oracle; 4099
    rows is ragged for both the 16-row (mma.sync) and 128-row (tcgen05)
    tiles, 1 and 127 leave most of a single tcgen05 tile empty."""
    import aqua
    import pyoracle

    k = aqua.NRC_KERNEL_MMA_SYNC if kernel == "mma_sync" else aqua.NRC_KERNEL_TCGEN05
    net = aqua.Nrc(gpu_ctx, seed=3, bbox_min=[-1, -1, -1], bbox_max=[1, 1, 1], forward_kernel=k)
    try:
        raw = rand_raw(rows, 2)
        x = net.encode(raw)
        w = net.weights()
        y = net.forward(x)
    finally:
        net.free()
    ref = pyoracle.mlp_forward(w, pyoracle.bf16_to_float(x), emulate_bf16=True)
    scale = np.abs(ref).max()
    assert np.abs(y - ref).max() <= 1e-2 * scale
    assert np.abs(y - ref).mean() <= 1e-3 * scale


def test_tcgen05_matches_mma_sync(gpu_ctx):
    """The two inference kernels on the same weights and 300K rows (many
    tiles per CTA): they differ only in FP32 accumulation order and the bf16
    rounding flips it causes, so outputs agree to the forward tolerance."""
    import aqua

    nets = [aqua.Nrc(gpu_ctx, seed=11, bbox_min=[-1, -1, -1], bbox_max=[1, 1, 1], forward_kernel=k)
            for k in (aqua.NRC_KERNEL_MMA_SYNC, aqua.NRC_KERNEL_TCGEN05)]
    try:
        rng = np.random.default_rng(12)
        w = (rng.uniform(-0.3, 0.3, aqua.NRC_PARAMS)).astype(np.float32)
        for n in nets:
            n.set_weights(w)
        raw = rand_raw(300_007, 13)
        x = nets[0].encode(raw)
        y0, y1 = (n.forward(x) for n in nets)
    finally:
        for n in nets:
            n.free()
    scale = np.abs(y0).max()
    d = np.abs(y0 - y1)
    assert d.max() <= 1e-2 * scale, d.max() / scale
    assert d.mean() <= 1e-3 * scale
    assert np.all(np.isfinite(y1))


def test_gradient_matches_oracle(net):
    import pyoracle

    raw = rand_raw(8192 + 37, 3)
    x = net.encode(raw)
    t = smooth_target(raw)
    w0 = net.weights()
    loss = net.train_step(x, t)
    g = net.gradients().astype(np.float64)
    gref, lref = pyoracle.mlp_grad(w0, pyoracle.bf16_to_float(x), t, emulate_bf16=True)
    assert abs(loss - lref) <= 1e-3 * lref
    rel = np.linalg.norm(g - gref) / np.linalg.norm(gref)
    cos = float(g @ gref / (np.linalg.norm(g) * np.linalg.norm(gref)))
    assert rel < 2e-2 and cos > 0.999, (rel, cos)
    # per layer too: every layer's gradient must agree, not just the total
    for l in range(6):
        sl = slice(l * 4096, l * 4096 + (4096 if l < 5 else 192))
        r = np.linalg.norm(g[sl] - gref[sl]) / (np.linalg.norm(gref[sl]) + 1e-30)
        assert r < 5e-2, (l, r)
    # against the unquantised FP64 network: bf16 tolerance
    g64, _ = pyoracle.mlp_grad(w0, pyoracle.bf16_to_float(x), t, emulate_bf16=False)
    cos64 = float(g @ g64 / (np.linalg.norm(g) * np.linalg.norm(g64)))
    assert cos64 > 0.99


def test_adam_step_closed_form(net):
    raw = rand_raw(2048, 4)
    x = net.encode(raw)
    t = smooth_target(raw)
    w0 = net.weights().astype(np.float64)
    net.train_step(x, t)
    g = net.gradients().astype(np.float64)
    w1 = net.weights().astype(np.float64)
    lr, b1, b2, eps = 1e-2, 0.9, 0.99, 1e-8
    m = (1 - b1) * g
    v = (1 - b2) * g * g
    expect = w0 - lr * (m / (1 - b1)) / (np.sqrt(v / (1 - b2)) + eps)
    np.testing.assert_allclose(w1, expect, rtol=1e-4, atol=1e-6)


def test_training_reduces_loss(net):
    import pyoracle

    raw = rand_raw(16384, 5)
    x = net.encode(raw)
    t = smooth_target(raw)
    losses = [net.train_step(x[i % 4 * 4096:(i % 4 + 1) * 4096], t[i % 4 * 4096:(i % 4 + 1) * 4096])
              for i in range(200)]
    assert losses[-1] < 0.1 * losses[0]
    held = rand_raw(2000, 6)
    y = net.forward(net.encode(held))
    th = smooth_target(held)
    assert float(np.mean((y - th) ** 2 / (th ** 2 + 0.01))) < 0.02


def test_set_weights_roundtrip_and_reset(net):
    rng = np.random.default_rng(7)
    w = (rng.uniform(-0.1, 0.1, 20672)).astype(np.float32)
    net.set_weights(w)
    np.testing.assert_array_equal(net.weights(), w)


def test_bad_nrc_arguments(gpu_ctx):
    import aqua

    with pytest.raises(aqua.AquaError) as e:
        aqua.Nrc(gpu_ctx, bbox_min=[0, 0, 0], bbox_max=[1, 0, 1])
    assert e.value.status == aqua.ERR_INVALID_ARG


@pytest.mark.parametrize("rows", [1, 511, 513, 8229, 70000])
def test_tcgen05_weight_gradients_equal_mma_sync(gpu_ctx, rows):
    """The training step's weight gradients on tcgen05 (512-row split-K
    chunks, TMEM accumulators) against the mma.sync path (128-row chunks) on
    the same batch: the same bf16 products summed in FP32 in another order,
    so every layer agrees to accumulation rounding (ragged chunk tails and a
    single row included). The two nets' forward and backward passes differ
    only in accumulation order too; rare bf16 rounding flips of the stored
    activations are the only other difference."""
    import aqua

    nets = [aqua.Nrc(gpu_ctx, seed=3, learning_rate=1e-2, bbox_min=[-1, -1, -1], bbox_max=[1, 1, 1],
                     forward_kernel=k) for k in (aqua.NRC_KERNEL_MMA_SYNC, aqua.NRC_KERNEL_TCGEN05)]
    try:
        raw = rand_raw(rows, 21)
        x = nets[0].encode(raw)
        t = smooth_target(raw)
        grads = []
        for n in nets:
            n.train_step(x, t)
            grads.append(n.gradients().astype(np.float64))
    finally:
        for n in nets:
            n.free()
    g0, g1 = grads
    for l in range(6):
        sl = slice(l * 4096, l * 4096 + (4096 if l < 5 else 192))
        scale = np.abs(g0[sl]).max() + 1e-30
        rel = np.linalg.norm(g1[sl] - g0[sl]) / (np.linalg.norm(g0[sl]) + 1e-30)
        assert rel < 1e-3 and np.abs(g1[sl] - g0[sl]).max() <= 1e-2 * scale, (l, rel)
    assert np.any(g1 != 0)
