"""The JPEG decoder behind `Image` textures (room.json:6).

1. Synthetic files from a small encoder written here (two-pass optimal
   Huffman tables, T.81 baseline and progressive syntax): the decoder's
   output must equal a float64 numpy decoding of the very coefficients the
   encoder wrote, to within one 8-bit level at rounding boundaries. Covered:
   4:4:4, 4:2:0, grey, restart intervals, progressive spectral selection
   with end-of-band runs and DC successive approximation.
2. The reference scene's 17 textures against nvJPEG (tests/golden/
   jpeg_facts.json, written by make_jpeg_facts.py on a GPU machine).
3. Refusals: not a JPEG, truncated, arithmetic coding.
"""
from __future__ import annotations

import heapq
import json
import os

import numpy as np
import pytest

import aqua

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
from conftest import reference_scene

TEXTURES = reference_scene("textures")
need_ref = pytest.mark.skipif(TEXTURES is None, reason="reference textures not staged")

# ---------------------------------------------------------------- encoder
ZZ = []
for s in range(15):
    lo, hi = max(0, s - 7), min(s, 7)
    ys = range(hi, lo - 1, -1) if s % 2 == 0 else range(lo, hi + 1)
    ZZ += [y * 8 + (s - y) for y in ys]
ZZ = np.array(ZZ)
M = np.array([[(np.sqrt(0.5) if u == 0 else 1.0) * 0.5 * np.cos((2 * x + 1) * u * np.pi / 16) for x in range(8)]
              for u in range(8)])  # orthonormal DCT-II: F = M B M^T


def category(v: int) -> int:
    return int(abs(v)).bit_length()


def magnitude_bits(v: int, s: int) -> int:
    return v if v >= 0 else v + (1 << s) - 1


class BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, v: int, n: int):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = 0
                self.n = 0

    def flush(self):
        while self.n:
            self.put(1, 1)


def huffman_table(freq: dict):
    """Code lengths by Huffman's algorithm (a reserved symbol keeps the
    all-ones code unused), canonical codes (T.81 Annex C)."""
    syms = sorted(freq) + [256]
    f = {**freq, 256: 1}
    heap = [(f[s], i, [s]) for i, s in enumerate(syms)]
    heapq.heapify(heap)
    length = {s: 0 for s in syms}
    uid = len(syms)
    if len(heap) == 1:
        length[syms[0]] = 1
    while len(heap) > 1:
        f1, _, a = heapq.heappop(heap)
        f2, _, b = heapq.heappop(heap)
        for s in a + b:
            length[s] += 1
        heapq.heappush(heap, (f1 + f2, uid, a + b))
        uid += 1
    del length[256]
    assert max(length.values()) <= 16
    vals = sorted(length, key=lambda s: (length[s], s))
    bits = [sum(1 for s in vals if length[s] == l) for l in range(1, 17)]
    codes, code, k = {}, 0, 0
    for l in range(1, 17):
        for _ in range(bits[l - 1]):
            codes[vals[k]] = (code, l)
            code += 1
            k += 1
        code <<= 1
    return bits, vals, codes


def seg(marker: int, body: bytes) -> bytes:
    return bytes([0xFF, marker]) + (len(body) + 2).to_bytes(2, "big") + body


class Component:
    def __init__(self, cid, h, v, plane, qt):
        self.cid, self.h, self.v, self.qt = cid, h, v, qt
        self.plane = plane


def encode(img: np.ndarray, sampling=(1, 1), grey=False, restart=0, progressive=False, quality_scale=1.0):
    """img: (H, W, 3) uint8. Returns (jpeg bytes, expected decode as float64 planes -> RGB uint8)."""
    H, W, _ = img.shape
    x = img.astype(np.float64)
    if grey:
        planes = [0.299 * x[..., 0] + 0.587 * x[..., 1] + 0.114 * x[..., 2]]
    else:
        y = 0.299 * x[..., 0] + 0.587 * x[..., 1] + 0.114 * x[..., 2]
        cb = -0.168736 * x[..., 0] - 0.331264 * x[..., 1] + 0.5 * x[..., 2] + 128
        cr = 0.5 * x[..., 0] - 0.418688 * x[..., 1] - 0.081312 * x[..., 2] + 128
        planes = [y, cb, cr]
    hmax, vmax = sampling
    rng = np.random.default_rng(7)
    qts = [np.clip(np.round((1 + rng.integers(0, 6, 64)) * quality_scale), 1, 255).astype(np.int64) for _ in range(2)]
    comps = []
    for i, p in enumerate(planes):
        h, v = (hmax, vmax) if i == 0 else (1, 1)
        if (h, v) != (hmax, vmax):  # box-filter subsampling
            ph = -(-p.shape[0] // vmax) * vmax
            pw = -(-p.shape[1] // hmax) * hmax
            pp = np.pad(p, ((0, ph - p.shape[0]), (0, pw - p.shape[1])), mode="edge")
            p = pp.reshape(ph // vmax, vmax, pw // hmax, hmax).mean(axis=(1, 3))
        comps.append(Component(i + 1, h, v, p, qts[0 if i == 0 else 1]))
    mcux, mcuy = -(-W // (8 * hmax)), -(-H // (8 * vmax))
    for c in comps:  # quantised coefficients on the padded block grid, natural order
        bw, bh = mcux * c.h, mcuy * c.v
        p = np.pad(c.plane, ((0, bh * 8 - c.plane.shape[0]), (0, bw * 8 - c.plane.shape[1])), mode="edge") - 128
        blocks = p.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)
        F = np.einsum("vy,abyx,ux->abvu", M, blocks, M)  # F[v][u], v = vertical frequency
        c.q = np.round(F.reshape(bh, bw, 64) / c.qt).astype(np.int64)
        c.bw, c.bh = bw, bh
        cw, ch = -(-W * c.h // hmax), -(-H * c.v // vmax)
        c.rbw, c.rbh = -(-cw // 8), -(-ch // 8)

    # ---- scans: (component list, ss, se, ah, al)
    if progressive:
        scans = [(comps, 0, 0, 0, 1), (comps, 0, 0, 1, 0)]
        for c in comps:
            scans += [([c], 1, 5, 0, 0), ([c], 6, 63, 0, 0)]
    else:
        scans = [(comps, 0, 63, 0, 0)]

    def units(sc):
        if len(sc) == 1:
            c = sc[0]
            for by in range(c.rbh):
                for bx in range(c.rbw):
                    yield [(c, bx, by)]
        else:
            for my in range(mcuy):
                for mx in range(mcux):
                    yield [(c, mx * c.h + hh, my * c.v + vv) for c in sc for vv in range(c.v) for hh in range(c.h)]

    def run_scan(sc, ss, se, ah, al, emit_dc, emit_ac, emit_bits, emit_restart):
        preds = {c.cid: 0 for c in sc}
        eobrun = [0]

        def flush_eob():
            if eobrun[0]:
                r = eobrun[0].bit_length() - 1
                emit_ac(sc[0], r << 4)
                if r:
                    emit_bits(eobrun[0] - (1 << r), r)
                eobrun[0] = 0

        for ui, unit in enumerate(units(sc)):
            if restart and ui and ui % restart == 0:
                flush_eob()
                emit_restart((ui // restart - 1) % 8)
                preds = {c.cid: 0 for c in sc}
            for c, bx, by in unit:
                coef = c.q[by, bx][ZZ]  # zig-zag order
                if ss == 0 and ah == 0:
                    dc = int(coef[0]) >> al
                    d = dc - preds[c.cid]
                    preds[c.cid] = dc
                    s = category(d)
                    emit_dc(c, s)
                    if s:
                        emit_bits(magnitude_bits(d, s), s)
                if ss == 0 and ah > 0:
                    emit_bits((int(coef[0]) >> al) & 1, 1)
                if se > 0 and (not progressive or ss > 0):
                    band = [int(v) >> al if v >= 0 else -((-int(v)) >> al) for v in coef[max(ss, 1):se + 1]]
                    last = max([i for i, v in enumerate(band) if v != 0], default=-1)
                    if progressive and last < 0:
                        eobrun[0] += 1
                        if eobrun[0] == 0x7FFF:
                            flush_eob()
                        continue
                    if progressive:
                        flush_eob()
                    run = 0
                    for v in band[:last + 1]:
                        if v == 0:
                            run += 1
                            continue
                        while run > 15:
                            emit_ac(c, 0xF0)
                            run -= 16
                        s = category(v)
                        emit_ac(c, (run << 4) | s)
                        emit_bits(magnitude_bits(v, s), s)
                        run = 0
                    if last < len(band) - 1:
                        if progressive:
                            eobrun[0] += 1
                        else:
                            emit_ac(c, 0x00)
        flush_eob()

    out = bytearray(b"\xFF\xD8")
    out += seg(0xE0, b"JFIF\0\x01\x02\0\0\x01\0\x01\0\0")
    for t, qt in enumerate(qts[:1 if grey else 2]):
        out += seg(0xDB, bytes([t]) + bytes(int(q) for q in qt[ZZ]))
    body = bytes([8]) + H.to_bytes(2, "big") + W.to_bytes(2, "big") + bytes([len(comps)])
    for c in comps:
        body += bytes([c.cid, (c.h << 4) | c.v, 0 if c.cid == 1 else 1])
    out += seg(0xC2 if progressive else 0xC0, body)
    if restart:
        out += seg(0xDD, restart.to_bytes(2, "big"))
    for sc, ss, se, ah, al in scans:
        # pass 1: symbol statistics per table class
        freq_dc, freq_ac = {}, {}

        def cnt_dc(c, s):
            d = freq_dc.setdefault(0 if c.cid == 1 else 1, {})
            d[s] = d.get(s, 0) + 1

        def cnt_ac(c, s):
            d = freq_ac.setdefault(0 if c.cid == 1 else 1, {})
            d[s] = d.get(s, 0) + 1

        run_scan(sc, ss, se, ah, al, cnt_dc, cnt_ac, lambda v, n: None, lambda m: None)
        tabs_dc = {k: huffman_table(v) for k, v in freq_dc.items()}
        tabs_ac = {k: huffman_table(v) for k, v in freq_ac.items()}
        for cls, tabs in ((0, tabs_dc), (1, tabs_ac)):
            for th, (bits, vals, _) in tabs.items():
                out += seg(0xC4, bytes([(cls << 4) | th]) + bytes(bits) + bytes(vals))
        body = bytes([len(sc)])
        for c in sc:
            t = 0 if c.cid == 1 else 1
            body += bytes([c.cid, (t << 4) | t])
        body += bytes([ss, se, (ah << 4) | al])
        out += seg(0xDA, body)
        bw = BitWriter()

        def put_dc(c, s):
            code, l = tabs_dc[0 if c.cid == 1 else 1][2][s]
            bw.put(code, l)

        def put_ac(c, s):
            code, l = tabs_ac[0 if c.cid == 1 else 1][2][s]
            bw.put(code, l)

        def put_rst(m):
            bw.flush()
            bw.out += bytes([0xFF, 0xD0 + m])

        run_scan(sc, ss, se, ah, al, put_dc, put_ac, bw.put, put_rst)
        bw.flush()
        out += bw.out
    out += b"\xFF\xD9"
    return bytes(out), reference_decode(comps, W, H, hmax, vmax, grey)


def lround(x):
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def reference_decode(comps, W, H, hmax, vmax, grey):
    """float64 decoding of the encoder's quantised coefficients, with the
    decoder's rounding points (T.81 A.3.3 IDCT, level shift, centred linear
    chroma upsampling, JFIF YCbCr -> RGB)."""
    planes = []
    for c in comps:
        F = (c.q * c.qt).reshape(c.bh, c.bw, 8, 8).astype(np.float64)
        B = np.einsum("vy,abvu,ux->abyx", M, F, M)
        B = np.clip(lround(B) + 128, 0, 255)
        planes.append(B.transpose(0, 2, 1, 3).reshape(c.bh * 8, c.bw * 8))
    if grey:
        g = planes[0][:H, :W]
        return np.repeat(g[..., None], 3, axis=2).astype(np.uint8)
    out = []
    for c, p in zip(comps, planes):
        if (c.h, c.v) == (hmax, vmax):
            out.append(p[:H, :W])
            continue
        cw, ch = -(-W * c.h // hmax), -(-H * c.v // vmax)
        fx = np.clip((np.arange(W) + 0.5) * c.h / hmax - 0.5, 0, cw - 1)
        fy = np.clip((np.arange(H) + 0.5) * c.v / vmax - 0.5, 0, ch - 1)
        x0, y0 = fx.astype(int), fy.astype(int)
        x1, y1 = np.minimum(x0 + 1, cw - 1), np.minimum(y0 + 1, ch - 1)
        ax, ay = (fx - x0)[None, :], (fy - y0)[:, None]
        a = p[y0][:, x0] + (p[y0][:, x1] - p[y0][:, x0]) * ax
        b = p[y1][:, x0] + (p[y1][:, x1] - p[y1][:, x0]) * ax
        out.append(a + (b - a) * ay)
    y, cb, cr = out[0], out[1] - 128, out[2] - 128
    rgb = np.stack([y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb], axis=-1)
    return np.clip(lround(rgb), 0, 255).astype(np.uint8)


def synthetic_image(h, w, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    base = np.stack([128 + 100 * np.sin(xx / 7.0 + s) * np.cos(yy / 11.0 - s) for s in (0.0, 1.0, 2.0)], axis=-1)
    return np.clip(base + rng.normal(0, 12, (h, w, 3)), 0, 255).astype(np.uint8)


@pytest.fixture(scope="module")
def ctx():
    c = aqua.Context(device=-2)  # AQUA_DEVICE_HOST_ONLY
    yield c
    c.close()


CASES = {
    "baseline-444": dict(),
    "baseline-420": dict(sampling=(2, 2)),
    "baseline-422-restart": dict(sampling=(2, 1), restart=3),
    "baseline-grey-restart": dict(grey=True, restart=5),
    "progressive-444": dict(progressive=True),
    "progressive-420": dict(progressive=True, sampling=(2, 2)),
    "progressive-grey-coarse": dict(progressive=True, grey=True, quality_scale=6.0),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_synthetic_matches_float64_decoding(ctx, name):
    img = synthetic_image(45, 77, seed=len(name))  # ragged: neither side a multiple of 16
    data, expect = encode(img, **CASES[name])
    got = ctx.decode_jpeg(data)
    assert got.shape == expect.shape == (45, 77, 3)
    d = np.abs(got.astype(np.int16) - expect.astype(np.int16))
    assert d.max() <= 1, (name, int(d.max()))
    assert d.mean() < 0.02, (name, float(d.mean()))


def test_synthetic_is_a_faithful_image(ctx):
    """The encoder itself is sane: a fine-quantised 4:4:4 file decodes close to
    its source image."""
    img = synthetic_image(32, 48, seed=3)
    data, _ = encode(img, quality_scale=0.01)  # all quantiser steps 1
    got = ctx.decode_jpeg(data).astype(np.float64)
    assert np.abs(got - img).mean() < 1.5


def test_refusals(ctx):
    with pytest.raises(aqua.AquaError) as e:
        ctx.decode_jpeg(b"\x89PNG\r\n\x1a\n" + b"\0" * 32)
    assert e.value.status == aqua.ERR_UNSUPPORTED
    data, _ = encode(synthetic_image(16, 16, 1))
    with pytest.raises(aqua.AquaError):
        ctx.decode_jpeg(data[:60])  # cut inside the headers
    arith = bytearray(data)
    i = arith.index(b"\xFF\xC0")
    arith[i + 1] = 0xC9  # same frame, arithmetic-coded SOF
    with pytest.raises(aqua.AquaError) as e:
        ctx.decode_jpeg(bytes(arith))
    assert e.value.status == aqua.ERR_UNSUPPORTED and "arithmetic" in str(e.value)


@pytest.mark.parametrize("name", ["jpeg_dht_overflow_a.jpg", "jpeg_dht_overflow_b.jpg"])
def test_overfull_huffman_table_is_refused(ctx, name):
    """Mutated test-encoder output whose DHT lists more codes of a length
    than that length holds (found by fuzzing: the decoder used to write its
    9-bit lookup table out of bounds before noticing)."""
    data = open(os.path.join(GOLDEN, name), "rb").read()
    with pytest.raises(aqua.AquaError) as e:
        ctx.decode_jpeg(data)
    assert e.value.status == aqua.ERR_UNSUPPORTED and "Huffman" in str(e.value)


# ---------------------------------------------------------------- reference textures vs nvJPEG
FACTS = json.load(open(os.path.join(GOLDEN, "jpeg_facts.json")))["files"]


def test_nvjpeg_comparison_recorded():
    """What make_jpeg_facts.py measured against nvJPEG on the GPU machine."""
    assert len(FACTS) == 17
    assert {f["frame"] for f in FACTS.values()} == {"sequential", "progressive"}
    for name, f in FACTS.items():
        assert f["mean_abs_diff"] < 0.5, name
        assert f["max_abs_diff"] <= (8 if name == "apple.jpg" else 3), name  # apple: 4:2:0 chroma edges
        assert f["frac_diff_gt_2"] < 0.005, name


@need_ref
@pytest.mark.parametrize("name", sorted(FACTS))
def test_reference_texture_matches_nvjpeg_mean(ctx, name):
    f = FACTS[name]
    img = ctx.decode_jpeg(open(os.path.join(TEXTURES, name), "rb").read())
    assert img.shape == (f["height"], f["width"], 3)
    mean = img.reshape(-1, 3).astype(np.float64).mean(0)
    # |mean(a) - mean(b)| per channel is at most 3x the recorded mean
    # absolute difference over all channels (it can sit in one channel).
    np.testing.assert_allclose(mean, f["nvjpeg_mean_rgb"], atol=3 * f["mean_abs_diff"] + 0.02)
