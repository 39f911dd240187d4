// jpeg.cpp — the JPEG subset described in jpeg.h, written from ITU-T T.81
// (09/92): marker syntax (Annex B), Huffman table specification and decoding
// (Annex C, F.2.2.3), sequential DCT decoding (Annex F.2), progressive DCT
// decoding with spectral selection and successive approximation (Annex G.1.2),
// the 8x8 inverse DCT of A.3.3, and the JFIF 1.02 YCbCr -> RGB transform.
//
// Decoding keeps every quantised coefficient until the last scan (a
// progressive frame refines them scan by scan), then dequantises, runs the
// inverse DCT per block, upsamples subsampled chroma with a centred linear
// filter and converts to RGB.
#include "jpeg.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace aq {
namespace {

struct ZigZag {
    uint8_t nat[64];  // scan position -> row-major index in the 8x8 block (T.81 Figure A.6)
    ZigZag() {
        int i = 0;
        for (int s = 0; s < 15; ++s) {  // anti-diagonal x + y = s, alternating direction
            int lo = std::max(0, s - 7), hi = std::min(s, 7);
            if (s % 2 == 0)
                for (int y = hi; y >= lo; --y) nat[i++] = (uint8_t)(y * 8 + (s - y));
            else
                for (int y = lo; y <= hi; ++y) nat[i++] = (uint8_t)(y * 8 + (s - y));
        }
    }
};
const ZigZag kZz;

// Inverse DCT basis: c[x][u] = C(u)/2 cos((2x+1) u pi / 16), C(0) = 1/sqrt2.
struct IdctBasis {
    float c[8][8];
    IdctBasis() {
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                c[x][u] = (float)((u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 *
                                  std::cos((2.0 * x + 1.0) * u * 3.14159265358979323846 / 16.0));
    }
};
const IdctBasis kIdct;

struct Huff {
    bool present = false;
    uint8_t look_len[512];  // 9-bit prefix -> code length (0: longer than 9 bits)
    uint8_t look_val[512];
    int32_t maxcode[17], mincode[17], valptr[17];
    uint8_t vals[256];
};

// Canonical code assignment of T.81 Annex C from BITS and HUFFVAL.
bool build_huff(Huff& h, const uint8_t* bits, const uint8_t* vals, int nvals) {
    memset(h.look_len, 0, sizeof(h.look_len));
    memcpy(h.vals, vals, (size_t)nvals);
    int k = 0;
    uint32_t code = 0;
    for (int l = 1; l <= 16; ++l) {
        h.valptr[l] = k;
        h.mincode[l] = (int32_t)code;
        for (int i = 0; i < bits[l - 1]; ++i, ++k, ++code) {
            if (code >= (1u << l)) return false;  // more codes than this length holds
            if (l <= 9) {
                uint32_t base = code << (9 - l);
                for (uint32_t j = 0; j < (1u << (9 - l)); ++j) {
                    h.look_len[base + j] = (uint8_t)l;
                    h.look_val[base + j] = vals[k];
                }
            }
        }
        h.maxcode[l] = bits[l - 1] ? (int32_t)code - 1 : -1;
        code <<= 1;
    }
    h.present = true;
    return true;
}

// Entropy-coded segment reader: removes stuffed zero bytes after 0xFF and
// feeds zeros once a marker is reached (T.81 F.2.2.5).
struct Bits {
    const uint8_t* p;
    const uint8_t* end;
    uint32_t acc = 0;
    int n = 0;
    bool at_marker = false;

    void fill() {
        while (n <= 24) {
            uint32_t b = 0;
            if (!at_marker && p < end) {
                if (*p == 0xFF) {
                    if (p + 1 < end && p[1] == 0x00) {
                        b = 0xFF;
                        p += 2;
                    } else {
                        at_marker = true;
                    }
                } else {
                    b = *p++;
                }
            }
            acc |= b << (24 - n);
            n += 8;
        }
    }
    uint32_t get(int k) {  // k in 1..16
        fill();
        uint32_t v = acc >> (32 - k);
        acc <<= k;
        n -= k;
        return v;
    }
    int bit() { return (int)get(1); }
    int decode(const Huff& h) {
        fill();
        uint32_t pre = acc >> 23;
        int l = h.look_len[pre];
        if (l) {
            acc <<= l;
            n -= l;
            return h.look_val[pre];
        }
        for (l = 10; l <= 16; ++l) {
            int32_t code = (int32_t)(acc >> (32 - l));
            if (code <= h.maxcode[l]) {
                acc <<= l;
                n -= l;
                return h.vals[h.valptr[l] + code - h.mincode[l]];
            }
        }
        return -1;
    }
    // Byte-aligns and consumes the RSTn marker a restart interval ends with.
    bool restart() {
        acc = 0;
        n = 0;
        if (!at_marker) {  // skip to the marker (padding bits are 1s)
            while (p + 1 < end && !(p[0] == 0xFF && p[1] != 0x00)) ++p;
        }
        at_marker = false;
        if (p + 1 < end && p[0] == 0xFF && p[1] >= 0xD0 && p[1] <= 0xD7) {
            p += 2;
            return true;
        }
        return false;
    }
};

// Sign extension of an s-bit magnitude category (T.81 F.2.2.1, EXTEND).
inline int extend(uint32_t v, int s) { return v < (1u << (s - 1)) ? (int)v - (1 << s) + 1 : (int)v; }

struct Comp {
    int id = 0, h = 1, v = 1, tq = 0;
    int bw = 0, bh = 0;    // blocks per row / column, padded to whole MCUs
    int rbw = 0, rbh = 0;  // blocks that cover the component's own samples
    int dc_pred = 0;
    int td = 0, ta = 0;    // table selectors of the current scan
    std::vector<int16_t> coef;  // bw * bh * 64, natural order
    std::vector<uint8_t> plane;  // (bw * 8) x (bh * 8) samples
};

struct Decoder {
    const uint8_t* d;
    size_t n;
    size_t pos = 0;
    uint16_t qt[4][64];  // natural order
    bool qt_set[4] = {false, false, false, false};
    Huff dc[4], ac[4];
    std::vector<Comp> comps;
    int W = 0, H = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    bool progressive = false, frame = false;
    int restart_interval = 0;
    int adobe_transform = -1;
    bool jfif = false;
    uint32_t eobrun = 0;

    uint16_t be16(size_t at) const { return (uint16_t)((d[at] << 8) | d[at + 1]); }

    std::string segment_dqt(size_t at, size_t len) {
        size_t e = at + len;
        while (at < e) {
            int pq = d[at] >> 4, tq = d[at] & 15;
            ++at;
            if (tq > 3 || pq > 1) return "bad DQT";
            size_t need = pq ? 128 : 64;
            if (at + need > e) return "short DQT";
            for (int k = 0; k < 64; ++k)
                qt[tq][kZz.nat[k]] = pq ? be16(at + 2 * (size_t)k) : d[at + (size_t)k];
            qt_set[tq] = true;
            at += need;
        }
        return "";
    }

    std::string segment_dht(size_t at, size_t len) {
        size_t e = at + len;
        while (at < e) {
            if (at + 17 > e) return "short DHT";
            int tc = d[at] >> 4, th = d[at] & 15;
            if (tc > 1 || th > 3) return "bad DHT";
            const uint8_t* bits = d + at + 1;
            int total = 0;
            for (int i = 0; i < 16; ++i) total += bits[i];
            if (total > 256 || at + 17 + (size_t)total > e) return "bad DHT counts";
            if (!build_huff(tc ? ac[th] : dc[th], bits, d + at + 17, total)) return "bad Huffman table";
            at += 17 + (size_t)total;
        }
        return "";
    }

    std::string segment_sof(size_t at, size_t len, int marker) {
        if (frame) return "second frame";
        if (len < 6) return "short SOF";
        if (d[at] != 8) return "only 8-bit samples are supported";
        H = be16(at + 1);
        W = be16(at + 3);
        int nc = d[at + 5];
        if (W == 0 || H == 0) return "image size 0 (DNL) is not supported";
        if (nc != 1 && nc != 3) return "only 1 or 3 components are supported";
        if (len < 6 + 3 * (size_t)nc) return "short SOF";
        progressive = marker == 0xC2;
        comps.resize((size_t)nc);
        for (int i = 0; i < nc; ++i) {
            Comp& c = comps[(size_t)i];
            c.id = d[at + 6 + 3 * i];
            c.h = d[at + 7 + 3 * i] >> 4;
            c.v = d[at + 7 + 3 * i] & 15;
            c.tq = d[at + 8 + 3 * i];
            if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3) return "bad component";
            hmax = std::max(hmax, c.h);
            vmax = std::max(vmax, c.v);
        }
        mcux = (W + 8 * hmax - 1) / (8 * hmax);
        mcuy = (H + 8 * vmax - 1) / (8 * vmax);
        if ((size_t)W * (size_t)H > (size_t)1 << 28) return "image too large";
        for (Comp& c : comps) {
            if (hmax % c.h || vmax % c.v) return "non-integer sampling ratios are not supported";
            c.bw = mcux * c.h;
            c.bh = mcuy * c.v;
            int cw = (W * c.h + hmax - 1) / hmax, ch = (H * c.v + vmax - 1) / vmax;
            c.rbw = (cw + 7) / 8;
            c.rbh = (ch + 7) / 8;
            c.coef.assign((size_t)c.bw * (size_t)c.bh * 64, 0);
        }
        frame = true;
        return "";
    }

    // One block of a sequential scan (T.81 F.2.2).
    bool block_sequential(Bits& b, Comp& c, int16_t* blk) {
        int t = b.decode(dc[c.td]);
        if (t < 0 || t > 11) return false;
        int diff = t ? extend(b.get(t), t) : 0;
        c.dc_pred += diff;
        blk[0] = (int16_t)c.dc_pred;
        for (int k = 1; k < 64;) {
            int rs = b.decode(ac[c.ta]);
            if (rs < 0) return false;
            int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r != 15) break;  // EOB
                k += 16;
                continue;
            }
            k += r;
            if (k > 63) return false;
            blk[kZz.nat[k]] = (int16_t)extend(b.get(s), s);
            ++k;
        }
        return true;
    }

    // Progressive DC scans, first and refining (T.81 G.1.2.1).
    bool block_dc(Bits& b, Comp& c, int16_t* blk, int ah, int al) {
        if (ah == 0) {
            int t = b.decode(dc[c.td]);
            if (t < 0 || t > 11) return false;
            int diff = t ? extend(b.get(t), t) : 0;
            c.dc_pred += diff;
            blk[0] = (int16_t)(c.dc_pred * (1 << al));
        } else if (b.bit()) {
            blk[0] = (int16_t)(blk[0] | (1 << al));
        }
        return true;
    }

    // Progressive AC first scan of band [ss, se] (T.81 G.1.2.2).
    bool block_ac_first(Bits& b, Comp& c, int16_t* blk, int ss, int se, int al) {
        if (eobrun) {
            --eobrun;
            return true;
        }
        for (int k = ss; k <= se; ++k) {
            int rs = b.decode(ac[c.ta]);
            if (rs < 0) return false;
            int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r < 15) {  // EOBr: this block and (2^r - 1 + bits) more end here
                    eobrun = (1u << r) - 1u;
                    if (r) eobrun += b.get(r);
                    break;
                }
                k += 15;  // ZRL
                continue;
            }
            k += r;
            if (k > se) return false;
            blk[kZz.nat[k]] = (int16_t)(extend(b.get(s), s) * (1 << al));
        }
        return true;
    }

    // Progressive AC refinement of band [ss, se] (T.81 G.1.2.3): one more
    // bit of every coefficient that is already non-zero, and new +-2^al
    // coefficients placed after skipping r zero-history positions.
    bool block_ac_refine(Bits& b, Comp& c, int16_t* blk, int ss, int se, int al) {
        const int p1 = 1 << al, m1 = -(1 << al);
        int k = ss;
        auto correct = [&](int16_t& co) {
            if (b.bit() && (co & p1) == 0) co = (int16_t)(co + (co >= 0 ? p1 : m1));
        };
        if (eobrun == 0) {
            for (; k <= se; ++k) {
                int rs = b.decode(ac[c.ta]);
                if (rs < 0) return false;
                int r = rs >> 4, s = rs & 15, val = 0;
                if (s) {
                    if (s != 1) return false;
                    val = b.bit() ? p1 : m1;
                } else if (r != 15) {
                    eobrun = 1u << r;
                    if (r) eobrun += b.get(r);
                    break;
                }
                while (k <= se) {
                    int16_t& co = blk[kZz.nat[k]];
                    if (co != 0) {
                        correct(co);
                    } else {
                        if (r == 0) break;
                        --r;
                    }
                    ++k;
                }
                if (val) {
                    if (k > se) return false;
                    blk[kZz.nat[k]] = (int16_t)val;
                }
            }
        }
        if (eobrun > 0) {
            for (; k <= se; ++k) {
                int16_t& co = blk[kZz.nat[k]];
                if (co != 0) correct(co);
            }
            --eobrun;
        }
        return true;
    }

    std::string scan(size_t at, size_t len, size_t& next) {
        if (!frame) return "scan before frame";
        int ns = d[at];
        if (ns < 1 || ns > 4 || len < 4 + 2 * (size_t)ns) return "bad SOS";
        std::vector<Comp*> sc;
        for (int i = 0; i < ns; ++i) {
            int cid = d[at + 1 + 2 * i], t = d[at + 2 + 2 * i];
            Comp* c = nullptr;
            for (Comp& x : comps)
                if (x.id == cid) c = &x;
            if (!c) return "scan names an unknown component";
            c->td = t >> 4;
            c->ta = t & 15;
            if (c->td > 3 || c->ta > 3) return "bad table selector";
            sc.push_back(c);
        }
        size_t q = at + 1 + 2 * (size_t)ns;
        int ss = d[q], se = d[q + 1], ah = d[q + 2] >> 4, al = d[q + 2] & 15;
        if (progressive) {
            if (ss > se || se > 63 || (ss == 0 && se != 0) || (ss > 0 && ns != 1) || al > 13)
                return "bad progressive scan parameters";
        } else if (ss != 0 || se != 63 || ah != 0 || al != 0) {
            return "bad sequential scan parameters";
        }
        for (Comp* c : sc) {
            bool need_dc = !progressive || (ss == 0 && ah == 0);
            bool need_ac = !progressive || ss > 0;
            if (need_dc && !dc[c->td].present) return "missing DC table";
            if (need_ac && !ac[c->ta].present) return "missing AC table";
            c->dc_pred = 0;
        }
        eobrun = 0;
        Bits b{d + at + len, d + n};
        auto one = [&](Comp& c, int bx, int by) -> bool {
            int16_t* blk = &c.coef[((size_t)by * (size_t)c.bw + (size_t)bx) * 64];
            if (!progressive) return block_sequential(b, c, blk);
            if (ss == 0) return block_dc(b, c, blk, ah, al);
            if (ah == 0) return block_ac_first(b, c, blk, ss, se, al);
            return block_ac_refine(b, c, blk, ss, se, al);
        };
        // A scan of one component walks that component's own blocks; an
        // interleaved scan walks MCUs (T.81 A.2).
        const bool single = ns == 1;
        const int units_x = single ? sc[0]->rbw : mcux, units_y = single ? sc[0]->rbh : mcuy;
        const long total = (long)units_x * units_y;
        long todo = restart_interval;
        for (long u = 0; u < total; ++u) {
            if (restart_interval && todo == 0) {
                b.restart();
                for (Comp* c : sc) c->dc_pred = 0;
                eobrun = 0;
                todo = restart_interval;
            }
            int ux = (int)(u % units_x), uy = (int)(u / units_x);
            if (single) {
                if (!one(*sc[0], ux, uy)) return "corrupt entropy-coded data";
            } else {
                for (Comp* c : sc)
                    for (int v = 0; v < c->v; ++v)
                        for (int h = 0; h < c->h; ++h)
                            if (!one(*c, ux * c->h + h, uy * c->v + v)) return "corrupt entropy-coded data";
            }
            if (restart_interval) --todo;
        }
        // Resume marker parsing at the next marker after the scan's data.
        const uint8_t* p = b.p;
        while (p + 1 < d + n && !(p[0] == 0xFF && p[1] != 0x00 && !(p[1] >= 0xD0 && p[1] <= 0xD7))) ++p;
        next = (size_t)(p - d);
        return "";
    }

    void idct_component(Comp& c) {
        c.plane.assign((size_t)c.bw * 8 * (size_t)c.bh * 8, 0);
        const size_t stride = (size_t)c.bw * 8;
        const uint16_t* q = qt[c.tq];
        float tmp[64], f[64];
        for (int by = 0; by < c.bh; ++by)
            for (int bx = 0; bx < c.bw; ++bx) {
                const int16_t* blk = &c.coef[((size_t)by * (size_t)c.bw + (size_t)bx) * 64];
                for (int i = 0; i < 64; ++i) f[i] = (float)blk[i] * (float)q[i];
                for (int y = 0; y < 8; ++y)  // columns: tmp[y][u] = sum_v c[y][v] F[v][u]
                    for (int u = 0; u < 8; ++u) {
                        float s = 0.0f;
                        for (int v = 0; v < 8; ++v) s += kIdct.c[y][v] * f[v * 8 + u];
                        tmp[y * 8 + u] = s;
                    }
                uint8_t* out = &c.plane[(size_t)by * 8 * stride + (size_t)bx * 8];
                for (int y = 0; y < 8; ++y)
                    for (int x = 0; x < 8; ++x) {
                        float s = 0.0f;
                        for (int u = 0; u < 8; ++u) s += kIdct.c[x][u] * tmp[y * 8 + u];
                        int val = (int)std::lround(s) + 128;
                        out[(size_t)y * stride + (size_t)x] = (uint8_t)std::min(255, std::max(0, val));
                    }
            }
    }

    // Sample of component c at image pixel (x, y): centred linear
    // interpolation when the component is subsampled.
    float sample(const Comp& c, int x, int y) const {
        const size_t stride = (size_t)c.bw * 8;
        if (c.h == hmax && c.v == vmax) return c.plane[(size_t)y * stride + (size_t)x];
        const int cw = (W * c.h + hmax - 1) / hmax, ch = (H * c.v + vmax - 1) / vmax;
        float fx = ((float)x + 0.5f) * (float)c.h / (float)hmax - 0.5f;
        float fy = ((float)y + 0.5f) * (float)c.v / (float)vmax - 0.5f;
        fx = std::min(std::max(fx, 0.0f), (float)(cw - 1));
        fy = std::min(std::max(fy, 0.0f), (float)(ch - 1));
        int x0 = (int)fx, y0 = (int)fy;
        int x1 = std::min(x0 + 1, cw - 1), y1 = std::min(y0 + 1, ch - 1);
        float ax = fx - (float)x0, ay = fy - (float)y0;
        auto at = [&](int xx, int yy) { return (float)c.plane[(size_t)yy * stride + (size_t)xx]; };
        float a = at(x0, y0) + (at(x1, y0) - at(x0, y0)) * ax;
        float bb = at(x0, y1) + (at(x1, y1) - at(x0, y1)) * ax;
        return a + (bb - a) * ay;
    }

    std::string finish(JpegImage& out) {
        for (Comp& c : comps) {
            if (!qt_set[c.tq]) return "missing quantisation table";
            idct_component(c);
        }
        out.w = W;
        out.h = H;
        out.components = (int)comps.size();
        out.progressive = progressive;
        out.rgb.assign((size_t)W * (size_t)H * 3, 0);
        // Three components are YCbCr unless an Adobe marker says transform 0
        // or the component ids spell R, G, B.
        bool rgb_coded = comps.size() == 3 &&
                         (adobe_transform == 0 ||
                          (!jfif && adobe_transform < 0 && comps[0].id == 'R' && comps[1].id == 'G' && comps[2].id == 'B'));
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                uint8_t* o = &out.rgb[((size_t)y * (size_t)W + (size_t)x) * 3];
                if (comps.size() == 1) {
                    o[0] = o[1] = o[2] = comps[0].plane[(size_t)y * (size_t)comps[0].bw * 8 + (size_t)x];
                    continue;
                }
                float c0 = sample(comps[0], x, y), c1 = sample(comps[1], x, y), c2 = sample(comps[2], x, y);
                float r, g, bl;
                if (rgb_coded) {
                    r = c0; g = c1; bl = c2;
                } else {
                    float cb = c1 - 128.0f, cr = c2 - 128.0f;
                    r = c0 + 1.402f * cr;
                    g = c0 - 0.344136f * cb - 0.714136f * cr;
                    bl = c0 + 1.772f * cb;
                }
                o[0] = (uint8_t)std::min(255L, std::max(0L, std::lround(r)));
                o[1] = (uint8_t)std::min(255L, std::max(0L, std::lround(g)));
                o[2] = (uint8_t)std::min(255L, std::max(0L, std::lround(bl)));
            }
        return "";
    }

    std::string run(JpegImage& out) {
        if (n < 4 || d[0] != 0xFF || d[1] != 0xD8) return "not a JPEG (no SOI)";
        pos = 2;
        bool scanned = false;
        while (pos + 4 <= n) {
            if (d[pos] != 0xFF) return "marker expected";
            int m = d[pos + 1];
            if (m == 0xFF) { ++pos; continue; }  // fill byte
            if (m == 0xD9) break;                 // EOI
            if (m >= 0xD0 && m <= 0xD7) { pos += 2; continue; }
            size_t len = be16(pos + 2);
            if (len < 2 || pos + 2 + len > n) return "truncated segment";
            size_t at = pos + 4, body = len - 2;
            std::string e;
            switch (m) {
                case 0xDB: e = segment_dqt(at, body); break;
                case 0xC4: e = segment_dht(at, body); break;
                case 0xC0: case 0xC1: case 0xC2: e = segment_sof(at, body, m); break;
                case 0xC3: case 0xC5: case 0xC6: case 0xC7: return "lossless and hierarchical JPEG are not supported";
                case 0xC9: case 0xCA: case 0xCB: case 0xCD: case 0xCE: case 0xCF:
                case 0xCC: return "arithmetic-coded JPEG is not supported";
                case 0xDD:
                    if (body < 2) return "short DRI";
                    restart_interval = be16(at);
                    break;
                case 0xE0:
                    if (body >= 5 && memcmp(d + at, "JFIF", 5) == 0) jfif = true;
                    break;
                case 0xEE:
                    if (body >= 12 && memcmp(d + at, "Adobe", 5) == 0) adobe_transform = d[at + 11];
                    break;
                case 0xDA: {
                    size_t next = 0;
                    e = scan(at, body, next);
                    if (!e.empty()) return e;
                    scanned = true;
                    pos = next;
                    continue;
                }
                default: break;  // APPn, COM, DNL-less extensions: skipped
            }
            if (!e.empty()) return e;
            pos += 2 + len;
        }
        if (!frame || !scanned) return "no frame or no scan";
        return finish(out);
    }
};

}  // namespace

std::string jpeg_decode(const uint8_t* data, size_t n, JpegImage& out) {
    out = JpegImage{};
    if (!data) return "no data";
    Decoder dec{data, n};
    return dec.run(out);
}

}  // namespace aq
