// scene.cpp — BSON .mesh reader, scene/integrator JSON loaders, and the
// seeded procedural scenes 1-5.
#include "scene.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iterator>
#include <map>
#include <sstream>
#include <thread>

#include "aq_math.h"
#include "jpeg.h"
#include "json.h"

namespace aq {

// ======================================================== deterministic math
// Range-reduced Taylor series in double; only + - * / are used, so every
// IEEE-754 host produces the same bits (no libm differences between hosts).
static const double kTwoPi = 6.283185307179586476925286766559;
double det_sin(double x) {
    double k = std::floor(x / kTwoPi + 0.5);
    double r = x - k * kTwoPi;  // [-pi, pi]
    // sin(r) = r - r^3/3! + ... up to r^25: error < 1e-16 on [-pi, pi]
    double r2 = r * r, term = r, sum = r;
    for (int n = 1; n <= 12; ++n) {
        term = -term * r2 / (double)((2 * n) * (2 * n + 1));
        sum += term;
    }
    return sum;
}
double det_cos(double x) { return det_sin(x + kTwoPi / 4.0); }
double det_exp(double x) {
    // exp(x) = 2^k * exp(r), |r| <= ln2/2
    const double ln2 = 0.693147180559945309417232121458;
    double k = std::floor(x / ln2 + 0.5);
    double r = x - k * ln2;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n <= 20; ++n) {
        term = term * r / (double)n;
        sum += term;
    }
    return std::ldexp(sum, (int)k);
}
double det_log(double x) {
    // log(x) = 2 atanh((m-1)/(m+1)) + e ln2, m in [sqrt(1/2), sqrt(2))
    const double ln2 = 0.693147180559945309417232121458;
    int e;
    double m = std::frexp(x, &e);  // [0.5, 1)
    if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
    double s = (m - 1.0) / (m + 1.0), s2 = s * s, term = s, sum = s;
    for (int n = 1; n <= 30; ++n) {
        term *= s2;
        sum += term / (double)(2 * n + 1);
    }
    return 2.0 * sum + (double)e * ln2;
}

// ======================================================== host RNG (PCG32)
struct HostRng {
    uint64_t state, inc;
    HostRng(uint64_t seed, uint64_t stream) { state = pcg32_seed(seed, stream, inc); }
    uint32_t next() { return pcg32_next(state, inc); }
    double uniform() { return (double)(next() >> 8) * (1.0 / 16777216.0); }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    double log_uniform(double a, double b) {
        return det_exp(det_log(a) + uniform() * (det_log(b) - det_log(a)));
    }
    int range(int n) { return (int)(uniform() * n) % n; }
};

// ======================================================== BSON
namespace {
struct BsonReader {
    const uint8_t* d;
    size_t n;
    std::string where;
    [[noreturn]] void fail(const std::string& m) {
        throw SceneError(AQUA_ERR_PARSE, where + ": BSON " + m);
    }
    int32_t i32(size_t off) {
        if (off + 4 > n) fail("truncated int32");
        int32_t v;
        memcpy(&v, d + off, 4);  // BSON is little-endian, as are both build hosts
        return v;
    }
    int64_t i64(size_t off) {
        if (off + 8 > n) fail("truncated int64");
        int64_t v;
        memcpy(&v, d + off, 8);
        return v;
    }
    double f64(size_t off) {
        if (off + 8 > n) fail("truncated double");
        double v;
        memcpy(&v, d + off, 8);
        return v;
    }
    std::string cstr(size_t& off) {
        size_t st = off;
        while (off < n && d[off] != 0) ++off;
        if (off >= n) fail("unterminated key");
        std::string s((const char*)d + st, off - st);
        ++off;
        return s;
    }
    // Calls fn(type, key, value_offset, end_of_value) for each element.
    template <class F>
    void walk(size_t off, F&& fn) {
        int32_t len = i32(off);
        if (len < 5 || off + (size_t)len > n) fail("bad document length");
        size_t end = off + (size_t)len - 1;
        if (d[end] != 0) fail("document not NUL-terminated");
        size_t p = off + 4;
        while (p < end) {
            uint8_t t = d[p++];
            std::string key = cstr(p);
            size_t vlen;
            switch (t) {
                case 0x01: vlen = 8; break;
                case 0x02: vlen = 4 + (size_t)i32(p); break;
                case 0x03:
                case 0x04: vlen = (size_t)i32(p); break;
                case 0x08: vlen = 1; break;
                case 0x0A: vlen = 0; break;
                case 0x10: vlen = 4; break;
                case 0x12: vlen = 8; break;
                default: fail("unsupported element type " + std::to_string(t));
            }
            if (p + vlen > end) fail("element overruns document");
            fn(t, key, p, p + vlen);
            p += vlen;
        }
    }
    double number(uint8_t t, size_t p) {
        if (t == 0x01) return f64(p);
        if (t == 0x10) return (double)i32(p);
        if (t == 0x12) return (double)i64(p);
        fail("expected a number");
    }
    // Array of arrays of numbers with `width` entries each.
    template <class T>
    void tuples(uint8_t t, size_t p, int width, std::vector<T>& out) {
        if (t != 0x04) fail("expected an array");
        walk(p, [&](uint8_t t2, const std::string&, size_t p2, size_t) {
            if (t2 != 0x04) fail("expected an inner array");
            int cnt = 0;
            walk(p2, [&](uint8_t t3, const std::string&, size_t p3, size_t) {
                out.push_back((T)number(t3, p3));
                ++cnt;
            });
            if (cnt != width) fail("inner array of length " + std::to_string(cnt) +
                                   ", expected " + std::to_string(width));
        });
    }
};
}  // namespace

MeshData parse_mesh_bson(const uint8_t* data, size_t n) {
    BsonReader r{data, n, "mesh"};
    MeshData m;
    bool have_v = false, have_i = false;
    r.walk(0, [&](uint8_t t, const std::string& key, size_t p, size_t) {
        if (key == "name") {
            if (t != 0x02) r.fail("name is not a string");
            int32_t l = r.i32(p);
            if (l < 1) r.fail("bad string length");
            m.name.assign((const char*)data + p + 4, (size_t)l - 1);
        } else if (key == "vertices") {
            r.tuples(t, p, 3, m.positions);
            have_v = true;
        } else if (key == "normals") {
            r.tuples(t, p, 3, m.normals);
        } else if (key == "texcoords") {
            r.tuples(t, p, 2, m.texcoords);
        } else if (key == "indices") {
            r.tuples(t, p, 3, m.indices);
            have_i = true;
        }
    });
    if (!have_v || !have_i) r.fail("missing vertices or indices");
    size_t nv = m.positions.size() / 3;
    for (int64_t ix : m.indices)
        if (ix < 0 || (size_t)ix >= nv) r.fail("index out of range");
    // A NaN or infinite coordinate would poison box bounds and shading.
    for (const std::vector<double>* v : {&m.positions, &m.normals, &m.texcoords})
        for (double x : *v)
            if (!std::isfinite(x)) r.fail("non-finite vertex attribute");
    if (!m.normals.empty() && m.normals.size() != m.positions.size()) m.normals.clear();
    if (!m.texcoords.empty() && m.texcoords.size() / 2 != nv) m.texcoords.clear();
    return m;
}

static std::vector<uint8_t> read_file(const std::string& path, aqua_status missing) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw SceneError(missing, "cannot open " + path);
    std::vector<uint8_t> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    return buf;
}

MeshData read_mesh_bson(const std::string& path) {
    auto buf = read_file(path, AQUA_ERR_MISSING_ASSET);
    try {
        return parse_mesh_bson(buf.data(), buf.size());
    } catch (SceneError& e) {
        throw SceneError(e.status, path + ": " + e.what());
    }
}

// ======================================================== camera / lights
aqua_camera make_camera(int w, int h, float fov_deg, float lens_radius, float focal,
                        const double t[3], const double rdeg[3]) {
    aqua_camera c{};
    c.width = w; c.height = h;
    c.fov_deg = fov_deg; c.lens_radius = lens_radius; c.focal = focal;
    const double d2r = 3.14159265358979323846 / 180.0;
    double cx = det_cos(rdeg[0] * d2r), sx = det_sin(rdeg[0] * d2r);
    double cy = det_cos(rdeg[1] * d2r), sy = det_sin(rdeg[1] * d2r);
    double cz = det_cos(rdeg[2] * d2r), sz = det_sin(rdeg[2] * d2r);
    // R = Rz * Ry * Rx; columns are the camera's right, up, back axes.
    double R[3][3] = {
        {cz * cy, cz * sy * sx - sz * cx, cz * sy * cx + sz * sx},
        {sz * cy, sz * sy * sx + cz * cx, sz * sy * cx - cz * sx},
        {-sy, cy * sx, cy * cx}};
    for (int i = 0; i < 3; ++i) {
        c.pos[i] = (float)t[i];
        c.right[i] = (float)R[i][0];
        c.up[i] = (float)R[i][1];
        c.back[i] = (float)R[i][2];
    }
    return c;
}

void camera_look_at(aqua_camera& c, const float eye[3], const float target[3], const float upv[3]) {
    v3 e = mk(eye[0], eye[1], eye[2]), t = mk(target[0], target[1], target[2]);
    v3 back = normalize(e - t);
    v3 right = normalize(cross(mk(upv[0], upv[1], upv[2]), back));
    v3 up = cross(back, right);
    for (int i = 0; i < 3; ++i) c.pos[i] = eye[i];
    c.right[0] = right.x; c.right[1] = right.y; c.right[2] = right.z;
    c.up[0] = up.x; c.up[1] = up.y; c.up[2] = up.z;
    c.back[0] = back.x; c.back[1] = back.y; c.back[2] = back.z;
}

static double light_power(const aqua_light& l) {
    double L = 0.2126 * l.radiance[0] + 0.7152 * l.radiance[1] + 0.0722 * l.radiance[2];
    if (l.type == AQUA_LIGHT_POINT) return L * 4.0 * 3.14159265358979323846;
    v3 e1 = mk(l.e1[0], l.e1[1], l.e1[2]), e2 = mk(l.e2[0], l.e2[1], l.e2[2]);
    double area = length(cross(e1, e2)) * (l.type == AQUA_LIGHT_TRIANGLE ? 0.5 : 1.0);
    return L * area * 3.14159265358979323846;
}

void finalize_lights(HostScene& s) {
    double total = 0.0;
    for (auto& l : s.lights) total += light_power(l);
    for (auto& l : s.lights)
        l.pmf = total > 0.0 ? (float)(light_power(l) / total) : 1.0f / (float)s.lights.size();
}

// ======================================================== scene JSON
namespace {

v3 read3(const Json& j) {
    if (!j.is_array() || j.arr.size() != 3) throw JsonError("expected a 3-array");
    return mk((float)j.arr[0].as_number(), (float)j.arr[1].as_number(), (float)j.arr[2].as_number());
}

// Texture enum (cbox.json:5-9, room.json:6): Float, Float3, Srgb, Image.
struct TexVal {
    v3 value{0, 0, 0};
    bool image = false;
    std::string path;
};
TexVal read_tex(const Json& j) {
    if (!j.is_object() || j.obj.size() != 1) throw JsonError("texture must be a one-key object");
    const std::string& tag = j.obj[0].first;
    const Json& v = j.obj[0].second;
    TexVal t;
    if (tag == "Float") {
        float f = (float)v.as_number();
        t.value = mk(f, f, f);
    } else if (tag == "Float3") {
        t.value = read3(v);
    } else if (tag == "Srgb") {
        v3 c = read3(v);
        t.value = mk((float)srgb_to_linear(c.x), (float)srgb_to_linear(c.y), (float)srgb_to_linear(c.z));
    } else if (tag == "Image") {
        t.image = true;
        t.path = v.as_string();
        std::replace(t.path.begin(), t.path.end(), '\\', '/');
    } else {
        throw JsonError("unknown texture variant \"" + tag + "\"");
    }
    return t;
}

struct Bsdf_ {
    aqua_material m;
    v3 emission;
};

// `Image` textures by file, so materials that share a file share a texture.
// Files are only checked while the JSON is read; decoding runs afterwards on
// all host threads (decode_textures). Texture rows are stored bottom-up
// (row 0 = the image's last row): v = 0 is the bottom edge of the image, as
// in the OBJ texture coordinates the .mesh files carry.
struct TexCache {
    HostScene& s;
    std::map<std::string, int> index;
    struct Pending {
        int tex;
        std::string path, bsdf;
    };
    std::vector<Pending> pending;
};

// Index of the texture for `full`, or -1 when the file is missing and
// allow_missing is set (the caller then uses mid-grey).
int image_texture(TexCache& tc, const std::string& full, bool allow_missing, const std::string& name) {
    auto it = tc.index.find(full);
    if (it != tc.index.end()) return it->second;
    std::ifstream f(full, std::ios::binary);
    if (!f) {
        if (allow_missing) return tc.index[full] = -1;
        throw SceneError(AQUA_ERR_MISSING_ASSET, "bsdf \"" + name + "\": texture " + full + " is missing");
    }
    tc.s.textures.push_back(Texture{});
    const int ti = (int)tc.s.textures.size() - 1;
    tc.pending.push_back({ti, full, name});
    return tc.index[full] = ti;
}

// Decodes the pending textures in parallel. A file the decoder refuses fails
// the load with AQUA_ERR_UNSUPPORTED, or with allow_missing becomes a 1x1
// texture of linear 0.5 (the mid-grey stand-in).
void decode_textures(TexCache& tc, bool allow_missing) {
    const size_t n = tc.pending.size();
    std::vector<std::string> errs(n);
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t k = next++; k < n; k = next++) {
            const TexCache::Pending& p = tc.pending[k];
            std::ifstream f(p.path, std::ios::binary);
            std::vector<uint8_t> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
            JpegImage img;
            errs[k] = jpeg_decode(data.data(), data.size(), img);
            Texture& t = tc.s.textures[(size_t)p.tex];
            if (!errs[k].empty()) {
                t.w = t.h = 1;
                t.rgba = {188, 188, 188, 255};  // sRGB encoding of linear 0.5
                continue;
            }
            t.w = img.w;
            t.h = img.h;
            t.rgba.resize((size_t)img.w * (size_t)img.h * 4);
            for (int y = 0; y < img.h; ++y) {
                const uint8_t* src = &img.rgb[(size_t)(img.h - 1 - y) * (size_t)img.w * 3];
                uint8_t* dst = &t.rgba[(size_t)y * (size_t)img.w * 4];
                for (int x = 0; x < img.w; ++x) {
                    dst[4 * x] = src[3 * x];
                    dst[4 * x + 1] = src[3 * x + 1];
                    dst[4 * x + 2] = src[3 * x + 2];
                    dst[4 * x + 3] = 255;
                }
            }
        }
    };
    const size_t threads = std::min<size_t>(n, std::max(1u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (size_t i = 1; i < threads; ++i) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    if (!allow_missing)
        for (size_t k = 0; k < n; ++k)
            if (!errs[k].empty())
                throw SceneError(AQUA_ERR_UNSUPPORTED, "bsdf \"" + tc.pending[k].bsdf + "\": texture " +
                                                           tc.pending[k].path + ": " + errs[k]);
    tc.pending.clear();
}

Bsdf_ read_bsdf(const Json& j, const std::string& dir, bool allow_missing, const std::string& name,
                TexCache& tc) {
    if (!j.is_object() || j.obj.size() != 1) throw JsonError("bsdf must be a one-key object");
    if (j.obj[0].first != "Principled")
        throw SceneError(AQUA_ERR_UNSUPPORTED, "bsdf \"" + name + "\": variant \"" + j.obj[0].first +
                                                   "\" is not supported (only Principled)");
    const Json& p = j.obj[0].second;
    Bsdf_ b{};
    b.m.base_texture = -1;
    b.m.reserved[0] = b.m.reserved[1] = 0;
    auto scalar = [&](const char* key, float dflt) {
        const Json* v = p.find(key);
        if (!v) return dflt;
        TexVal t = read_tex(*v);
        if (t.image)
            throw SceneError(AQUA_ERR_UNSUPPORTED, std::string("bsdf \"") + name + "\": image-valued " + key);
        return t.value.x;
    };
    const Json* col = p.find("color");
    v3 base = mk(0.8f, 0.8f, 0.8f);
    if (col) {
        TexVal t = read_tex(*col);
        if (t.image) {
            int ti = image_texture(tc, t.path[0] == '/' ? t.path : dir + "/" + t.path, allow_missing, name);
            if (ti >= 0) {
                base = mk(1.0f, 1.0f, 1.0f);  // the texture is the base colour
                b.m.base_texture = ti;
            } else {
                base = mk(0.5f, 0.5f, 0.5f);  // mid-grey stand-in
            }
        } else {
            base = t.value;
        }
    }
    b.m.base_color[0] = base.x; b.m.base_color[1] = base.y; b.m.base_color[2] = base.z;
    b.m.metallic = scalar("metallic", 0.0f);
    b.m.roughness = scalar("roughness", 0.5f);
    b.m.specular = scalar("specular", 0.5f);
    b.m.specular_tint = scalar("specular_tint", 0.0f);
    b.m.sheen = scalar("sheen", 0.0f);
    b.m.sheen_tint = scalar("sheen_tint", 0.5f);
    b.m.clearcoat = scalar("clearcoat", 0.0f);
    b.m.clearcoat_roughness = scalar("clearcoat_roughness", 0.03f);
    b.m.transmission = scalar("transmission", 0.0f);
    b.m.ior = scalar("ior", 1.45f);
    const Json* em = p.find("emission");
    b.emission = mk(0, 0, 0);
    if (em) {
        TexVal t = read_tex(*em);
        if (t.image) throw SceneError(AQUA_ERR_UNSUPPORTED, "bsdf \"" + name + "\": image-valued emission");
        b.emission = t.value;
    }
    // Principled parameters live in [0, 1]; colours and emission are
    // non-negative. Outside that the lobe weights turn negative or NaN.
    auto unit = [&](const char* key, float v) {
        if (!(v >= 0.0f && v <= 1.0f)) throw JsonError("bsdf \"" + name + "\": " + key + " must lie in [0, 1]");
    };
    unit("metallic", b.m.metallic);
    unit("roughness", b.m.roughness);
    unit("specular", b.m.specular);
    unit("specular_tint", b.m.specular_tint);
    unit("sheen", b.m.sheen);
    unit("sheen_tint", b.m.sheen_tint);
    unit("clearcoat", b.m.clearcoat);
    unit("clearcoat_roughness", b.m.clearcoat_roughness);
    unit("transmission", b.m.transmission);
    if (!(b.m.ior >= 1.0f && b.m.ior <= 4.0f)) throw JsonError("bsdf \"" + name + "\": ior must lie in [1, 4]");
    if (!(base.x >= 0.0f && base.y >= 0.0f && base.z >= 0.0f))
        throw JsonError("bsdf \"" + name + "\": color must be non-negative");
    if (!(b.emission.x >= 0.0f && b.emission.y >= 0.0f && b.emission.z >= 0.0f))
        throw JsonError("bsdf \"" + name + "\": emission must be non-negative");
    return b;
}

}  // namespace

static void push_tri(HostScene& s, v3 a, v3 b, v3 c, int mat, const float* uv = nullptr) {
    float v[9] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z};
    s.verts.insert(s.verts.end(), v, v + 9);
    if (uv) s.uvs.insert(s.uvs.end(), uv, uv + 6);
    else s.uvs.insert(s.uvs.end(), 6, 0.0f);
    s.tri_mat.push_back(mat);
}

HostScene load_scene_json(const std::string& path, bool allow_missing) {
    std::vector<uint8_t> raw = read_file(path, AQUA_ERR_IO);
    std::string text(raw.begin(), raw.end());
    std::string dir = ".";
    size_t slash = path.find_last_of('/');
    if (slash != std::string::npos) dir = path.substr(0, slash);
    HostScene s;
    TexCache tc{s, {}};
    bool any_normals = false;
    std::vector<v3> mat_emission;
    try {
        Json root = json_parse(text);
        if (!root.is_object()) throw JsonError("scene root must be an object");
        // named_bsdfs (cbox.json:2)
        std::vector<std::string> names;
        if (const Json* nb = root.find("named_bsdfs")) {
            for (auto& kv : nb->obj) {
                Bsdf_ b = read_bsdf(kv.second, dir, allow_missing, kv.first, tc);
                s.mats.push_back(b.m);
                s.mat_names.push_back(kv.first);
                mat_emission.push_back(b.emission);
            }
        }
        // camera (cbox.json:516-543)
        const Json& cam = root.at("camera");
        if (!cam.is_object() || cam.obj.size() != 1 || cam.obj[0].first != "Perspective")
            throw JsonError("camera must be {\"Perspective\": {...}}");
        const Json& pc = cam.obj[0].second;
        const Json& res = pc.at("res");
        if (!res.is_array() || res.arr.size() != 2) throw JsonError("camera res must be [w, h]");
        const double wd = res.arr[0].as_number(), hd = res.arr[1].as_number();
        // the same bound as aqua_scene_set_resolution
        if (!(wd >= 1 && hd >= 1 && wd <= 16384 && hd <= 16384) || wd != std::floor(wd) || hd != std::floor(hd))
            throw JsonError("camera res must be two integers in [1, 16384]");
        const int W = (int)wd, H = (int)hd;
        double t[3] = {0, 0, 0}, r[3] = {0, 0, 0};
        if (const Json* tr = pc.find("transform")) {
            if (const Json* tt = tr->find("translate")) { v3 v = read3(*tt); t[0] = v.x; t[1] = v.y; t[2] = v.z; }
            if (const Json* rr = tr->find("rotate")) { v3 v = read3(*rr); r[0] = v.x; r[1] = v.y; r[2] = v.z; }
        }
        const double fov = pc.at("fov").as_number();
        const double lens = pc.find("lens_radius") ? pc.at("lens_radius").as_number() : 0.0;
        const double focal = pc.find("focal") ? pc.at("focal").as_number() : 1.0;
        if (!(fov > 0 && fov < 180)) throw JsonError("camera fov must lie in (0, 180) degrees");
        if (!(lens >= 0 && lens < 1e30) || !(focal > 0 && focal < 1e30))
            throw JsonError("camera lens_radius must be >= 0 and focal > 0");
        s.cam = make_camera(W, H, (float)fov, (float)lens, (float)focal, t, r);
        // lights (cbox.json:544-561)
        if (const Json* ls = root.find("lights")) {
            for (auto& l : ls->arr) {
                if (!l.is_object() || l.obj.size() != 1) throw JsonError("light must be a one-key object");
                if (l.obj[0].first != "Point")
                    throw SceneError(AQUA_ERR_UNSUPPORTED, "light variant \"" + l.obj[0].first + "\" is not supported");
                const Json& pl = l.obj[0].second;
                aqua_light L{};
                L.type = AQUA_LIGHT_POINT;
                v3 p = read3(pl.at("pos"));
                TexVal e = read_tex(pl.at("emission"));
                if (e.image) throw SceneError(AQUA_ERR_UNSUPPORTED, "image-valued light emission");
                L.p0[0] = p.x; L.p0[1] = p.y; L.p0[2] = p.z;
                L.radiance[0] = e.value.x; L.radiance[1] = e.value.y; L.radiance[2] = e.value.z;
                s.lights.push_back(L);
            }
        }
        // shapes (cbox.json:562-627)
        const Json& shapes = root.at("shapes");
        for (auto& sh : shapes.arr) {
            if (!sh.is_object() || sh.obj.size() != 1 || sh.obj[0].first != "Mesh")
                throw SceneError(AQUA_ERR_UNSUPPORTED, "only Mesh shapes are supported");
            const Json& m = sh.obj[0].second;
            if (!m.is_array() || m.arr.size() != 2) throw JsonError("Mesh must be [file, bsdf]");
            std::string file = m.arr[0].as_string();
            std::replace(file.begin(), file.end(), '\\', '/');
            const Json& bref = m.arr[1];
            int mat = -1;
            if (bref.is_object() && bref.obj.size() == 1 && bref.obj[0].first == "Named") {
                const std::string& nm = bref.obj[0].second.as_string();
                for (size_t i = 0; i < s.mat_names.size(); ++i)
                    if (s.mat_names[i] == nm) mat = (int)i;
                if (mat < 0) throw JsonError("shape refers to unknown bsdf \"" + nm + "\"");
            } else {
                Bsdf_ b = read_bsdf(bref, dir, allow_missing, file, tc);
                s.mats.push_back(b.m);
                s.mat_names.push_back(file);
                mat_emission.push_back(b.emission);
                mat = (int)s.mats.size() - 1;
            }
            MeshData md;
            try {
                md = read_mesh_bson(!file.empty() && file[0] == '/' ? file : dir + "/" + file);
            } catch (SceneError& e) {
                if (e.status == AQUA_ERR_MISSING_ASSET && allow_missing) continue;
                throw;
            }
            s.num_meshes++;
            v3 em = mat_emission[(size_t)mat];
            bool emissive = em.x > 0 || em.y > 0 || em.z > 0;
            size_t ntri = md.indices.size() / 3;
            bool has_uv = !md.texcoords.empty();
            const bool has_n = !md.normals.empty();
            any_normals = any_normals || has_n;
            for (size_t k = 0; k < ntri; ++k) {
                v3 P[3];
                float uv[6] = {0, 0, 0, 0, 0, 0};
                float nv[9];
                for (int c = 0; c < 3; ++c) {
                    size_t vi = (size_t)md.indices[3 * k + c];
                    P[c] = mk((float)md.positions[3 * vi], (float)md.positions[3 * vi + 1],
                              (float)md.positions[3 * vi + 2]);
                    if (has_uv) {
                        uv[2 * c] = (float)md.texcoords[2 * vi];
                        uv[2 * c + 1] = (float)md.texcoords[2 * vi + 1];
                    }
                    for (int a = 0; a < 3; ++a) nv[3 * c + a] = has_n ? (float)md.normals[3 * vi + (size_t)a] : 0.0f;
                }
                if (!has_n) {  // a flat mesh among smooth ones: its face normal at every vertex
                    double e1[3], e2[3];
                    for (int a = 0; a < 3; ++a) {
                        e1[a] = (double)comp(P[1], a) - comp(P[0], a);
                        e2[a] = (double)comp(P[2], a) - comp(P[0], a);
                    }
                    double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                    e1[0] * e2[1] - e1[1] * e2[0]};
                    double l = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
                    for (int c = 0; c < 3; ++c)
                        for (int a = 0; a < 3; ++a) nv[3 * c + a] = l > 0.0 ? (float)(cr[a] / l) : 0.0f;
                }
                s.nrm.insert(s.nrm.end(), nv, nv + 9);
                push_tri(s, P[0], P[1], P[2], mat, uv);
                if (emissive) {
                    aqua_light L{};
                    L.type = AQUA_LIGHT_TRIANGLE;
                    v3 e1 = P[1] - P[0], e2 = P[2] - P[0];
                    for (int c = 0; c < 3; ++c) {
                        L.p0[c] = comp(P[0], c); L.e1[c] = comp(e1, c); L.e2[c] = comp(e2, c);
                        L.radiance[c] = comp(em, c);
                    }
                    s.lights.push_back(L);
                    s.tri_light.push_back((int32_t)s.lights.size() - 1);
                } else {
                    s.tri_light.push_back(-1);
                }
            }
        }
    } catch (JsonError& e) {
        throw SceneError(AQUA_ERR_PARSE, path + ": " + e.what());
    }
    decode_textures(tc, allow_missing);
    if (!any_normals) s.nrm.clear();
    finalize_lights(s);
    return s;
}

void load_integrator_json(const std::string& path, aqua_integrator_cfg* cfg) {
    std::vector<uint8_t> raw = read_file(path, AQUA_ERR_IO);
    std::string text(raw.begin(), raw.end());
    try {
        Json j = json_parse(text);
        if (!j.is_object()) throw JsonError("integrator root must be an object");
        if (const Json* t = j.find("type")) {
            const std::string& ty = t->as_string();
            if (ty == "nrc") cfg->type = AQUA_INTEGRATOR_NRC;
            else if (ty == "pt" || ty == "path") cfg->type = AQUA_INTEGRATOR_PATH;
            else throw JsonError("unknown integrator type \"" + ty + "\"");
        }
        auto geti = [&](const char* k, int32_t& dst) {
            if (const Json* v = j.find(k)) {
                double d = v->as_number();
                if (d < 0 || d > 2147483647.0 || d != std::floor(d))
                    throw JsonError(std::string(k) + " must be a non-negative integer");
                dst = (int32_t)d;
            }
        };
        geti("spp", cfg->spp);
        geti("batch_size", cfg->batch_size);
        geti("max_depth", cfg->max_depth);
        geti("training_iters", cfg->training_iters);
        if (const Json* v = j.find("learning_rate")) {
            const double lr = v->as_number();
            if (!(lr > 0.0) || lr > 3.0e38) throw JsonError("learning_rate must be a positive number");
            cfg->learning_rate = (float)lr;
        }
        if (const Json* v = j.find("visualize_cache")) {
            if (v->kind != Json::Bool) throw JsonError("visualize_cache must be a boolean");
            cfg->visualize_cache = v->b ? 1 : 0;
        }
        if (const Json* v = j.find("seed")) {
            const double d = v->as_number();
            if (d < 0 || d >= 18446744073709551616.0 || d != std::floor(d))
                throw JsonError("seed must be a non-negative integer below 2^64");
            cfg->seed = (uint64_t)d;
        }
    } catch (JsonError& e) {
        throw SceneError(AQUA_ERR_PARSE, path + ": " + e.what());
    }
}

// ======================================================== procedural scenes
namespace {

struct Builder {
    HostScene& s;
    int add_material(v3 color, float metallic, float roughness, float specular, int tex = -1) {
        aqua_material m{};
        m.base_color[0] = color.x; m.base_color[1] = color.y; m.base_color[2] = color.z;
        m.base_texture = tex;
        m.metallic = metallic; m.roughness = roughness; m.specular = specular;
        m.sheen_tint = 0.5f; m.clearcoat_roughness = 0.03f; m.ior = 1.45f;  // defaults of the unused lobes
        s.mats.push_back(m);
        s.mat_names.push_back("m" + std::to_string(s.mats.size() - 1));
        return (int)s.mats.size() - 1;
    }
    void tri(v3 a, v3 b, v3 c, int mat, int light, const float* uv = nullptr) {
        push_tri(s, a, b, c, mat, uv);
        s.tri_light.push_back(light);
    }
    // Parallelogram p, p+u, p+u+v, p+v (two triangles); normal = u x v.
    void quad(v3 p, v3 u, v3 v, int mat, int light = -1, float us = 1.0f, float vs = 1.0f) {
        float uv0[6] = {0, 0, us, 0, us, vs};
        float uv1[6] = {0, 0, us, vs, 0, vs};
        tri(p, p + u, p + u + v, mat, light, uv0);
        tri(p, p + u + v, p + v, mat, light, uv1);
    }
    int quad_light(v3 p, v3 u, v3 v, v3 radiance, int mat) {
        aqua_light L{};
        L.type = AQUA_LIGHT_QUAD;
        for (int c = 0; c < 3; ++c) {
            L.p0[c] = comp(p, c); L.e1[c] = comp(u, c); L.e2[c] = comp(v, c);
            L.radiance[c] = comp(radiance, c);
        }
        s.lights.push_back(L);
        int id = (int)s.lights.size() - 1;
        quad(p, u, v, mat, id);
        s.num_meshes++;
        return id;
    }
    // Box of half-extents h, rotated about +y by (cos, sin), centred at c.
    void box(v3 c, v3 h, double cs, double sn, int mat) {
        auto X = [&](double x, double y, double z) {
            double rx = cs * x + sn * z, rz = -sn * x + cs * z;
            return mk((float)(c.x + rx), (float)(c.y + y), (float)(c.z + rz));
        };
        v3 P[8];
        for (int i = 0; i < 8; ++i)
            P[i] = X((i & 1) ? h.x : -h.x, (i & 2) ? h.y : -h.y, (i & 4) ? h.z : -h.z);
        // faces with outward normals (counter-clockwise seen from outside)
        const int F[6][4] = {{0, 4, 6, 2}, {1, 3, 7, 5}, {0, 1, 5, 4}, {2, 6, 7, 3}, {0, 2, 3, 1}, {4, 5, 7, 6}};
        for (auto& f : F) {
            float uv0[6] = {0, 0, 1, 0, 1, 1}, uv1[6] = {0, 0, 1, 1, 0, 1};
            tri(P[f[0]], P[f[1]], P[f[2]], mat, -1, uv0);
            tri(P[f[0]], P[f[2]], P[f[3]], mat, -1, uv1);
        }
        s.num_meshes++;
    }
    // UV sphere with `rings` latitude bands and `segs` longitude segments.
    void sphere(v3 c, float r, int rings, int segs, int mat, float uv_scale) {
        std::vector<v3> P((size_t)(rings + 1) * (size_t)(segs + 1));
        std::vector<float> U(P.size()), V(P.size());
        for (int i = 0; i <= rings; ++i) {
            double th = 3.14159265358979323846 * (double)i / rings;
            double st = det_sin(th), ct = det_cos(th);
            for (int j = 0; j <= segs; ++j) {
                double ph = kTwoPi * (double)j / segs;
                size_t k = (size_t)i * (size_t)(segs + 1) + (size_t)j;
                P[k] = mk((float)(c.x + r * st * det_cos(ph)), (float)(c.y + r * ct),
                          (float)(c.z + r * st * det_sin(ph)));
                U[k] = uv_scale * (float)j / (float)segs;
                V[k] = uv_scale * 0.5f * (float)i / (float)rings;
            }
        }
        auto id = [&](int i, int j) { return (size_t)i * (size_t)(segs + 1) + (size_t)j; };
        for (int i = 0; i < rings; ++i)
            for (int j = 0; j < segs; ++j) {
                size_t a = id(i, j), b = id(i + 1, j), cc = id(i + 1, j + 1), d = id(i, j + 1);
                if (i != 0) {
                    float uv[6] = {U[a], V[a], U[d], V[d], U[cc], V[cc]};
                    tri(P[a], P[d], P[cc], mat, -1, uv);
                }
                if (i != rings - 1) {
                    float uv[6] = {U[a], V[a], U[cc], V[cc], U[b], V[b]};
                    tri(P[a], P[cc], P[b], mat, -1, uv);
                }
            }
        s.num_meshes++;
    }
    // Grid of nu x nv cells over p + [0,1]u + [0,1]v, displaced along n by
    // amp * value_noise.
    void displaced_plane(v3 p, v3 u, v3 v, int nu, int nv, float amp, uint32_t nseed, int mat,
                         float uv_scale) {
        v3 n = normalize(cross(u, v));
        std::vector<v3> P((size_t)(nu + 1) * (size_t)(nv + 1));
        std::vector<float> U(P.size()), V(P.size());
        for (int i = 0; i <= nv; ++i)
            for (int j = 0; j <= nu; ++j) {
                float fu = (float)j / nu, fv = (float)i / nv;
                float h = amp > 0 ? amp * (value_noise(fu * 8.0f, fv * 8.0f, 8, nseed) * 2.0f - 1.0f) : 0.0f;
                size_t k = (size_t)i * (size_t)(nu + 1) + (size_t)j;
                P[k] = p + u * fu + v * fv + n * h;
                U[k] = fu * uv_scale;
                V[k] = fv * uv_scale;
            }
        auto id = [&](int i, int j) { return (size_t)i * (size_t)(nu + 1) + (size_t)j; };
        for (int i = 0; i < nv; ++i)
            for (int j = 0; j < nu; ++j) {
                size_t a = id(i, j), b = id(i, j + 1), cc = id(i + 1, j + 1), d = id(i + 1, j);
                float uv0[6] = {U[a], V[a], U[b], V[b], U[cc], V[cc]};
                float uv1[6] = {U[a], V[a], U[cc], V[cc], U[d], V[d]};
                tri(P[a], P[b], P[cc], mat, -1, uv0);
                tri(P[a], P[cc], P[d], mat, -1, uv1);
            }
        s.num_meshes++;
    }
    static uint32_t hash3(uint32_t x, uint32_t y, uint32_t z) {
        uint64_t h = splitmix64(((uint64_t)x << 32) ^ ((uint64_t)y << 11) ^ (uint64_t)z * 0x9E3779B97F4A7C15ULL);
        return (uint32_t)(h >> 32);
    }
    // Periodic value noise on a lattice of `period` cells, smoothstep blend.
    static float value_noise(float x, float y, int period, uint32_t seed) {
        float fx = std::floor(x), fy = std::floor(y);
        int ix = (int)fx, iy = (int)fy;
        float tx = x - fx, ty = y - fy;
        tx = tx * tx * (3.0f - 2.0f * tx);
        ty = ty * ty * (3.0f - 2.0f * ty);
        auto L = [&](int a, int b) {
            uint32_t pa = (uint32_t)(((a % period) + period) % period), pb = (uint32_t)(((b % period) + period) % period);
            return (float)(hash3(pa, pb, seed) >> 8) * (1.0f / 16777216.0f);
        };
        float v00 = L(ix, iy), v10 = L(ix + 1, iy), v01 = L(ix, iy + 1), v11 = L(ix + 1, iy + 1);
        float a = v00 + (v10 - v00) * tx, b = v01 + (v11 - v01) * tx;
        return a + (b - a) * ty;
    }
};

uint8_t enc_srgb(double lin) {
    double c = lin <= 0.0031308 ? 12.92 * lin : 1.055 * std::pow(lin, 1.0 / 2.4) - 0.055;
    int v = (int)(c * 255.0 + 0.5);
    return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
}

// 2048^2 RGBA8 textures: even = fractal value noise between two colours,
// odd = checker. Stored sRGB-encoded, decoded to linear at lookup.
Texture make_texture(int idx, int size, uint64_t seed) {
    Texture t;
    t.w = t.h = size;
    t.rgba.resize((size_t)size * size * 4);
    HostRng rng(seed ^ 0x7E47ULL, 1000 + (uint64_t)idx);
    v3 c0 = mk((float)rng.uniform(0.05, 0.9), (float)rng.uniform(0.05, 0.9), (float)rng.uniform(0.05, 0.9));
    v3 c1 = mk((float)rng.uniform(0.05, 0.9), (float)rng.uniform(0.05, 0.9), (float)rng.uniform(0.05, 0.9));
    int cells = 8 << rng.range(4);  // 8..64
    uint32_t nseed = rng.next();
    unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned w = 0; w < nth; ++w)
        th.emplace_back([&, w]() {
            for (int y = (int)w; y < size; y += (int)nth)
                for (int x = 0; x < size; ++x) {
                    float m;
                    if (idx % 2 == 0) {
                        float fx = (float)x / size, fy = (float)y / size, amp = 0.5f, sum = 0.0f, norm = 0.0f;
                        int per = 8;
                        for (int o = 0; o < 5; ++o) {
                            sum += amp * Builder::value_noise(fx * per, fy * per, per, nseed + (uint32_t)o);
                            norm += amp;
                            amp *= 0.5f;
                            per *= 2;
                        }
                        m = sum / norm;
                    } else {
                        int cx = x * cells / size, cy = y * cells / size;
                        m = ((cx + cy) & 1) ? 1.0f : 0.0f;
                    }
                    v3 c = lerp(c0, c1, m);
                    uint8_t* px = &t.rgba[((size_t)y * size + x) * 4];
                    px[0] = enc_srgb(c.x); px[1] = enc_srgb(c.y); px[2] = enc_srgb(c.z); px[3] = 255;
                }
        });
    for (auto& x : th) x.join();
    return t;
}

void cornell(HostScene& s, bool ggx, uint64_t seed) {
    Builder b{s};
    const v3 white = mk(0.725f, 0.71f, 0.68f), red = mk(0.63f, 0.065f, 0.05f), green = mk(0.14f, 0.45f, 0.09f);
    // Materials: floor, ceiling, back, left, right, short box, tall box, light.
    v3 cols[7] = {white, white, white, red, green, white, white};
    HostRng rng(seed, 0xC0B0ULL);
    int mats[7];
    for (int i = 0; i < 7; ++i) {
        if (ggx) {
            float rough = (float)rng.uniform(0.05, 0.8);
            float metal = rng.uniform() < 0.5 ? 0.0f : 1.0f;
            mats[i] = b.add_material(cols[i], metal, rough, 0.5f);
        } else {
            mats[i] = b.add_material(cols[i], 0.0f, 1.0f, 0.0f);  // Lambert: no specular lobe
        }
    }
    int light_mat = b.add_material(mk(0.78f, 0.78f, 0.78f), 0.0f, 1.0f, 0.0f);
    const char* names[8] = {"floor", "ceiling", "backWall", "leftWall", "rightWall", "shortBox", "tallBox", "light"};
    for (int i = 0; i < 8; ++i) s.mat_names[(size_t)i] = names[i];
    // Unit box x in [-0.5,0.5], y in [0,1], z in [-0.5,0.5], open towards +z.
    b.quad(mk(-0.5f, 0, 0.5f), mk(1, 0, 0), mk(0, 0, -1), mats[0]);            // floor, n=+y
    b.quad(mk(-0.5f, 1, -0.5f), mk(1, 0, 0), mk(0, 0, 1), mats[1]);            // ceiling, n=-y
    b.quad(mk(-0.5f, 0, -0.5f), mk(1, 0, 0), mk(0, 1, 0), mats[2]);            // back, n=+z
    b.quad(mk(-0.5f, 0, 0.5f), mk(0, 0, -1), mk(0, 1, 0), mats[3]);            // left, n=+x
    b.quad(mk(0.5f, 0, -0.5f), mk(0, 0, 1), mk(0, 1, 0), mats[4]);             // right, n=-x
    s.num_meshes += 5;
    // Rotations by the Pythagorean angle cos = 0.96, sin = 0.28 (16.26 deg).
    b.box(mk(0.165f, 0.15f, 0.19f), mk(0.15f, 0.15f, 0.15f), 0.96, -0.28, mats[5]);   // short, h 0.3
    b.box(mk(-0.17f, 0.3f, -0.145f), mk(0.15f, 0.3f, 0.15f), 0.96, 0.28, mats[6]);    // tall, h 0.6
    // Ceiling light 0.24 x 0.19 at y = 0.995, facing down, radiance (17,12,4).
    b.quad_light(mk(-0.12f, 0.995f, -0.095f), mk(0.24f, 0, 0), mk(0, 0, 0.19f), mk(17, 12, 4), light_mat);
    double t[3] = {0.0, 0.5, 4.5}, r[3] = {0, 0, 0};
    s.cam = make_camera(256, 256, 15.0f, 0.0f, 1.0f, t, r);
}

void interior(HostScene& s, uint64_t seed) {
    Builder b{s};
    HostRng rng(seed, 0x1A7E5ULL);
    const int ntex = 8;
    for (int i = 0; i < ntex; ++i) s.textures.push_back(make_texture(i, 2048, seed));
    // 32 surface materials: 8 textured, 24 plain.
    std::vector<int> mats;
    for (int i = 0; i < 32; ++i) {
        float rough = (float)rng.uniform(0.02, 1.0);
        if (i < ntex) {
            mats.push_back(b.add_material(mk(1, 1, 1), 0.0f, rough, 0.5f, i));
        } else {
            v3 c = mk((float)rng.uniform(0.05, 0.9), (float)rng.uniform(0.05, 0.9), (float)rng.uniform(0.05, 0.9));
            float metal = rng.uniform() < 0.25 ? 1.0f : 0.0f;
            mats.push_back(b.add_material(c, metal, rough, 0.5f));
        }
    }
    int wall_mat = b.add_material(mk(0.7f, 0.68f, 0.62f), 0.0f, 0.9f, 0.5f);
    int ceil_mat = b.add_material(mk(0.8f, 0.8f, 0.8f), 0.0f, 1.0f, 0.0f);
    int light_mat = b.add_material(mk(0.8f, 0.8f, 0.8f), 0.0f, 1.0f, 0.0f);
    // Room 20 x 4 x 14: floor, ceiling, four walls (6 meshes).
    const float X0 = -10, X1 = 10, Y1 = 4, Z0 = -7, Z1 = 7;
    b.displaced_plane(mk(X0, 0, Z1), mk(X1 - X0, 0, 0), mk(0, 0, Z0 - Z1), 192, 192, 0.015f, rng.next(), mats[0], 5.0f);
    b.displaced_plane(mk(X0, Y1, Z0), mk(X1 - X0, 0, 0), mk(0, 0, Z1 - Z0), 32, 32, 0.0f, 0, ceil_mat, 1.0f);
    b.displaced_plane(mk(X0, 0, Z0), mk(X1 - X0, 0, 0), mk(0, Y1, 0), 96, 32, 0.03f, rng.next(), wall_mat, 1.0f);
    b.displaced_plane(mk(X1, 0, Z1), mk(X0 - X1, 0, 0), mk(0, Y1, 0), 96, 32, 0.03f, rng.next(), wall_mat, 1.0f);
    b.displaced_plane(mk(X0, 0, Z1), mk(0, 0, Z0 - Z1), mk(0, Y1, 0), 96, 32, 0.03f, rng.next(), wall_mat, 1.0f);
    b.displaced_plane(mk(X1, 0, Z0), mk(0, 0, Z1 - Z0), mk(0, Y1, 0), 96, 32, 0.03f, rng.next(), mats[1], 3.0f);
    // 16 ceiling quad lights on a jittered 4 x 4 grid, radiance U[5,30].
    for (int i = 0; i < 16; ++i) {
        float w = (float)rng.log_uniform(0.6, 1.4), d = (float)rng.log_uniform(0.6, 1.4);
        float cx = X0 + (X1 - X0) * ((float)(i % 4) + 0.5f) / 4.0f + (float)rng.uniform(-1.0, 1.0);
        float cz = Z0 + (Z1 - Z0) * ((float)(i / 4) + 0.5f) / 4.0f + (float)rng.uniform(-0.8, 0.8);
        float L = (float)rng.uniform(5.0, 30.0);
        v3 tint = mk(1.0f, (float)rng.uniform(0.8, 1.0), (float)rng.uniform(0.6, 1.0));
        b.quad_light(mk(cx - w / 2, Y1 - 0.01f, cz - d / 2), mk(w, 0, 0), mk(0, 0, d), tint * L, light_mat);
    }
    // 131 objects: 56 instanced boxes, 55 tessellated spheres, 20 displaced planes.
    for (int i = 0; i < 56; ++i) {
        v3 h = mk((float)rng.log_uniform(0.1, 0.75), (float)rng.log_uniform(0.1, 0.75), (float)rng.log_uniform(0.1, 0.75));
        double ang = rng.uniform(0.0, kTwoPi);
        v3 c = mk((float)rng.uniform(X0 + 1, X1 - 1), h.y, (float)rng.uniform(Z0 + 1, Z1 - 1));
        b.box(c, h, det_cos(ang), det_sin(ang), mats[(size_t)rng.range(32)]);
    }
    for (int i = 0; i < 55; ++i) {
        float r = (float)rng.log_uniform(0.15, 0.9);
        bool floating = rng.uniform() < 0.3;
        float y = floating ? (float)rng.uniform(r + 0.5, Y1 - r - 0.3) : r;
        v3 c = mk((float)rng.uniform(X0 + 1, X1 - 1), y, (float)rng.uniform(Z0 + 1, Z1 - 1));
        b.sphere(c, r, 64, 128, mats[(size_t)rng.range(32)], 2.0f);
    }
    for (int i = 0; i < 20; ++i) {
        float sz = (float)rng.log_uniform(0.4, 2.5);
        double a1 = rng.uniform(0.0, kTwoPi), tilt = rng.uniform(-0.6, 0.6);
        v3 u = mk((float)(sz * det_cos(a1)), 0.0f, (float)(sz * det_sin(a1)));
        v3 v = mk((float)(-sz * det_sin(a1) * det_cos(tilt)), (float)(sz * det_sin(tilt)), (float)(sz * det_cos(a1) * det_cos(tilt)));
        v3 p = mk((float)rng.uniform(X0 + 1, X1 - 3), (float)rng.uniform(0.3, 2.5), (float)rng.uniform(Z0 + 1, Z1 - 3));
        b.displaced_plane(p, u, v, 64, 64, 0.05f * sz, rng.next(), mats[(size_t)rng.range(32)], 2.0f);
    }
    s.cam = aqua_camera{};
    s.cam.width = 1920; s.cam.height = 1080; s.cam.fov_deg = 65.0f; s.cam.focal = 1.0f;
    float eye[3] = {-8.5f, 1.7f, 5.5f}, tgt[3] = {3.0f, 1.0f, -3.0f}, up[3] = {0, 1, 0};
    camera_look_at(s.cam, eye, tgt, up);
}

void sphere_field(HostScene& s, uint64_t seed) {
    Builder b{s};
    HostRng rng(seed, 0x5F1E1DULL);
    std::vector<int> mats;
    for (int i = 0; i < 16; ++i) {
        v3 c = mk((float)rng.uniform(0.1, 0.9), (float)rng.uniform(0.1, 0.9), (float)rng.uniform(0.1, 0.9));
        mats.push_back(b.add_material(c, rng.uniform() < 0.3 ? 1.0f : 0.0f, (float)rng.uniform(0.05, 1.0), 0.5f));
    }
    int ground = b.add_material(mk(0.5f, 0.5f, 0.5f), 0.0f, 0.8f, 0.5f);
    int light_mat = b.add_material(mk(0, 0, 0), 0.0f, 1.0f, 0.0f);
    b.quad(mk(-60, 0, 60), mk(120, 0, 0), mk(0, 0, -120), ground);
    s.num_meshes++;
    for (int i = 0; i < 1008; ++i) {
        float r = (float)rng.log_uniform(0.2, 1.5);
        v3 c = mk((float)rng.uniform(-40, 40), r, (float)rng.uniform(-40, 40));
        b.sphere(c, r, 32, 64, mats[(size_t)rng.range(16)], 1.0f);
    }
    for (int i = 0; i < 4; ++i) {
        float cx = (i % 2) ? 15.0f : -15.0f, cz = (i / 2) ? 15.0f : -15.0f;
        b.quad_light(mk(cx - 4, 30, cz - 4), mk(8, 0, 0), mk(0, 0, 8), mk(12, 11, 10), light_mat);
    }
    s.env[0] = 0.10f; s.env[1] = 0.12f; s.env[2] = 0.16f;
    s.cam = aqua_camera{};
    s.cam.width = 512; s.cam.height = 512; s.cam.fov_deg = 50.0f; s.cam.focal = 1.0f;
    float eye[3] = {0.0f, 25.0f, 55.0f}, tgt[3] = {0.0f, 0.0f, 0.0f}, up[3] = {0, 1, 0};
    camera_look_at(s.cam, eye, tgt, up);
}

}  // namespace

HostScene make_procedural(int config_id, uint64_t seed, int width, int height) {
    HostScene s;
    switch (config_id) {
        case 1: cornell(s, false, seed); break;
        case 2: cornell(s, true, seed); s.cam.width = s.cam.height = 1024; break;
        case 3:
        case 4: interior(s, seed); break;
        case 5: sphere_field(s, seed); break;
        default: throw SceneError(AQUA_ERR_INVALID_ARG, "procedural config must be 1..5");
    }
    if (width > 0 && height > 0) { s.cam.width = width; s.cam.height = height; }
    finalize_lights(s);
    return s;
}

}  // namespace aq
