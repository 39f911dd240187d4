// obj.cpp — OBJ/MTL -> BSON meshes + scene JSON, and film writers.
//
// OBJ (Wavefront "Advanced Visualizer" appendix B1): v, vt, vn, f with
// v / v/vt / v//vn / v/vt/vn references (negative = relative), g / o start a
// mesh, usemtl switches material (a change inside a group starts another mesh
// of the same name), mtllib names the material libraries. Faces are fanned
// into triangles (0, i, i+1). Each mesh gets one vertex per distinct
// (position, texcoord, normal) reference in order of first use; without vn
// the vertex normal is the normalised sum of the unit normals of the faces
// that use it.
//
// MTL: newmtl, Kd (linear diffuse -> `Srgb` colour, so that decoding gives
// Kd back as in scenes/cbox.json:5 vs CornellBox-Original.mtl:37), Ke
// (emission), map_Kd (`Image` texture). Metallic and specular are 0 and
// roughness 0.4, as every converted material of scenes/cbox.json has.
#include "obj.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <tuple>
#include <vector>

#include <strings.h>

#include "scene.h"

namespace aq {
namespace {

struct Ref {
    int v, t, n;  // 0-based, -1 = absent
    bool operator<(const Ref& o) const { return std::tie(v, t, n) < std::tie(o.v, o.t, o.n); }
};

struct Group {
    std::string name, mtl;
    std::vector<std::array<Ref, 3>> tris;
};

struct Mtl {
    std::string name;
    double kd[3] = {0.8, 0.8, 0.8};
    double ke[3] = {0, 0, 0};
    std::string map_kd;  // path as written in the MTL
};

std::vector<std::string> tokens(const std::string& line) {
    std::vector<std::string> t;
    std::string cur;
    for (char c : line) {
        if (c == '#') break;
        if (c == ' ' || c == '\t' || c == '\r' || c == '\n') {
            if (!cur.empty()) t.push_back(cur), cur.clear();
        } else {
            cur.push_back(c);
        }
    }
    if (!cur.empty()) t.push_back(cur);
    return t;
}

double num(const std::string& s, const std::string& where) {
    char* end = nullptr;
    double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str() || *end || !std::isfinite(v))
        throw SceneError(AQUA_ERR_PARSE, where + ": bad number \"" + s + "\"");
    return v;
}

int ref_index(const std::string& s, size_t count, const std::string& where) {
    if (s.empty()) return -1;
    long i = std::strtol(s.c_str(), nullptr, 10);
    long r = i < 0 ? (long)count + i : i - 1;
    if (i == 0 || r < 0 || (size_t)r >= count) throw SceneError(AQUA_ERR_PARSE, where + ": index " + s + " out of range");
    return (int)r;
}

std::string dir_of(const std::string& p) {
    size_t s = p.find_last_of('/');
    return s == std::string::npos ? std::string(".") : p.substr(0, s);
}

std::string stem_of(const std::string& p) {
    size_t s = p.find_last_of('/');
    std::string f = s == std::string::npos ? p : p.substr(s + 1);
    size_t d = f.find_last_of('.');
    return d == std::string::npos ? f : f.substr(0, d);
}

std::string join_path(const std::string& dir, const std::string& f) {
    if (!f.empty() && f[0] == '/') return f;
    return dir + "/" + f;
}

std::vector<Mtl> parse_mtl(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw SceneError(AQUA_ERR_IO, "cannot open material library " + path);
    std::vector<Mtl> out;
    std::string line;
    int ln = 0;
    while (std::getline(in, line)) {
        ++ln;
        auto t = tokens(line);
        if (t.empty()) continue;
        std::string where = path + ":" + std::to_string(ln);
        if (t[0] == "newmtl") {
            out.push_back(Mtl{});
            out.back().name = t.size() > 1 ? t[1] : "";
        } else if (out.empty()) {
            continue;
        } else if ((t[0] == "Kd" || t[0] == "Ke") && t.size() >= 4) {
            double* d = t[0] == "Kd" ? out.back().kd : out.back().ke;
            for (int i = 0; i < 3; ++i) d[i] = num(t[(size_t)i + 1], where);
        } else if (t[0] == "map_Kd" && t.size() >= 2) {
            out.back().map_kd = t.back();  // options (-s, -o, ...) precede the file
            std::replace(out.back().map_kd.begin(), out.back().map_kd.end(), '\\', '/');
        }
    }
    return out;
}

// ---------------------------------------------------------------- BSON
struct BsonOut {
    std::vector<uint8_t> b;
    void u8(uint8_t x) { b.push_back(x); }
    void le(uint64_t x, int n) {
        for (int i = 0; i < n; ++i) b.push_back((uint8_t)(x >> (8 * i)));
    }
    void key(const std::string& k) {
        b.insert(b.end(), k.begin(), k.end());
        b.push_back(0);
    }
    size_t open() {
        size_t at = b.size();
        le(0, 4);
        return at;
    }
    void close(size_t at) {
        b.push_back(0);
        uint32_t n = (uint32_t)(b.size() - at);
        for (int i = 0; i < 4; ++i) b[at + (size_t)i] = (uint8_t)(n >> (8 * i));
    }
    void dbl(const std::string& k, double v) {
        uint64_t bits;
        memcpy(&bits, &v, 8);
        u8(0x01);
        key(k);
        le(bits, 8);
    }
    void i64(const std::string& k, int64_t v) {
        u8(0x12);
        key(k);
        le((uint64_t)v, 8);
    }
    void str(const std::string& k, const std::string& s) {
        u8(0x02);
        key(k);
        le((uint32_t)s.size() + 1, 4);
        b.insert(b.end(), s.begin(), s.end());
        b.push_back(0);
    }
    size_t array(const std::string& k) {
        u8(0x04);
        key(k);
        return open();
    }
};

void write_file(const std::string& path, const void* data, size_t n) {
    std::ofstream out(path, std::ios::binary);
    if (!out) throw SceneError(AQUA_ERR_IO, "cannot write " + path);
    out.write((const char*)data, (std::streamsize)n);
    if (!out) throw SceneError(AQUA_ERR_IO, "write failed: " + path);
}

std::string jstr(const std::string& s) {
    std::string o = "\"";
    for (char c : s) {
        if (c == '"' || c == '\\') o += '\\', o += c;
        else if ((unsigned char)c < 0x20) {
            char buf[8];
            snprintf(buf, sizeof buf, "\\u%04x", (unsigned)(unsigned char)c);
            o += buf;
        } else o += c;
    }
    return o + "\"";
}

std::string jnum(double v) {
    char buf[40];
    snprintf(buf, sizeof buf, "%.17g", v);
    return buf;
}

double linear_to_srgb(double c) {
    c = std::min(std::max(c, 0.0), 1.0);
    return c <= 0.0031308 ? 12.92 * c : 1.055 * std::pow(c, 1.0 / 2.4) - 0.055;
}

}  // namespace

ObjConvertResult convert_obj(const std::string& obj_path, const std::string& out_dir, const std::string& scene_name,
                             int width, int height) {
    std::ifstream in(obj_path);
    if (!in) throw SceneError(AQUA_ERR_IO, "cannot open " + obj_path);
    const std::string odir = dir_of(obj_path);
    std::vector<float> pos, tex, nrm;
    std::vector<Group> groups(1);
    groups[0].name = "default";
    std::vector<std::string> libs;
    std::string line, cur_mtl;
    int ln = 0;
    while (std::getline(in, line)) {
        ++ln;
        auto t = tokens(line);
        if (t.empty()) continue;
        const std::string where = obj_path + ":" + std::to_string(ln);
        const std::string& k = t[0];
        if (k == "v" && t.size() >= 4) {
            for (int i = 1; i <= 3; ++i) pos.push_back((float)num(t[(size_t)i], where));
        } else if (k == "vt" && t.size() >= 3) {
            for (int i = 1; i <= 2; ++i) tex.push_back((float)num(t[(size_t)i], where));
        } else if (k == "vn" && t.size() >= 4) {
            for (int i = 1; i <= 3; ++i) nrm.push_back((float)num(t[(size_t)i], where));
        } else if (k == "g" || k == "o") {
            std::string name;
            for (size_t i = 1; i < t.size(); ++i) name += (i > 1 ? " " : "") + t[i];
            if (name.empty()) name = "default";
            if (!groups.back().tris.empty()) groups.push_back(Group{});
            groups.back().name = name;
            groups.back().mtl = cur_mtl;
        } else if (k == "usemtl") {
            cur_mtl = t.size() > 1 ? t[1] : "";
            if (!groups.back().tris.empty() && groups.back().mtl != cur_mtl) {
                Group g;
                g.name = groups.back().name;
                groups.push_back(g);
            }
            groups.back().mtl = cur_mtl;
        } else if (k == "mtllib") {
            for (size_t i = 1; i < t.size(); ++i) libs.push_back(t[i]);
        } else if (k == "f") {
            if (t.size() < 4) throw SceneError(AQUA_ERR_PARSE, where + ": a face needs 3 vertices");
            std::vector<Ref> f;
            for (size_t i = 1; i < t.size(); ++i) {
                std::string a = t[i], b, c;
                size_t s1 = a.find('/');
                if (s1 != std::string::npos) {
                    b = a.substr(s1 + 1);
                    a = a.substr(0, s1);
                    size_t s2 = b.find('/');
                    if (s2 != std::string::npos) {
                        c = b.substr(s2 + 1);
                        b = b.substr(0, s2);
                    }
                }
                f.push_back(Ref{ref_index(a, pos.size() / 3, where), ref_index(b, tex.size() / 2, where),
                                ref_index(c, nrm.size() / 3, where)});
                if (f.back().v < 0) throw SceneError(AQUA_ERR_PARSE, where + ": face vertex without a position");
            }
            for (size_t i = 1; i + 1 < f.size(); ++i) groups.back().tris.push_back({f[0], f[i], f[i + 1]});
        }
    }
    std::vector<Mtl> mtls;
    for (const std::string& l : libs) {
        auto m = parse_mtl(join_path(odir, l));
        mtls.insert(mtls.end(), m.begin(), m.end());
    }
    auto find_mtl = [&](const std::string& n) -> const Mtl* {
        for (const Mtl& m : mtls)
            if (m.name == n) return &m;
        return nullptr;
    };

    ObjConvertResult res;
    const std::string stem = stem_of(obj_path);
    std::string shapes;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    std::vector<std::string> used;  // materials referenced, in first-use order
    int k = 0;
    for (const Group& g : groups) {
        if (g.tris.empty()) continue;
        std::map<Ref, int> index;
        std::vector<Ref> verts;
        std::vector<std::array<int, 3>> idx;
        for (const auto& tri : g.tris) {
            std::array<int, 3> o;
            for (int j = 0; j < 3; ++j) {
                auto it = index.find(tri[(size_t)j]);
                if (it == index.end()) {
                    it = index.emplace(tri[(size_t)j], (int)verts.size()).first;
                    verts.push_back(tri[(size_t)j]);
                }
                o[(size_t)j] = it->second;
            }
            idx.push_back(o);
        }
        const bool have_t = std::all_of(verts.begin(), verts.end(), [](const Ref& r) { return r.t >= 0; });
        const bool have_n = std::all_of(verts.begin(), verts.end(), [](const Ref& r) { return r.n >= 0; });
        std::vector<double> N(verts.size() * 3, 0.0);
        if (have_n) {
            for (size_t i = 0; i < verts.size(); ++i)
                for (int a = 0; a < 3; ++a) N[3 * i + (size_t)a] = nrm[3 * (size_t)verts[i].n + (size_t)a];
        } else {
            for (const auto& o : idx) {
                const float* p0 = &pos[3 * (size_t)verts[(size_t)o[0]].v];
                const float* p1 = &pos[3 * (size_t)verts[(size_t)o[1]].v];
                const float* p2 = &pos[3 * (size_t)verts[(size_t)o[2]].v];
                double e1[3], e2[3];
                for (int a = 0; a < 3; ++a) e1[a] = (double)p1[a] - p0[a], e2[a] = (double)p2[a] - p0[a];
                double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                               e1[0] * e2[1] - e1[1] * e2[0]};
                double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
                if (l == 0.0) continue;
                for (int j = 0; j < 3; ++j)
                    for (int a = 0; a < 3; ++a) N[3 * (size_t)o[(size_t)j] + (size_t)a] += c[a] / l;
            }
            for (size_t i = 0; i < verts.size(); ++i) {
                double* n = &N[3 * i];
                double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                if (l > 0.0)
                    for (int a = 0; a < 3; ++a) n[a] /= l;
            }
        }
        BsonOut b;
        size_t root = b.open();
        b.str("name", g.name);
        size_t av = b.array("vertices");
        for (size_t i = 0; i < verts.size(); ++i) {
            size_t e = b.array(std::to_string(i));
            for (int a = 0; a < 3; ++a) {
                double p = (double)pos[3 * (size_t)verts[i].v + (size_t)a];
                b.dbl(std::to_string(a), p);
                lo[a] = std::min(lo[a], p);
                hi[a] = std::max(hi[a], p);
            }
            b.close(e);
        }
        b.close(av);
        size_t an = b.array("normals");
        for (size_t i = 0; i < verts.size(); ++i) {
            size_t e = b.array(std::to_string(i));
            for (int a = 0; a < 3; ++a) b.dbl(std::to_string(a), N[3 * i + (size_t)a]);
            b.close(e);
        }
        b.close(an);
        size_t at = b.array("texcoords");
        if (have_t)
            for (size_t i = 0; i < verts.size(); ++i) {
                size_t e = b.array(std::to_string(i));
                for (int a = 0; a < 2; ++a) b.dbl(std::to_string(a), tex[2 * (size_t)verts[i].t + (size_t)a]);
                b.close(e);
            }
        b.close(at);
        size_t ai = b.array("indices");
        for (size_t i = 0; i < idx.size(); ++i) {
            size_t e = b.array(std::to_string(i));
            for (int a = 0; a < 3; ++a) b.i64(std::to_string(a), idx[i][(size_t)a]);
            b.close(e);
        }
        b.close(ai);
        b.close(root);
        const std::string file = stem + "_" + g.name + "_" + std::to_string(k) + ".mesh";
        write_file(out_dir + "/" + file, b.b.data(), b.b.size());
        std::string mname = g.mtl.empty() ? "default" : g.mtl;
        if (std::find(used.begin(), used.end(), mname) == used.end()) used.push_back(mname);
        shapes += std::string(shapes.empty() ? "" : ",\n") + "    {\"Mesh\": [" + jstr(file) +
                  ", {\"Named\": " + jstr(mname) + "}]}";
        res.triangles += (int)idx.size();
        ++k;
    }
    if (k == 0) throw SceneError(AQUA_ERR_PARSE, obj_path + ": no faces");
    res.meshes = k;

    std::string bsdfs;
    for (const std::string& n : used) {
        const Mtl* m = find_mtl(n);
        Mtl dflt;
        if (!m) m = &dflt;
        std::string color;
        if (!m->map_kd.empty()) {
            std::string tex_path = join_path(odir, m->map_kd);
            if (dir_of(obj_path) != out_dir && tex_path[0] != '/') {
                char buf[4096];
                if (realpath(tex_path.c_str(), buf)) tex_path = buf;
            } else if (tex_path.rfind(odir + "/", 0) == 0) {
                tex_path = tex_path.substr(odir.size() + 1);
            }
            color = "{\"Image\": " + jstr(tex_path) + "}";
        } else {
            color = "{\"Srgb\": [" + jnum(linear_to_srgb(m->kd[0])) + ", " + jnum(linear_to_srgb(m->kd[1])) + ", " +
                    jnum(linear_to_srgb(m->kd[2])) + "]}";
        }
        std::string emission = (m->ke[0] > 0 || m->ke[1] > 0 || m->ke[2] > 0)
                                   ? "{\"Float3\": [" + jnum(m->ke[0]) + ", " + jnum(m->ke[1]) + ", " + jnum(m->ke[2]) + "]}"
                                   : "{\"Float\": 0.0}";
        bsdfs += std::string(bsdfs.empty() ? "" : ",\n") + "    " + jstr(n) + ": {\"Principled\": {\"color\": " + color +
                 ", \"metallic\": {\"Float\": 0.0}, \"specular\": {\"Float\": 0.0}, \"roughness\": {\"Float\": 0.4}"
                 ", \"emission\": " + emission + "}}";
    }
    res.materials = (int)used.size();
    // Camera on +z of the bounding box, looking down -z, 40 degrees vertical.
    double c[3], ext = 0.0;
    for (int a = 0; a < 3; ++a) c[a] = 0.5 * (lo[a] + hi[a]), ext = std::max(ext, hi[a] - lo[a]);
    const double dist = 0.5 * ext / std::tan(20.0 * 3.14159265358979323846 / 180.0) * 1.1 + 0.5 * (hi[2] - lo[2]);
    std::string json = "{\n  \"named_bsdfs\": {\n" + bsdfs + "\n  },\n  \"camera\": {\"Perspective\": {\"res\": [" +
                       std::to_string(width) + ", " + std::to_string(height) +
                       "], \"fov\": 40.0, \"lens_radius\": 0.0, \"focal\": 1.0, \"transform\": {\"translate\": [" +
                       jnum(c[0]) + ", " + jnum(c[1]) + ", " + jnum(c[2] + dist) +
                       "], \"rotate\": [0.0, 0.0, 0.0], \"scale\": [1.0, 1.0, 1.0]}}},\n  \"lights\": [],\n"
                       "  \"shapes\": [\n" + shapes + "\n  ]\n}\n";
    write_file(out_dir + "/" + scene_name, json.data(), json.size());
    return res;
}

void write_image(const std::string& path, const float* rgb, int w, int h) {
    auto ends = [&](const char* s) {
        size_t n = strlen(s);
        return path.size() >= n && strcasecmp(path.c_str() + path.size() - n, s) == 0;
    };
    std::string out;
    if (ends(".pfm")) {
        out = "PF\n" + std::to_string(w) + " " + std::to_string(h) + "\n-1.0\n";
        size_t hdr = out.size();
        out.resize(hdr + (size_t)w * (size_t)h * 12);
        uint8_t* p = (uint8_t*)&out[hdr];
        for (int y = h - 1; y >= 0; --y)
            for (size_t i = 0; i < (size_t)w * 3; ++i) {
                uint32_t bits;
                memcpy(&bits, &rgb[(size_t)y * (size_t)w * 3 + i], 4);
                for (int b = 0; b < 4; ++b) *p++ = (uint8_t)(bits >> (8 * b));  // little-endian
            }
    } else if (ends(".ppm")) {
        out = "P6\n" + std::to_string(w) + " " + std::to_string(h) + "\n255\n";
        for (size_t i = 0; i < (size_t)w * (size_t)h * 3; ++i)
            out.push_back((char)(uint8_t)std::lround(linear_to_srgb((double)rgb[i]) * 255.0));
    } else {
        throw SceneError(AQUA_ERR_INVALID_ARG, "image path must end in .pfm or .ppm: " + path);
    }
    write_file(path, out.data(), out.size());
}

}  // namespace aq
