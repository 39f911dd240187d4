// capi.cpp — the C ABI (include/aqua.h): handle lifetime, status codes and
// error text, scene upload, and dispatch into the CUDA translation units.
// No C++ exception crosses this boundary.
#include <algorithm>
#include <memory>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>

#include "internal.h"
#include "jpeg.h"
#include "obj.h"
#include "nrc.h"

namespace {
thread_local std::string g_create_error;
}

namespace aq {

void dev_alloc(aqua_ctx* ctx, DevBuf& b, size_t bytes) {
    ++ctx->alloc_count;
    if (ctx->fail_alloc_after && ctx->alloc_count >= ctx->fail_alloc_after)
        throw Error(AQUA_ERR_OOM, "device allocation of " + std::to_string(bytes) +
                                      " bytes refused by the fail_alloc_after test hook");
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 256));
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(e == cudaErrorMemoryAllocation ? AQUA_ERR_OOM : AQUA_ERR_CUDA,
                    "cudaMalloc(" + std::to_string(bytes) + "): " + cudaGetErrorString(e));
    }
    b.ptr = p;
    b.bytes = bytes;
}

void dev_free(DevBuf& b) {
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

DevCamera dev_camera(const aqua_camera& c) {
    DevCamera d{};
    for (int i = 0; i < 3; ++i) {
        d.pos[i] = c.pos[i];
        d.right[i] = c.right[i];
        d.up[i] = c.up[i];
        d.back[i] = c.back[i];
    }
    d.tan_half = (float)std::tan(0.5 * (double)c.fov_deg * 3.14159265358979323846 / 180.0);
    d.aspect = (float)c.width / (float)c.height;
    d.lens_radius = c.lens_radius;
    d.focal = c.focal;
    d.width = c.width;
    d.height = c.height;
    return d;
}

static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

static void free_staging(aqua_scene* s) {
    if (s->pinned) {
        if (s->pinned_is_cuda) cudaFreeHost(s->pinned);
        else free(s->pinned);
    }
    s->pinned = nullptr;
}

void scene_release(aqua_scene* s) {
    dev_free(s->dev);
    free_staging(s);
}

// Device image: nodes | triangle words | uvs | materials | lights | textures | texels.
void scene_build_device(aqua_ctx* ctx, aqua_scene* s, bool rebuild_bvh) {
    const HostScene& h = s->host;
    size_t nt = h.num_tris();
    if (h.mats.size() > 65535) throw Error(AQUA_ERR_UNSUPPORTED, "more than 65535 materials");
    if (h.lights.size() > 65534) throw Error(AQUA_ERR_UNSUPPORTED, "more than 65534 lights");
    if (nt >= (1u << 28)) throw Error(AQUA_ERR_UNSUPPORTED, "more than 2^28 triangles");
    if (rebuild_bvh || s->bvh.nodes.empty()) {
        s->bvh = build_bvh(h.verts.data(), nt);
        if (s->bvh.max_stack >= kBvhStackSize)
            throw Error(AQUA_ERR_UNSUPPORTED, "BVH deeper than the traversal stack");
        s->qnodes = quantize_bvh(s->bvh);
    }
    size_t nn = (size_t)s->bvh.num_nodes();
    // Quantized nodes when asked, or (automatic) for trees whose
    // full-precision nodes exceed kQuantizeAbove: half the node bytes, a
    // few more instructions per visit.
    const bool use_q = s->bvh_format == AQUA_BVH_QUANTIZED ||
                       (s->bvh_format == AQUA_BVH_AUTO && nn * sizeof(float) * kBvhNodeFloats > kQuantizeAbove);
    const size_t node_floats = use_q ? kBvhQNodeFloats : kBvhNodeFloats;
    size_t texels = 0;
    for (auto& t : h.textures) texels += (size_t)t.w * (size_t)t.h;
    size_t o_nodes = 0, o_tris = align256(o_nodes + sizeof(float) * node_floats * nn), o_uvs = align256(o_tris + 48 * nt),
           o_mats = align256(o_uvs + 24 * nt), o_lights = align256(o_mats + 32 * h.mats.size()),
           o_texs = align256(o_lights + 64 * h.lights.size()),
           o_texels = align256(o_texs + 16 * h.textures.size()), o_nrm = align256(o_texels + 4 * texels),
           o_mext = align256(o_nrm + (h.nrm.empty() ? 0 : 48 * nt));
    bool full_bsdf = false;
    for (const aqua_material& m : h.mats)
        if (m.specular_tint > 0.0f || m.sheen > 0.0f || m.clearcoat > 0.0f || m.transmission > 0.0f) full_bsdf = true;
    size_t total = align256(o_mext + (full_bsdf ? 32 * h.mats.size() : 0));
    free_staging(s);
    if (ctx->host_only) {
        s->pinned = malloc(total);
        if (!s->pinned) throw std::bad_alloc();
        s->pinned_is_cuda = false;
    } else {
        AQ_CUDA(cudaHostAlloc(&s->pinned, total, cudaHostAllocDefault));
        s->pinned_is_cuda = true;
    }
    char* p = (char*)s->pinned;
    memset(p, 0, total);
    memcpy(p + o_nodes, use_q ? s->qnodes.data() : s->bvh.nodes.data(), sizeof(float) * node_floats * nn);
    float* tw = (float*)(p + o_tris);
    float* uw = (float*)(p + o_uvs);
    float* nw = h.nrm.empty() ? nullptr : (float*)(p + o_nrm);
    for (size_t k = 0; k < nt; ++k) {
        int32_t i = s->bvh.tri_order[k];
        if (nw)
            for (int c = 0; c < 3; ++c)
                for (int a = 0; a < 3; ++a) nw[12 * k + 4 * (size_t)c + (size_t)a] = h.nrm[9 * (size_t)i + 3 * (size_t)c + (size_t)a];
        const float* v = &h.verts[9 * (size_t)i];
        uint32_t info = (uint32_t)h.tri_mat[(size_t)i] | ((uint32_t)(h.tri_light[(size_t)i] + 1) << 16);
        float* o = tw + 12 * k;
        o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; memcpy(&o[3], &i, 4);
        o[4] = v[3]; o[5] = v[4]; o[6] = v[5]; memcpy(&o[7], &info, 4);
        o[8] = v[6]; o[9] = v[7]; o[10] = v[8]; o[11] = 0.0f;
        memcpy(uw + 6 * k, &h.uvs[6 * (size_t)i], 24);
    }
    DevMaterial* mw = (DevMaterial*)(p + o_mats);
    for (size_t i = 0; i < h.mats.size(); ++i) {
        const aqua_material& m = h.mats[i];
        int32_t tex = m.base_texture;
        if (tex >= (int32_t)h.textures.size()) throw Error(AQUA_ERR_INVALID_ARG, "material refers to a missing texture");
        float tf;
        memcpy(&tf, &tex, 4);
        mw[i].a = make_float4(m.base_color[0], m.base_color[1], m.base_color[2], tf);
        mw[i].b = make_float4(m.metallic, m.roughness, m.specular, 0.0f);
    }
    if (full_bsdf) {
        float4* xw = (float4*)(p + o_mext);
        for (size_t i = 0; i < h.mats.size(); ++i) {
            const aqua_material& m = h.mats[i];
            xw[2 * i] = make_float4(m.specular_tint, m.sheen, m.sheen_tint, m.clearcoat);
            xw[2 * i + 1] = make_float4(m.clearcoat_roughness, m.transmission, m.ior, 0.0f);
        }
    }
    DevLight* lw = (DevLight*)(p + o_lights);
    double cdf = 0.0;
    for (size_t i = 0; i < h.lights.size(); ++i) {
        const aqua_light& l = h.lights[i];
        float tyf;
        memcpy(&tyf, &l.type, 4);
        v3 e1 = mk(l.e1[0], l.e1[1], l.e1[2]), e2 = mk(l.e2[0], l.e2[1], l.e2[2]);
        float area = length(cross(e1, e2)) * (l.type == AQUA_LIGHT_TRIANGLE ? 0.5f : 1.0f);
        cdf += l.pmf;
        float c = i + 1 == h.lights.size() ? 1.0f : (float)cdf;
        lw[i].p0 = make_float4(l.p0[0], l.p0[1], l.p0[2], tyf);
        lw[i].e1 = make_float4(l.e1[0], l.e1[1], l.e1[2], area);
        lw[i].e2 = make_float4(l.e2[0], l.e2[1], l.e2[2], l.pmf);
        lw[i].le = make_float4(l.radiance[0], l.radiance[1], l.radiance[2], c);
    }
    DevTexture* xw = (DevTexture*)(p + o_texs);
    uint32_t off = 0;
    for (size_t i = 0; i < h.textures.size(); ++i) {
        xw[i].offset = off;
        xw[i].w = h.textures[i].w;
        xw[i].h = h.textures[i].h;
        xw[i].pad = 0;
        memcpy(p + o_texels + 4 * (size_t)off, h.textures[i].rgba.data(), h.textures[i].rgba.size());
        off += (uint32_t)(h.textures[i].w * h.textures[i].h);
    }
    s->bytes = total;
    s->bvh_format_used = use_q ? AQUA_BVH_QUANTIZED : AQUA_BVH_FULL;
    if (ctx->host_only) return;  // host-only context: no device image
    dev_free(s->dev);
    dev_alloc(ctx, s->dev, total);
    char* d = (char*)s->dev.ptr;
    DevScene& ds = s->ds;
    ds.nodes = (const float4*)(d + o_nodes);
    ds.qbvh = use_q ? 1 : 0;
    ds.tris = (const float4*)(d + o_tris);
    ds.uvs = (const float2*)(d + o_uvs);
    ds.mats = (const DevMaterial*)(d + o_mats);
    ds.lights = (const DevLight*)(d + o_lights);
    ds.texs = (const DevTexture*)(d + o_texs);
    ds.texels = (const uint32_t*)(d + o_texels);
    ds.nrm = h.nrm.empty() ? nullptr : (const float4*)(d + o_nrm);
    ds.mext = full_bsdf ? (const float4*)(d + o_mext) : nullptr;
    ds.n_nodes = (int32_t)nn;
    ds.n_tris = (int32_t)nt;
    ds.n_mats = (int32_t)h.mats.size();
    ds.n_lights = (int32_t)h.lights.size();
    ds.n_texs = (int32_t)h.textures.size();
    for (int i = 0; i < 3; ++i) ds.env[i] = h.env[i];
    ds.cam = dev_camera(h.cam);
    scene_upload(ctx, s);
}

void scene_upload(aqua_ctx* ctx, aqua_scene* s) {
    if (ctx->host_only) throw Error(AQUA_ERR_UNSUPPORTED, "host-only context has no device");
    AQ_CUDA(cudaMemcpyAsync(s->dev.ptr, s->pinned, s->bytes, cudaMemcpyHostToDevice, ctx->stream));
    AQ_CUDA(cudaStreamSynchronize(ctx->stream));
    s->uploaded = true;
}

}  // namespace aq

using namespace aq;

// ---------------------------------------------------------------- ABI helpers
// Error text as aqua_last_error hands it out: messages quote parts of the
// input (a malformed OBJ line, a file name), so bytes that are neither
// printable ASCII nor part of a well-formed UTF-8 sequence are written as
// \xNN, and the text is cut at 1024 bytes. Callers can decode it as UTF-8.
static std::string clean_message(const char* m) {
    std::string out;
    const unsigned char* p = reinterpret_cast<const unsigned char*>(m);
    const size_t n = strlen(m);
    auto cont = [&](size_t i, unsigned lo, unsigned hi) { return i < n && p[i] >= lo && p[i] <= hi; };
    size_t i = 0;
    while (i < n && out.size() < 1024) {
        const unsigned c = p[i];
        size_t len = 0;
        if (c >= 0x20 && c < 0x7f) len = 1;
        else if (c >= 0xc2 && c <= 0xdf) len = cont(i + 1, 0x80, 0xbf) ? 2 : 0;
        else if (c >= 0xe0 && c <= 0xef) {
            const unsigned lo = c == 0xe0 ? 0xa0 : 0x80, hi = c == 0xed ? 0x9f : 0xbf;
            len = cont(i + 1, lo, hi) && cont(i + 2, 0x80, 0xbf) ? 3 : 0;
        } else if (c >= 0xf0 && c <= 0xf4) {
            const unsigned lo = c == 0xf0 ? 0x90 : 0x80, hi = c == 0xf4 ? 0x8f : 0xbf;
            len = cont(i + 1, lo, hi) && cont(i + 2, 0x80, 0xbf) && cont(i + 3, 0x80, 0xbf) ? 4 : 0;
        }
        if (len) {
            out.append(m + i, len);
            i += len;
        } else {
            static const char* hex = "0123456789abcdef";
            out += "\\x";
            out += hex[c >> 4];
            out += hex[c & 15];
            ++i;
        }
    }
    return out;
}

template <class F>
static aqua_status guard(aqua_ctx* ctx, F&& f) {
    if (!ctx) return AQUA_ERR_INVALID_ARG;
    ctx->err.clear();
    try {
        if (!ctx->host_only && cudaSetDevice(ctx->device) != cudaSuccess)
            throw Error(AQUA_ERR_CUDA, "cudaSetDevice failed");
        f();
        return AQUA_OK;
    } catch (Error& e) {
        ctx->err = clean_message(e.what());
        return e.status;
    } catch (SceneError& e) {
        ctx->err = clean_message(e.what());
        return e.status;
    } catch (std::bad_alloc&) {
        ctx->err = "host allocation failed";
        return AQUA_ERR_OOM;
    } catch (std::exception& e) {
        ctx->err = clean_message(e.what());
        return AQUA_ERR_INVALID_ARG;
    }
}

static void need(bool c, const char* msg) {
    if (!c) throw Error(AQUA_ERR_INVALID_ARG, msg);
}

static void need_device(aqua_ctx* ctx) {
    if (ctx->host_only) throw Error(AQUA_ERR_UNSUPPORTED, "this call needs a CUDA device; the context is host-only");
}

extern "C" {

AQUA_API int aqua_version(void) { return AQUA_VERSION; }

AQUA_API const char* aqua_status_string(aqua_status s) {
    switch (s) {
        case AQUA_OK: return "ok";
        case AQUA_ERR_INVALID_ARG: return "invalid argument";
        case AQUA_ERR_IO: return "i/o error";
        case AQUA_ERR_PARSE: return "parse error";
        case AQUA_ERR_MISSING_ASSET: return "missing asset";
        case AQUA_ERR_CUDA: return "cuda error";
        case AQUA_ERR_OOM: return "out of memory";
        case AQUA_ERR_TIMEOUT: return "timeout";
        case AQUA_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

AQUA_API const char* aqua_last_error(const aqua_ctx* ctx) {
    if (!ctx) return g_create_error.c_str();
    return ctx->err.c_str();
}

AQUA_API aqua_status aqua_create(aqua_ctx** out, const aqua_options* opt) {
    g_create_error.clear();
    if (!out) { g_create_error = "out is NULL"; return AQUA_ERR_INVALID_ARG; }
    *out = nullptr;
    aqua_ctx* ctx = new (std::nothrow) aqua_ctx();
    if (!ctx) { g_create_error = "host allocation failed"; return AQUA_ERR_OOM; }
    int dev = opt ? opt->device : -1;
    if (dev == AQUA_DEVICE_HOST_ONLY) {
        ctx->host_only = true;
        ctx->device = -1;
        ctx->verbose = opt->verbose;
        *out = ctx;
        return AQUA_OK;
    }
    if (dev < 0) {
        if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    }
    cudaError_t e = cudaSetDevice(dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&ctx->pinned_counter, 64, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        g_create_error = std::string("CUDA initialisation failed: ") + cudaGetErrorString(e);
        cudaGetLastError();
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return AQUA_ERR_CUDA;
    }
    ctx->device = dev;
    ctx->verbose = opt ? opt->verbose : 0;
    ctx->fail_alloc_after = opt ? opt->fail_alloc_after : 0;
    *out = ctx;
    return AQUA_OK;
}

AQUA_API void aqua_destroy(aqua_ctx* ctx) {
    if (!ctx) return;
    if (ctx->host_only) {
        delete ctx;
        return;
    }
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    workspace_release(ctx);
    batch_release(ctx);
    dev_free(ctx->nrc_ws.block);
    dev_free(ctx->trace_rays);
    dev_free(ctx->trace_hits);
    dev_free(ctx->persist_film);
    dev_free(ctx->trace_stats);
    for (auto e : ctx->events) cudaEventDestroy(e);
    if (ctx->pinned_counter) cudaFreeHost(ctx->pinned_counter);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

AQUA_API aqua_status aqua_load_scene_json(aqua_ctx* ctx, const char* path, int32_t allow_missing,
                                          aqua_scene** out) {
    return guard(ctx, [&]() {
        need(path && out, "path and out must be non-NULL");
        *out = nullptr;
        aqua_scene* s = new aqua_scene();
        try {
            s->host = load_scene_json(path, allow_missing != 0);
            scene_build_device(ctx, s);
        } catch (...) {
            scene_release(s);
            delete s;
            throw;
        }
        *out = s;
    });
}

AQUA_API aqua_status aqua_make_procedural_scene(aqua_ctx* ctx, int32_t config_id, uint64_t seed, int32_t width,
                                                int32_t height, aqua_scene** out) {
    return guard(ctx, [&]() {
        need(out != nullptr, "out must be non-NULL");
        *out = nullptr;
        need(width <= 16384 && height <= 16384, "resolution above 16384");
        aqua_scene* s = new aqua_scene();
        try {
            s->host = make_procedural(config_id, seed, width, height);
            scene_build_device(ctx, s);
        } catch (...) {
            scene_release(s);
            delete s;
            throw;
        }
        *out = s;
    });
}

AQUA_API aqua_status aqua_scene_free(aqua_ctx* ctx, aqua_scene* scene) {
    return guard(ctx, [&]() {
        if (!scene) return;
        if (!ctx->host_only) cudaStreamSynchronize(ctx->stream);
        scene_release(scene);
        delete scene;
    });
}

AQUA_API aqua_status aqua_scene_set_resolution(aqua_ctx* ctx, aqua_scene* s, int32_t width, int32_t height) {
    return guard(ctx, [&]() {
        need(s != nullptr, "scene is NULL");
        need(width > 0 && height > 0 && width <= 16384 && height <= 16384, "resolution out of range");
        s->host.cam.width = width;
        s->host.cam.height = height;
        s->ds.cam = dev_camera(s->host.cam);
    });
}

AQUA_API aqua_status aqua_scene_upload(aqua_ctx* ctx, aqua_scene* s) {
    return guard(ctx, [&]() {
        need(s != nullptr, "scene is NULL");
        scene_upload(ctx, s);
    });
}

AQUA_API aqua_status aqua_scene_get_info(aqua_ctx* ctx, const aqua_scene* s, aqua_scene_info* out) {
    return guard(ctx, [&]() {
        need(s && out, "scene and out must be non-NULL");
        memset(out, 0, sizeof(*out));
        out->width = s->host.cam.width;
        out->height = s->host.cam.height;
        out->num_triangles = (int32_t)s->host.num_tris();
        out->num_materials = (int32_t)s->host.mats.size();
        out->num_lights = (int32_t)s->host.lights.size();
        out->num_textures = (int32_t)s->host.textures.size();
        out->num_meshes = s->host.num_meshes;
        out->num_bvh_nodes = s->bvh.num_nodes();
        out->bvh_depth = s->bvh.depth;
        out->max_leaf_size = s->bvh.max_leaf;
        out->device_bytes = s->dev.bytes;
        out->upload_bytes = s->bytes;
        for (int i = 0; i < 3; ++i) out->env[i] = s->host.env[i];
        out->bvh_format = s->bvh_format_used;
    });
}

AQUA_API aqua_status aqua_scene_export_triangles(aqua_ctx* ctx, const aqua_scene* s, float* verts, float* uvs,
                                                 int32_t* mat, int32_t* light) {
    return guard(ctx, [&]() {
        need(s != nullptr, "scene is NULL");
        size_t n = s->host.num_tris();
        if (verts) memcpy(verts, s->host.verts.data(), 36 * n);
        if (uvs) memcpy(uvs, s->host.uvs.data(), 24 * n);
        if (mat) memcpy(mat, s->host.tri_mat.data(), 4 * n);
        if (light) memcpy(light, s->host.tri_light.data(), 4 * n);
    });
}

AQUA_API aqua_status aqua_scene_export_camera(aqua_ctx* ctx, const aqua_scene* s, aqua_camera* out) {
    return guard(ctx, [&]() {
        need(s && out, "scene and out must be non-NULL");
        *out = s->host.cam;
    });
}

AQUA_API aqua_status aqua_scene_export_materials(aqua_ctx* ctx, const aqua_scene* s, aqua_material* out) {
    return guard(ctx, [&]() {
        need(s && out, "scene and out must be non-NULL");
        if (!s->host.mats.empty()) memcpy(out, s->host.mats.data(), sizeof(aqua_material) * s->host.mats.size());
    });
}

AQUA_API aqua_status aqua_scene_export_lights(aqua_ctx* ctx, const aqua_scene* s, aqua_light* out) {
    return guard(ctx, [&]() {
        need(s && out, "scene and out must be non-NULL");
        if (!s->host.lights.empty())
            memcpy(out, s->host.lights.data(), sizeof(aqua_light) * s->host.lights.size());
    });
}

AQUA_API aqua_status aqua_scene_export_texture(aqua_ctx* ctx, const aqua_scene* s, int32_t i, int32_t* w,
                                               int32_t* h, uint8_t* rgba) {
    return guard(ctx, [&]() {
        need(s != nullptr, "scene is NULL");
        need(i >= 0 && (size_t)i < s->host.textures.size(), "texture index out of range");
        const Texture& t = s->host.textures[(size_t)i];
        if (w) *w = t.w;
        if (h) *h = t.h;
        if (rgba) memcpy(rgba, t.rgba.data(), t.rgba.size());
    });
}

AQUA_API aqua_status aqua_decode_jpeg(aqua_ctx* ctx, const uint8_t* data, size_t n, int32_t* w, int32_t* h,
                                      uint8_t* rgb) {
    return guard(ctx, [&]() {
        need(data != nullptr || n == 0, "data is NULL");
        JpegImage img;
        std::string err = jpeg_decode(data, n, img);
        if (!err.empty()) throw Error(AQUA_ERR_UNSUPPORTED, "JPEG: " + err);
        if (w) *w = img.w;
        if (h) *h = img.h;
        if (rgb) memcpy(rgb, img.rgb.data(), img.rgb.size());
    });
}

AQUA_API aqua_status aqua_convert_obj(aqua_ctx* ctx, const char* obj_path, const char* out_dir,
                                      const char* scene_name, int32_t width, int32_t height, int32_t* meshes,
                                      int32_t* triangles) {
    return guard(ctx, [&]() {
        need(obj_path && out_dir && scene_name, "obj_path, out_dir and scene_name must be non-NULL");
        need(width > 0 && height > 0, "width and height must be positive");
        ObjConvertResult r = convert_obj(obj_path, out_dir, scene_name, width, height);
        if (meshes) *meshes = r.meshes;
        if (triangles) *triangles = r.triangles;
    });
}

AQUA_API aqua_status aqua_write_image(aqua_ctx* ctx, const char* path, const float* rgb, int32_t width,
                                      int32_t height) {
    return guard(ctx, [&]() {
        need(path && rgb, "path and rgb must be non-NULL");
        need(width > 0 && height > 0, "width and height must be positive");
        write_image(path, rgb, width, height);
    });
}

AQUA_API aqua_status aqua_scene_export_normals(aqua_ctx* ctx, const aqua_scene* s, float* nrm, int32_t* present) {
    return guard(ctx, [&]() {
        need(s != nullptr, "scene is NULL");
        if (present) *present = s->host.nrm.empty() ? 0 : 1;
        if (nrm && !s->host.nrm.empty()) memcpy(nrm, s->host.nrm.data(), 4 * s->host.nrm.size());
    });
}

AQUA_API aqua_status aqua_scene_export_bvh_quantized(aqua_ctx* ctx, const aqua_scene* s, float* nodes) {
    return guard(ctx, [&]() {
        need(s != nullptr, "scene is NULL");
        if (nodes) memcpy(nodes, s->qnodes.data(), 4 * s->qnodes.size());
    });
}

AQUA_API aqua_status aqua_scene_set_bvh_format(aqua_ctx* ctx, aqua_scene* s, int32_t format) {
    return guard(ctx, [&]() {
        need(s != nullptr, "scene is NULL");
        need(format == AQUA_BVH_AUTO || format == AQUA_BVH_FULL || format == AQUA_BVH_QUANTIZED,
             "format must be an AQUA_BVH_* value");
        s->bvh_format = format;
        scene_build_device(ctx, s, false);
    });
}

AQUA_API aqua_status aqua_scene_export_bvh(aqua_ctx* ctx, const aqua_scene* s, float* nodes, int32_t* tri_order) {
    return guard(ctx, [&]() {
        need(s != nullptr, "scene is NULL");
        if (nodes) memcpy(nodes, s->bvh.nodes.data(), 4 * s->bvh.nodes.size());
        if (tri_order) memcpy(tri_order, s->bvh.tri_order.data(), 4 * s->bvh.tri_order.size());
    });
}

AQUA_API void aqua_integrator_defaults(aqua_integrator_cfg* c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->type = AQUA_INTEGRATOR_PATH;
    c->spp = 4;             // scenes/integrator.json:3
    c->max_depth = 5;       // scenes/integrator.json:5
    c->rr_depth = 3;
    c->batch_size = 512;    // scenes/integrator.json:4
    c->training_iters = 2048;  // scenes/integrator.json:6
    c->learning_rate = 1e-3f;  // scenes/integrator.json:7
    c->visualize_cache = 0;    // scenes/integrator.json:8
    c->seed = 0;
    c->spp_offset = 0;
    c->nrc_train_samples = 65536;
    // Query where the path spread first exceeds 0.01 x the first-hit footprint:
    // on the interior at 1080p, 1 spp per frame, it reaches relMSE 1e-3 in 0.30x
    // the plain tracer's time, against 0.67-0.87x for fixed vertices 2..5.
    c->nrc_query_vertex = AQUA_NRC_QUERY_SPREAD;
}

AQUA_API void aqua_tuning_defaults(aqua_tuning* t) {
    if (!t) return;
    memset(t, 0, sizeof(*t));
    t->block_trace = 128;
    t->block_shade = 128;
    t->sort_by_material = 0;  // unsorted with deep queues beats the material sort (render.cu, plan_slots)
    t->iters_per_graph = 16;
}

AQUA_API aqua_status aqua_load_integrator_json(aqua_ctx* ctx, const char* path, aqua_integrator_cfg* out) {
    return guard(ctx, [&]() {
        need(path && out, "path and out must be non-NULL");
        aqua_integrator_cfg c;
        aqua_integrator_defaults(&c);
        load_integrator_json(path, &c);
        *out = c;
    });
}

AQUA_API aqua_status aqua_trace(aqua_ctx* ctx, aqua_scene* s, const aqua_ray* rays, size_t n, aqua_hit* out,
                                uint32_t flags, aqua_trace_counts* counts) {
    return guard(ctx, [&]() {
        need(s != nullptr, "scene is NULL");
        need_device(ctx);
        need(n == 0 || (rays && out), "rays and out must be non-NULL");
        need(n < ((size_t)1 << 34), "too many rays");
        trace_rays(ctx, s, rays, n, out, flags, counts);
    });
}

AQUA_API aqua_status aqua_render(aqua_ctx* ctx, aqua_scene* s, const aqua_integrator_cfg* cfg,
                                 const aqua_tuning* tuning, float* rgb_out, uint32_t flags, aqua_stats* stats) {
    return guard(ctx, [&]() {
        need(s && cfg && rgb_out, "scene, cfg and rgb_out must be non-NULL");
        need_device(ctx);
        aqua_tuning t;
        if (tuning) t = *tuning;
        else aqua_tuning_defaults(&t);
        if (cfg->type != AQUA_INTEGRATOR_PATH)
            throw Error(AQUA_ERR_UNSUPPORTED, "integrator type not available in aqua_render");
        need(t.kernel == AQUA_KERNEL_WAVEFRONT || t.kernel == AQUA_KERNEL_PERSISTENT,
             "tuning.kernel must be an AQUA_KERNEL_* value");
        const uint32_t wavefront_only = AQUA_RENDER_COUNT | AQUA_RENDER_STAGE_TIMING | AQUA_RENDER_ACCUMULATE;
        if (t.kernel == AQUA_KERNEL_PERSISTENT && !(flags & wavefront_only) && cfg->spp_offset == 0 &&
            cfg->row_step <= 1)
            render_persistent(ctx, s, *cfg, t, rgb_out, flags, stats);
        else
            render_path(ctx, s, *cfg, t, rgb_out, flags, stats);
    });
}

// Autotuner: times short renders (at most 16 spp) of every candidate launch
// shape of both integrator kernels (wavefront, persistent), two runs each,
// and keeps the fastest by device time.
AQUA_API aqua_status aqua_autotune(aqua_ctx* ctx, aqua_scene* s, const aqua_integrator_cfg* cfg, aqua_tuning* out) {
    return guard(ctx, [&]() {
        need(s && cfg && out, "scene, cfg and out must be non-NULL");
        need_device(ctx);
        if (cfg->type != AQUA_INTEGRATOR_PATH)
            throw Error(AQUA_ERR_UNSUPPORTED, "the autotuner tunes the path integrator");
        aqua_integrator_cfg c = *cfg;
        c.spp = std::max(1, std::min(cfg->spp, 16));
        c.row_begin = c.row_step = 0;  // tuned on the whole image
        size_t pixels = (size_t)s->host.cam.width * (size_t)s->host.cam.height;
        DevBuf film;
        dev_alloc(ctx, film, 12 * pixels);
        aqua_tuning best;
        aqua_tuning_defaults(&best);
        double best_ms = 1e300;
        try {
            for (int sort : {0, 1})
                for (int bt : {64, 128})
                    for (int bs : {64, 128})
                        for (int bps : {0, 4, 8}) {
                            aqua_tuning t;
                            aqua_tuning_defaults(&t);
                            t.sort_by_material = sort;
                            t.block_trace = bt;
                            t.block_shade = bs;
                            t.blocks_per_sm = bps;
                            double ms = 0.0;
                            for (int rep = 0; rep < 2; ++rep) {
                                aqua_stats st;
                                render_path(ctx, s, c, t, (float*)film.ptr, AQUA_RENDER_DEVICE_FILM, &st);
                                if (rep == 1) ms = st.device_ms;
                            }
                            if (ms < best_ms) {
                                best_ms = ms;
                                best = t;
                            }
                        }
            // The persistent kernel: block size x resident blocks.
            for (int block : {128, 256})
                for (int bps : {0, 4, 8}) {
                    aqua_tuning t;
                    aqua_tuning_defaults(&t);
                    t.kernel = AQUA_KERNEL_PERSISTENT;
                    t.block_trace = block;
                    t.blocks_per_sm = bps;
                    double ms = 0.0;
                    for (int rep = 0; rep < 2; ++rep) {
                        aqua_stats st;
                        render_persistent(ctx, s, c, t, (float*)film.ptr, AQUA_RENDER_DEVICE_FILM, &st);
                        if (rep == 1) ms = st.device_ms;
                    }
                    if (ms < best_ms) {
                        best_ms = ms;
                        best = t;
                    }
                }
        } catch (...) {
            dev_free(film);
            throw;
        }
        dev_free(film);
        *out = best;
    });
}

// Batch autotuner: block size x blocks per SM, timed on the same jobs with
// their sample counts divided by 32 (at least 1).
AQUA_API aqua_status aqua_autotune_batch(aqua_ctx* ctx, const aqua_job* jobs, size_t n, aqua_tuning* out) {
    return guard(ctx, [&]() {
        need(jobs && n > 0 && out, "jobs and out must be non-NULL and n > 0");
        need_device(ctx);
        std::vector<aqua_job> small(jobs, jobs + n);
        for (auto& j : small) j.spp = std::max(1, j.spp / 32);
        aqua_tuning best;
        aqua_tuning_defaults(&best);
        best.use_graph = 1;
        double best_ms = 1e300;
        for (int block : {64, 128, 256})
            for (int bps : {0, 2, 4, 8}) {
                aqua_tuning t;
                aqua_tuning_defaults(&t);
                t.block_trace = block;
                t.blocks_per_sm = bps;
                t.use_graph = 1;
                double ms = 0.0;
                for (int rep = 0; rep < 2; ++rep) {
                    aqua_batch_stats st{};
                    render_batch(ctx, small.data(), n, t, &st);
                    if (rep == 1) ms = st.device_ms;
                }
                if (ms < best_ms) {
                    best_ms = ms;
                    best = t;
                }
            }
        *out = best;
    });
}

AQUA_API aqua_status aqua_render_batch(aqua_ctx* ctx, const aqua_job* jobs, size_t n, const aqua_tuning* tuning,
                                       aqua_batch_stats* stats) {
    return guard(ctx, [&]() {
        need(jobs != nullptr || n == 0, "jobs is NULL");
        need_device(ctx);
        aqua_tuning t;
        if (tuning) t = *tuning;
        else {
            aqua_tuning_defaults(&t);
            t.use_graph = 1;
        }
        render_batch(ctx, jobs, n, t, stats);
    });
}

AQUA_API uint64_t aqua_workspace_bytes(const aqua_ctx* ctx) { return ctx ? ctx->ws.block.bytes : 0; }

AQUA_API aqua_status aqua_render_noalloc(aqua_ctx* ctx, aqua_scene* s, const aqua_integrator_cfg* cfg,
                                         float* rgb_out_device, aqua_stats* stats) {
    return guard(ctx, [&]() {
        need(s && cfg && rgb_out_device, "scene, cfg and rgb_out_device must be non-NULL");
        need_device(ctx);
        if (cfg->type != AQUA_INTEGRATOR_PATH)
            throw Error(AQUA_ERR_UNSUPPORTED, "aqua_render_noalloc renders the path integrator only");
        render_noalloc(ctx, s, *cfg, rgb_out_device, stats);
    });
}

AQUA_API uint64_t aqua_render_noalloc_max_pixels(void) { return (uint64_t)render_noalloc_max_pixels(); }

// ---------------------------------------------------------------- radiance cache
static_assert(AQUA_NRC_PARAMS == kNrcParams, "parameter count");
static_assert(AQUA_NRC_RAW == kNrcRaw, "raw feature count");

static void stage(aqua_ctx* ctx, DevBuf& b, size_t bytes) {
    if (b.bytes >= bytes && b.ptr) return;
    dev_free(b);
    dev_alloc(ctx, b, bytes);
}

AQUA_API void aqua_nrc_defaults(aqua_nrc_cfg* c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->learning_rate = 1e-2f;
    c->beta1 = 0.9f;
    c->beta2 = 0.99f;
    c->eps = 1e-8f;
    c->seed = 1;
    for (int i = 0; i < 3; ++i) { c->bbox_min[i] = 0.0f; c->bbox_max[i] = 1.0f; }
}

AQUA_API aqua_status aqua_nrc_create(aqua_ctx* ctx, const aqua_nrc_cfg* cfg, aqua_nrc** out) {
    return guard(ctx, [&]() {
        need(out != nullptr, "out must be non-NULL");
        need_device(ctx);
        *out = nullptr;
        aqua_nrc_cfg c;
        if (cfg) c = *cfg;
        else aqua_nrc_defaults(&c);
        for (int i = 0; i < 3; ++i)
            need(c.bbox_max[i] > c.bbox_min[i], "bbox_max must exceed bbox_min on every axis");
        need(c.learning_rate > 0.0f, "learning_rate must be positive");
        aqua_nrc* n = new aqua_nrc();
        try {
            n->net.lr = c.learning_rate;
            n->net.beta1 = c.beta1;
            n->net.beta2 = c.beta2;
            n->net.eps = c.eps;
            need(c.ema_decay >= 0.0f && c.ema_decay < 1.0f, "ema_decay must be in [0, 1)");
            n->net.ema_decay = c.ema_decay;
            need(c.forward_kernel >= AQUA_NRC_KERNEL_AUTO && c.forward_kernel <= AQUA_NRC_KERNEL_TCGEN05,
                 "forward_kernel must be an AQUA_NRC_KERNEL_* value");
            n->net.forward_tc = c.forward_kernel != AQUA_NRC_KERNEL_MMA_SYNC;
            for (int i = 0; i < 3; ++i) {
                n->net.bmin[i] = c.bbox_min[i];
                n->net.bext[i] = c.bbox_max[i] - c.bbox_min[i];
            }
            nrc_alloc(ctx, n->net);
            nrc_init_weights(ctx, n->net, c.seed);
        } catch (...) {
            nrc_release(n->net);
            delete n;
            throw;
        }
        *out = n;
    });
}

AQUA_API aqua_status aqua_nrc_destroy(aqua_ctx* ctx, aqua_nrc* n) {
    return guard(ctx, [&]() {
        if (!n) return;
        cudaStreamSynchronize(ctx->stream);
        nrc_release(n->net);
        dev_free(n->stage_in);
        dev_free(n->stage_tgt);
        dev_free(n->stage_out);
        delete n;
    });
}

AQUA_API aqua_status aqua_nrc_set_weights(aqua_ctx* ctx, aqua_nrc* n, const float* w) {
    return guard(ctx, [&]() {
        need(n && w, "nrc and w must be non-NULL");
        nrc_set_weights(ctx, n->net, w);
    });
}

AQUA_API aqua_status aqua_nrc_get_weights(aqua_ctx* ctx, aqua_nrc* n, float* w) {
    return guard(ctx, [&]() {
        need(n && w, "nrc and w must be non-NULL");
        AQ_CUDA(cudaMemcpyAsync(w, n->net.w, 4 * kNrcParams, cudaMemcpyDeviceToHost, ctx->stream));
        AQ_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

AQUA_API aqua_status aqua_nrc_get_gradients(aqua_ctx* ctx, aqua_nrc* n, float* g) {
    return guard(ctx, [&]() {
        need(n && g, "nrc and g must be non-NULL");
        AQ_CUDA(cudaMemcpyAsync(g, n->net.grad, 4 * kNrcParams, cudaMemcpyDeviceToHost, ctx->stream));
        AQ_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

AQUA_API aqua_status aqua_nrc_encode(aqua_ctx* ctx, aqua_nrc* n, const float* raw, size_t cnt, uint16_t* x,
                                     uint32_t flags) {
    return guard(ctx, [&]() {
        need(n != nullptr, "nrc is NULL");
        need(cnt == 0 || (raw && x), "raw and x must be non-NULL");
        need(cnt < (1u << 30), "too many rows");
        if (cnt == 0) return;
        const float* d_raw = raw;
        uint16_t* d_x = x;
        if (!(flags & AQUA_NRC_DEVICE_PTRS)) {
            stage(ctx, n->stage_in, 4 * kNrcRaw * cnt);
            stage(ctx, n->stage_out, 128 * cnt);
            AQ_CUDA(cudaMemcpyAsync(n->stage_in.ptr, raw, 4 * kNrcRaw * cnt, cudaMemcpyHostToDevice, ctx->stream));
            d_raw = (const float*)n->stage_in.ptr;
            d_x = (uint16_t*)n->stage_out.ptr;
        }
        nrc_encode_dev(ctx, n->net, d_raw, (int)cnt, d_x);
        if (!(flags & AQUA_NRC_DEVICE_PTRS))
            AQ_CUDA(cudaMemcpyAsync(x, d_x, 128 * cnt, cudaMemcpyDeviceToHost, ctx->stream));
        AQ_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

AQUA_API aqua_status aqua_nrc_forward(aqua_ctx* ctx, aqua_nrc* n, const uint16_t* x, size_t cnt, float* out,
                                      uint32_t flags) {
    return guard(ctx, [&]() {
        need(n != nullptr, "nrc is NULL");
        need(cnt == 0 || (x && out), "x and out must be non-NULL");
        need(cnt < (1u << 30), "too many rows");
        if (cnt == 0) return;
        const uint16_t* d_x = x;
        float* d_out = out;
        if (!(flags & AQUA_NRC_DEVICE_PTRS)) {
            stage(ctx, n->stage_in, 128 * cnt);
            stage(ctx, n->stage_out, 12 * cnt);
            AQ_CUDA(cudaMemcpyAsync(n->stage_in.ptr, x, 128 * cnt, cudaMemcpyHostToDevice, ctx->stream));
            d_x = (const uint16_t*)n->stage_in.ptr;
            d_out = (float*)n->stage_out.ptr;
        } else {
            need(((uintptr_t)x & 15) == 0, "x must be 16-byte aligned");
        }
        std::unique_ptr<EventPair> ev;
        if (flags & AQUA_NRC_TIMING) {
            ev.reset(new EventPair());
            AQ_CUDA(cudaEventRecord(ev->e[0], ctx->stream));
        }
        nrc_forward_dev(ctx, n->net, d_x, (int)cnt, d_out);
        if (ev) AQ_CUDA(cudaEventRecord(ev->e[1], ctx->stream));
        if (!(flags & AQUA_NRC_DEVICE_PTRS))
            AQ_CUDA(cudaMemcpyAsync(out, d_out, 12 * cnt, cudaMemcpyDeviceToHost, ctx->stream));
        AQ_CUDA(cudaStreamSynchronize(ctx->stream));
        nrc_check_tc(ctx, n->net);
        if (ev) n->last_ms = ev->ms();
    });
}

AQUA_API aqua_status aqua_nrc_last_ms(aqua_ctx* ctx, aqua_nrc* n, float* ms) {
    return guard(ctx, [&]() {
        need(n && ms, "nrc and ms must be non-NULL");
        *ms = n->last_ms;
    });
}

AQUA_API aqua_status aqua_render_nrc(aqua_ctx* ctx, aqua_scene* s, const aqua_integrator_cfg* cfg,
                                     const aqua_tuning* tuning, aqua_nrc* nrc, float* rgb_out, uint32_t flags,
                                     aqua_stats* stats) {
    return guard(ctx, [&]() {
        need(s && cfg && nrc && rgb_out, "scene, cfg, nrc and rgb_out must be non-NULL");
        need_device(ctx);
        aqua_tuning t;
        if (tuning) t = *tuning;
        else aqua_tuning_defaults(&t);
        render_nrc(ctx, s, *cfg, t, nrc, rgb_out, flags, stats);
    });
}

AQUA_API aqua_status aqua_nrc_train_step(aqua_ctx* ctx, aqua_nrc* n, const uint16_t* x, const float* target,
                                         size_t cnt, double* loss, uint32_t flags) {
    return guard(ctx, [&]() {
        need(n != nullptr, "nrc is NULL");
        need(cnt > 0 && x && target, "x and target must be non-NULL and n > 0");
        need(cnt < (1u << 26), "too many rows");
        const uint16_t* d_x = x;
        const float* d_t = target;
        if (!(flags & AQUA_NRC_DEVICE_PTRS)) {
            stage(ctx, n->stage_in, 128 * cnt);
            stage(ctx, n->stage_tgt, 12 * cnt);
            AQ_CUDA(cudaMemcpyAsync(n->stage_in.ptr, x, 128 * cnt, cudaMemcpyHostToDevice, ctx->stream));
            AQ_CUDA(cudaMemcpyAsync(n->stage_tgt.ptr, target, 12 * cnt, cudaMemcpyHostToDevice, ctx->stream));
            d_x = (const uint16_t*)n->stage_in.ptr;
            d_t = (const float*)n->stage_tgt.ptr;
        } else {
            need(((uintptr_t)x & 15) == 0, "x must be 16-byte aligned");
        }
        std::unique_ptr<EventPair> ev;
        if (flags & AQUA_NRC_TIMING) {
            ev.reset(new EventPair());
            AQ_CUDA(cudaEventRecord(ev->e[0], ctx->stream));
        }
        nrc_train_step_dev(ctx, n->net, d_x, d_t, (int)cnt);
        if (ev) AQ_CUDA(cudaEventRecord(ev->e[1], ctx->stream));
        struct {
            double loss;
            uint32_t tc_err, pad;
        } rb{};  // the loss and, right after it, the tcgen05 error flag
        AQ_CUDA(cudaMemcpyAsync(&rb, n->net.loss, 16, cudaMemcpyDeviceToHost, ctx->stream));
        AQ_CUDA(cudaStreamSynchronize(ctx->stream));
        if (rb.tc_err) nrc_check_tc(ctx, n->net);  // resets the flag and throws
        if (ev) n->last_ms = ev->ms();
        const double l = rb.loss;
        if (loss) *loss = l / (double)(cnt * kNrcOut);
    });
}

}  // extern "C"
