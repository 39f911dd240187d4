/*
 * aqua.h — C ABI of libaqua, the GB300 (sm_103a) light-transport hot path.
 *
 * The reference crate (`arukas`, Cargo.toml:2-5) never wrote its renderer API:
 * src/lib.rs is empty. Its de-facto contract is the on-disk data it ships:
 *   - scene JSON        scenes/cbox.json:1-628, scenes/room.json:1-3900
 *   - integrator JSON   scenes/integrator.json:1-9
 *   - BSON `.mesh`      scenes/<name>.mesh (name, vertices, normals, texcoords, indices)
 * Each entry point below names the part of that contract (file:line) it serves.
 * A Rust `extern "C"` crate binds these 1:1 (no torch types, plain pointers and
 * sizes, no exceptions across the boundary).
 *
 * Threading: one aqua_ctx owns one CUDA device and one stream. Calls on the same
 * context must be serialised by the caller; different contexts may be used from
 * different threads.
 */
#ifndef AQUA_H
#define AQUA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define AQUA_API __declspec(dllexport)
#else
#define AQUA_API __attribute__((visibility("default")))
#endif

/* ---------------------------------------------------------------- status */
typedef enum aqua_status {
    AQUA_OK = 0,
    AQUA_ERR_INVALID_ARG = 1,   /* null handle, bad size, bad enum            */
    AQUA_ERR_IO = 2,            /* file cannot be opened or read              */
    AQUA_ERR_PARSE = 3,         /* malformed JSON / BSON / unknown enum tag   */
    AQUA_ERR_MISSING_ASSET = 4, /* a referenced .mesh or texture is absent    */
    AQUA_ERR_CUDA = 5,          /* a CUDA runtime call failed                 */
    AQUA_ERR_OOM = 6,           /* host or device allocation failed           */
    AQUA_ERR_TIMEOUT = 7,       /* a bounded device wait gave up              */
    AQUA_ERR_UNSUPPORTED = 8    /* valid input this build does not implement  */
} aqua_status;

typedef struct aqua_ctx aqua_ctx;
typedef struct aqua_scene aqua_scene;

/* aqua_options.device value for a context without a GPU: scenes load, BVHs
 * build and every export works; trace and render return AQUA_ERR_UNSUPPORTED. */
#define AQUA_DEVICE_HOST_ONLY (-2)

typedef struct aqua_options {
    int32_t device;        /* CUDA ordinal; -1 = current device; AQUA_DEVICE_HOST_ONLY */
    int32_t verbose;       /* 0 = silent                                         */
    uint64_t fail_alloc_after; /* test hook: 0 = off; n = the n-th device
                                  allocation of this context fails with OOM      */
} aqua_options;

/* One ray, 32 bytes: two 16-byte halves so the device reads it with two
 * 128-bit loads. Directions need not be normalised; t is in units of |d|. */
typedef struct aqua_ray {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
} aqua_ray;

/* Closest hit, 16 bytes. prim = index of the triangle in scene order
 * (the order of aqua_scene_export_triangles), -1 on a miss. The hit point is
 * (1-u-v)*v0 + u*v1 + v*v2. For AQUA_TRACE_ANY_HIT, prim is 1 when occluded
 * and -1 when not, and t/u/v are 0. */
typedef struct aqua_hit {
    float t, u, v;
    int32_t prim;
} aqua_hit;

enum {
    AQUA_TRACE_DEVICE_PTRS = 1u << 0, /* rays/hits are device pointers        */
    AQUA_TRACE_ANY_HIT = 1u << 1,     /* occlusion query, early exit          */
    AQUA_TRACE_COUNT = 1u << 2        /* fill aqua_trace_counts (slower)      */
};

/* Per-call traversal work, summed over all rays (node visits = internal nodes
 * whose two child boxes were tested; tri tests = ray-triangle tests). */
typedef struct aqua_trace_counts {
    uint64_t node_visits;
    uint64_t tri_tests;
    double kernel_ms;     /* device time of the traversal kernel             */
} aqua_trace_counts;

/* Integrator settings. Mirrors scenes/integrator.json:1-9 (type, spp,
 * batch_size, max_depth, training_iters, learning_rate, visualize_cache),
 * plus the knobs the render path needs. */
enum { AQUA_INTEGRATOR_PATH = 0, AQUA_INTEGRATOR_NRC = 1 };
enum { AQUA_NRC_QUERY_SPREAD = -1 };

typedef struct aqua_integrator_cfg {
    int32_t type;            /* AQUA_INTEGRATOR_PATH or AQUA_INTEGRATOR_NRC */
    int32_t spp;             /* samples per pixel                           */
    int32_t max_depth;       /* bounces; NEE at vertices 0..max_depth-1;
                                [0, 250], else AQUA_ERR_INVALID_ARG          */
    int32_t rr_depth;        /* Russian roulette from this bounce on; [0, 250]
                                (above max_depth: no roulette)              */
    int32_t batch_size;      /* NRC: training batch (integrator.json:4)     */
    int32_t training_iters;  /* NRC: optimizer steps per frame              */
    float learning_rate;     /* NRC: Adam step size (integrator.json:7)     */
    int32_t visualize_cache; /* NRC: write the cache instead of radiance    */
    uint64_t seed;           /* RNG seed: PCG32 stream per pixel            */
    int32_t spp_offset;      /* first sample index (progressive rendering)  */
    int32_t nrc_train_samples; /* NRC: training records per frame          */
    int32_t nrc_query_vertex;  /* NRC: query the cache at this vertex (>= 2),
                                  or AQUA_NRC_QUERY_SPREAD (the default):
                                  where the path's spread first exceeds 0.01 x
                                  its first-hit footprint (Mueller et al.
                                  2021), at vertex 2 or later */
    /* Row subset (wavefront renders): with row_step > 1 only the camera
     * image's rows row_begin, row_begin + row_step, ... are rendered, and
     * rgb_out holds just those rows in order (rows x width x 3). Every pixel
     * keeps the random-number stream of its place in the full image, so the
     * rows equal the same rows of a full render with the same seed. 0 or 1 =
     * the whole image (row_begin 0). The persistent kernel renders whole
     * images only (aqua_render then runs the wavefront). */
    int32_t row_begin, row_step;
    int32_t reserved0;
} aqua_integrator_cfg;

/* Launch shape of the wavefront. 0 in any field = the library default.
 * For a given `replicas` value every choice gives a bit-identical image: each
 * pixel (or, with replicas, each pixel's film copy) is owned by exactly one
 * path slot, which runs its samples in order. Automatic replicas aim at
 * about 2^24 paths in flight (2^20 with the material sort and in the cache
 * mode), so the automatic count can differ between sorted and unsorted
 * renders of an image. */
typedef struct aqua_tuning {
    int32_t slots;          /* paths in flight (0 = one per pixel, capped at
                               2^24, or 2^20 sorted)                         */
    int32_t block_trace;    /* threads per block, traversal kernels          */
    int32_t block_shade;    /* threads per block, shading kernel             */
    int32_t sort_by_material; /* 1 = bin hits by material before shading
                                 (default 0)                                 */
    int32_t blocks_per_sm;  /* persistent grid = SMs * this                  */
    int32_t use_graph;      /* 1 = replay iterations from a CUDA graph       */
    int32_t iters_per_graph;/* iterations between host checks of the queue  */
    int32_t replicas;       /* sample replicas per pixel: 0 = automatic (images
                               below the paths-in-flight target get several
                               slots per pixel, each with its own film
                               copy), 1 = off, k = k copies                  */
    int32_t kernel;         /* AQUA_KERNEL_*: the wavefront (three launches per
                               bounce over compacted queues)
                               or one persistent launch whose lanes each keep a
                               path in flight and regenerate it in place (the
                               aqua_render_batch kernel; block_trace and
                               blocks_per_sm shape it). Same image either way.
                               Renders with AQUA_RENDER_COUNT, _STAGE_TIMING or
                               _ACCUMULATE, or a non-zero spp_offset, run on the
                               wavefront. aqua_autotune times both.           */
} aqua_tuning;

enum { AQUA_KERNEL_WAVEFRONT = 0, AQUA_KERNEL_PERSISTENT = 1 };

typedef struct aqua_stats {
    uint64_t paths;          /* camera paths completed                       */
    uint64_t ext_rays;       /* closest-hit rays traced                      */
    uint64_t shadow_rays;    /* any-hit rays traced                          */
    uint64_t iterations;     /* wavefront iterations                         */
    double device_ms;        /* device time of the whole render              */
    /* With AQUA_RENDER_STAGE_TIMING, every 8th wavefront iteration has its
     * three launches bracketed by CUDA events; *_ms sum those launches and
     * *_launches count them. Without it, *_launches count every launch. */
    double trace_ms;         /* closest-hit (extension ray) launches         */
    double shadow_ms;        /* any-hit (shadow ray) launches                */
    double shade_ms;         /* shading launches                             */
    uint64_t trace_launches;
    uint64_t shadow_launches;
    uint64_t shade_launches;
    uint64_t total_launches; /* every kernel this call launched              */
    uint64_t node_visits;    /* filled when stage counting is requested      */
    uint64_t tri_tests;
    uint64_t shadow_node_visits;
    uint64_t shadow_tri_tests;
    uint64_t nrc_queries;    /* NRC: cache queries                           */
    uint64_t nrc_train_records;
    double nrc_ms;           /* NRC: device time of MLP kernels              */
    double nrc_loss;         /* NRC: last training loss                      */
} aqua_stats;

enum {
    AQUA_RENDER_DEVICE_FILM = 1u << 0, /* rgb_out is a device pointer         */
    AQUA_RENDER_STAGE_TIMING = 1u << 1,/* fill the *_ms stage times          */
    AQUA_RENDER_COUNT = 1u << 2,       /* fill node/tri counters (slower)    */
    AQUA_RENDER_ACCUMULATE = 1u << 3   /* rgb_out += sum (no divide, no clear) */
};

/* Scene summary. */
typedef struct aqua_scene_info {
    int32_t width, height;
    int32_t num_triangles, num_materials, num_lights, num_textures;
    int32_t num_meshes, num_bvh_nodes; /* nodes of the four-wide BVH     */
    int32_t bvh_depth, max_leaf_size;  /* wide nodes on the longest path  */
    uint64_t device_bytes;   /* device memory held by the scene             */
    uint64_t upload_bytes;   /* bytes copied host->device by one upload     */
    float env[3];            /* constant radiance seen by escaping rays     */
    int32_t bvh_format;      /* AQUA_BVH_FULL or AQUA_BVH_QUANTIZED: the node
                                format the device walks                     */
} aqua_scene_info;

/* BVH node formats. The tree is the same; quantized nodes (64 bytes) hold
 * the child boxes as 8-bit offsets in a per-node frame, rounded outward
 * (layout in bvh.h), so walks find the same closest hits from half the node
 * bytes, at the cost of a few instructions per visit (on GB300 the
 * full-precision walk is faster for trees of millions of triangles). AUTO
 * picks quantized nodes only when the full-precision ones exceed 8 GiB. */
enum { AQUA_BVH_AUTO = -1, AQUA_BVH_FULL = 0, AQUA_BVH_QUANTIZED = 1 };

/* Camera, after parsing scenes/cbox.json:516-543 (`Perspective`). */
typedef struct aqua_camera {
    int32_t width, height;
    float fov_deg;            /* full vertical field of view                */
    float lens_radius, focal;
    float pos[3];
    float right[3], up[3], back[3]; /* camera looks along -back          */
} aqua_camera;

/* Material, the Lambert + GGX subset of `Principled` (scenes/cbox.json:3-62). */
/* The `Principled` parameters (scenes/cbox.json:3-62) the renderer
 * consumes. Lambert diffuse, sheen (Burley 2012), GGX specular with
 * Schlick Fresnel and specular tint, a clearcoat GTR1 lobe (Burley 2012)
 * and a rough dielectric transmission lobe (Walter et al. 2007) with the
 * given ior. subsurface*, anisotropic* and `hint` are not consumed. All
 * weights lie in [0, 1]; ior in [1, 4]. */
typedef struct aqua_material {
    float base_color[3];      /* linear RGB (Srgb values are decoded)       */
    int32_t base_texture;     /* -1 = none, else texture index              */
    float metallic, roughness, specular;
    float specular_tint;      /* dielectric F0 tinted toward the base hue   */
    float sheen, sheen_tint;
    float clearcoat, clearcoat_roughness;
    float transmission, ior;  /* glass lobe weight (1-metallic)*transmission */
    int32_t reserved[2];
} aqua_material;

enum { AQUA_LIGHT_QUAD = 0, AQUA_LIGHT_POINT = 1, AQUA_LIGHT_TRIANGLE = 2 };

typedef struct aqua_light {
    int32_t type;
    float p0[3], e1[3], e2[3]; /* quad: p0 + a*e1 + b*e2 (a, b in [0,1]);
                                  triangle: the same with a + b <= 1;
                                  both emit on the side of e1 x e2         */
    float radiance[3];         /* quad: radiance; point: intensity          */
    float pmf;                 /* selection probability (power-weighted)    */
} aqua_light;

/* A batched job: one view of one scene. */
typedef struct aqua_job {
    aqua_scene* scene;
    int32_t width, height, spp, max_depth;
    uint64_t seed;
    float* rgb_out;           /* device pointer, width*height*3 floats      */
} aqua_job;

typedef struct aqua_batch_stats {
    double device_ms;         /* whole batch, device time                   */
    uint64_t paths;
    double* job_ms;           /* optional, n entries: completion time of each
                                 job measured from the start of the batch   */
} aqua_batch_stats;

/* ---------------------------------------------------------------- lifetime */
AQUA_API aqua_status aqua_create(aqua_ctx** out, const aqua_options* opt);
AQUA_API void aqua_destroy(aqua_ctx* ctx);
/* Message of the last failing call on ctx ("" when none). Valid until the
 * next call on ctx. aqua_create failures are reported by aqua_last_error(NULL).
 * The text is UTF-8 (input bytes it quotes that are not are written as \xNN),
 * at most 1024 bytes. */
AQUA_API const char* aqua_last_error(const aqua_ctx* ctx);
AQUA_API const char* aqua_status_string(aqua_status s);
/* ABI version: 100 x major + minor. Major 3: 64-byte aqua_material with the
 * Principled lobes, integrator row subsets, BVH node formats. Major 2:
 * aqua_scene_export_bvh returns the four-wide tree (32 floats per node;
 * major 1 returned a binary tree of 16 floats per node). */
#define AQUA_VERSION 300
AQUA_API int aqua_version(void);

/* ---------------------------------------------------------------- scenes */
/* Loads a scene JSON (scenes/cbox.json:1-628 schema: named_bsdfs, camera,
 * lights, shapes) with its BSON meshes from the JSON's directory. A missing
 * mesh (e.g. living_room_Default_43.mesh, .MISSING_LARGE_BLOBS:1) fails with
 * AQUA_ERR_MISSING_ASSET unless allow_missing is set, which skips it. Image
 * textures (room.json:6) are decoded, on all host threads, by the built-in
 * JPEG decoder (Huffman sequential and progressive, 8-bit, grey or YCbCr); a
 * file it refuses (arithmetic coding, 12-bit, lossless) fails with
 * AQUA_ERR_UNSUPPORTED and a missing file with AQUA_ERR_MISSING_ASSET, unless
 * allow_missing is set, which replaces the texture by mid-grey. Texture rows are stored bottom-up, so
 * v = 0 is the bottom edge of the image (OBJ texture coordinates). */
AQUA_API aqua_status aqua_load_scene_json(aqua_ctx* ctx, const char* path,
                                          int32_t allow_missing, aqua_scene** out);
/* Procedural scenes 1..5: 1 = Cornell box (Lambert), 2 = Cornell box with GGX
 * (roughness U[0.05,0.8], metallic {0,1}), 3 = synthetic interior (153 meshes,
 * ~1.2M triangles, 8 textures 2048^2, 16 quad lights), 4 = scene 3 for the
 * radiance cache, 5 = random-sphere field (~4M triangles).
 * width/height <= 0 keep the scene's own resolution. */
AQUA_API aqua_status aqua_make_procedural_scene(aqua_ctx* ctx, int32_t config_id,
                                                uint64_t seed, int32_t width,
                                                int32_t height, aqua_scene** out);
AQUA_API aqua_status aqua_scene_free(aqua_ctx* ctx, aqua_scene* scene);
AQUA_API aqua_status aqua_scene_set_resolution(aqua_ctx* ctx, aqua_scene* scene,
                                               int32_t width, int32_t height);
/* Re-copies the scene's device arrays from its pinned host copy (what a
 * loader does after building); used to time uploads end to end. */
AQUA_API aqua_status aqua_scene_upload(aqua_ctx* ctx, aqua_scene* scene);
AQUA_API aqua_status aqua_scene_get_info(aqua_ctx* ctx, const aqua_scene* scene,
                                         aqua_scene_info* out);

/* Host copies of the scene, for checkers and tools. Triangles in scene order:
 * verts = 9 floats per triangle, uvs = 6 floats per triangle, mat = material
 * index per triangle, light = index of the light the triangle is part of or -1.
 * Any output may be NULL. */
AQUA_API aqua_status aqua_scene_export_triangles(aqua_ctx* ctx, const aqua_scene* scene,
                                                 float* verts, float* uvs, int32_t* mat,
                                                 int32_t* light);
AQUA_API aqua_status aqua_scene_export_camera(aqua_ctx* ctx, const aqua_scene* scene,
                                              aqua_camera* out);
AQUA_API aqua_status aqua_scene_export_materials(aqua_ctx* ctx, const aqua_scene* scene,
                                                 aqua_material* out);
AQUA_API aqua_status aqua_scene_export_lights(aqua_ctx* ctx, const aqua_scene* scene,
                                              aqua_light* out);
/* Texture i as RGBA8, row-major from v = 0, sRGB-encoded. Pass rgba = NULL to query the size. */
AQUA_API aqua_status aqua_scene_export_texture(aqua_ctx* ctx, const aqua_scene* scene,
                                               int32_t i, int32_t* width, int32_t* height,
                                               uint8_t* rgba);
/* Vertex normals, 9 floats per triangle in aqua_scene_export_triangles order,
 * from the meshes' `normals` (a mesh without them contributes its face
 * normal). *present = 0 when no mesh of the scene has normals: the scene is
 * then shaded with geometric normals and nrm is left untouched. nrm may be
 * NULL to query presence. */
AQUA_API aqua_status aqua_scene_export_normals(aqua_ctx* ctx, const aqua_scene* scene, float* nrm,
                                               int32_t* present);
/* Decodes JPEG bytes (the decoder `Image` textures go through; it stands in
 * for the reference's `image` crate, Cargo.toml:13) into 8-bit RGB, row 0 =
 * the top of the image. Pass rgb = NULL to query the size. Works on a
 * host-only context. */
AQUA_API aqua_status aqua_decode_jpeg(aqua_ctx* ctx, const uint8_t* data, size_t n, int32_t* width,
                                      int32_t* height, uint8_t* rgb);
/* Converts a Wavefront OBJ and the MTL libraries it names into the scene
 * format aqua_load_scene_json reads, as the reference's tobj-based
 * conversion (Cargo.toml:23) produced scenes/CornellBox-Original_*.mesh and
 * scenes/cbox.json: one BSON .mesh per OBJ group, `<obj stem>_<group>_<k>.mesh`
 * (name, vertices, normals, texcoords, indices; faces fanned into
 * triangles), and out_dir/scene_name with the MTL materials (Kd as an Srgb
 * colour, Ke as emission, map_Kd as an Image texture; metallic 0, specular
 * 0, roughness 0.4), a camera of width x height framing the model, and the
 * shapes. meshes / triangles may be NULL. Works on a host-only context. */
AQUA_API aqua_status aqua_convert_obj(aqua_ctx* ctx, const char* obj_path, const char* out_dir,
                                      const char* scene_name, int32_t width, int32_t height,
                                      int32_t* meshes, int32_t* triangles);
/* Writes a W x H x 3 float film (row 0 at the top) to `path`: ".pfm" as
 * little-endian float PFM, ".ppm" as 8-bit P6 of the sRGB-encoded film
 * clamped to [0, 1]. */
AQUA_API aqua_status aqua_write_image(aqua_ctx* ctx, const char* path, const float* rgb, int32_t width,
                                      int32_t height);
/* The flattened BVH as the device holds it: a four-wide tree, nodes = 32
 * floats per node (eight 16-byte words: lo.x, hi.x, lo.y, hi.y, lo.z, hi.z of
 * the four child boxes, then the four child links and the four leaf counts as
 * int32; layout in bvh.h), tri_order[k] = scene index of the k-th triangle in
 * leaf order. */
AQUA_API aqua_status aqua_scene_export_bvh(aqua_ctx* ctx, const aqua_scene* scene,
                                           float* nodes, int32_t* tri_order);
/* The quantized copy of the same tree: 16 floats per node (bvh.h). */
AQUA_API aqua_status aqua_scene_export_bvh_quantized(aqua_ctx* ctx, const aqua_scene* scene, float* nodes);
/* Selects the node format the device walks (AQUA_BVH_*) and rebuilds the
 * scene's device image from the tree already built. */
AQUA_API aqua_status aqua_scene_set_bvh_format(aqua_ctx* ctx, aqua_scene* scene, int32_t format);

/* ---------------------------------------------------------------- integrator */
/* Parses scenes/integrator.json:1-9. Unknown `type` strings fail with
 * AQUA_ERR_PARSE. Fields absent from the file keep aqua_integrator_defaults. */
AQUA_API aqua_status aqua_load_integrator_json(aqua_ctx* ctx, const char* path,
                                               aqua_integrator_cfg* out);
AQUA_API void aqua_integrator_defaults(aqua_integrator_cfg* out);
AQUA_API void aqua_tuning_defaults(aqua_tuning* out);

/* ---------------------------------------------------------------- the hot path */
/* Traces n rays against the scene BVH (closest hit, or any hit with
 * AQUA_TRACE_ANY_HIT). counts may be NULL. */
AQUA_API aqua_status aqua_trace(aqua_ctx* ctx, aqua_scene* scene, const aqua_ray* rays,
                                size_t n, aqua_hit* out, uint32_t flags,
                                aqua_trace_counts* counts);

/* Renders the scene: rgb_out receives width*height*3 floats, the mean of spp
 * samples per pixel (linear radiance), row 0 at the top. tuning and stats may
 * be NULL. */
AQUA_API aqua_status aqua_render(aqua_ctx* ctx, aqua_scene* scene,
                                 const aqua_integrator_cfg* cfg, const aqua_tuning* tuning,
                                 float* rgb_out, uint32_t flags, aqua_stats* stats);

/* Times short renders (at most 16 spp) over a grid of launch shapes —
 * material sort, traversal and shading block sizes, blocks per SM — and
 * returns the fastest. The image does not depend on the choice. */
AQUA_API aqua_status aqua_autotune(aqua_ctx* ctx, aqua_scene* scene,
                                   const aqua_integrator_cfg* cfg, aqua_tuning* out);

/* Renders n jobs (views of up to n scenes, uneven resolutions and spp; at
 * most 1024 jobs) in one persistent launch replayed from a captured CUDA
 * graph (tuning->use_graph, on when tuning is NULL). Each lane owns one
 * pixel and runs its samples one path after another; idle lanes take the
 * next pixels from a global queue on which the jobs are laid out shortest
 * first (pixels x spp), so small jobs complete early. Every job's image
 * equals aqua_render's. rgb_out of each job is a device buffer. stats->job_ms,
 * when non-NULL, receives each job's completion time from the start of the
 * launch (device clock). tuning->block_trace = threads per block (64, 128,
 * 256), tuning->blocks_per_sm = persistent blocks per SM (0 = occupancy). */
AQUA_API aqua_status aqua_render_batch(aqua_ctx* ctx, const aqua_job* jobs, size_t n,
                                       const aqua_tuning* tuning, aqua_batch_stats* stats);
/* Times the batch's launch shapes on the same jobs at spp / 32 and returns
 * the fastest (block size, blocks per SM). */
AQUA_API aqua_status aqua_autotune_batch(aqua_ctx* ctx, const aqua_job* jobs, size_t n, aqua_tuning* out);

/* Device memory currently held by the context's render workspace. */
AQUA_API uint64_t aqua_workspace_bytes(const aqua_ctx* ctx);

/* ---------------------------------------------------------------- radiance cache */
/* The network of the `"type": "nrc"` integrator (scenes/integrator.json:2-7):
 * 64 encoded inputs -> 5 hidden layers of 64 (ReLU) -> RGB radiance, BF16
 * weights and activations with FP32 accumulation on tensor cores, trained
 * online with Adam on a relative L2 loss. Weights are FP32 row-major
 * [out][in]: W1..W5 (64x64) then W6 (3x64), AQUA_NRC_PARAMS values. */
typedef struct aqua_nrc aqua_nrc;

enum { AQUA_NRC_PARAMS = 20672, AQUA_NRC_INPUTS = 64, AQUA_NRC_RAW = 16 };
enum {
    AQUA_NRC_DEVICE_PTRS = 1u << 0, /* x / raw / out / target are device pointers */
    AQUA_NRC_TIMING = 1u << 1       /* time the call's device work (aqua_nrc_forward,
                                       aqua_nrc_train_step) with CUDA events on
                                       the context's stream; read it with
                                       aqua_nrc_last_ms                          */
};

typedef struct aqua_nrc_cfg {
    float learning_rate;          /* Adam step size                         */
    float beta1, beta2, eps;      /* Adam moments                           */
    uint64_t seed;                /* He-uniform initial weights             */
    float bbox_min[3], bbox_max[3]; /* box that normalises positions        */
    float ema_decay;              /* > 0: inference (aqua_nrc_forward and the
                                     cached renderer) uses an exponential
                                     moving average of the trained weights  */
    int32_t forward_kernel;       /* inference kernel, AQUA_NRC_KERNEL_*    */
} aqua_nrc_cfg;

/* Inference kernels: AUTO picks TCGEN05 (5th-generation tensor cores, the
 * accumulator in tensor memory); MMA_SYNC is the warp-level tensor-core
 * kernel the training step also uses. Both give the same results up to the
 * order of FP32 accumulation. */
enum { AQUA_NRC_KERNEL_AUTO = 0, AQUA_NRC_KERNEL_MMA_SYNC = 1, AQUA_NRC_KERNEL_TCGEN05 = 2 };

AQUA_API void aqua_nrc_defaults(aqua_nrc_cfg* cfg);
AQUA_API aqua_status aqua_nrc_create(aqua_ctx* ctx, const aqua_nrc_cfg* cfg, aqua_nrc** out);
AQUA_API aqua_status aqua_nrc_destroy(aqua_ctx* ctx, aqua_nrc* nrc);
/* Replaces the weights (and resets the Adam state). */
AQUA_API aqua_status aqua_nrc_set_weights(aqua_ctx* ctx, aqua_nrc* nrc, const float* w);
AQUA_API aqua_status aqua_nrc_get_weights(aqua_ctx* ctx, aqua_nrc* nrc, float* w);
/* Gradient of the mean loss used by the last training step. */
AQUA_API aqua_status aqua_nrc_get_gradients(aqua_ctx* ctx, aqua_nrc* nrc, float* g);
/* raw: n x AQUA_NRC_RAW floats per vertex (position 3, outgoing direction 3,
 * normal 3, roughness, diffuse albedo 3, specular F0 3); x: n x 64 bf16. */
AQUA_API aqua_status aqua_nrc_encode(aqua_ctx* ctx, aqua_nrc* nrc, const float* raw, size_t n, uint16_t* x,
                                     uint32_t flags);
/* out: n x 3 floats (radiance). */
AQUA_API aqua_status aqua_nrc_forward(aqua_ctx* ctx, aqua_nrc* nrc, const uint16_t* x, size_t n, float* out,
                                      uint32_t flags);
/* Device milliseconds of the last call made with AQUA_NRC_TIMING. */
AQUA_API aqua_status aqua_nrc_last_ms(aqua_ctx* ctx, aqua_nrc* nrc, float* ms);
/* One Adam step on a batch of n records (x, target radiance n x 3); loss =
 * the batch's mean relative L2 loss before the step (may be NULL). */
AQUA_API aqua_status aqua_nrc_train_step(aqua_ctx* ctx, aqua_nrc* nrc, const uint16_t* x, const float* target,
                                         size_t n, double* loss, uint32_t flags);

/* One frame of the cached renderer (`"type": "nrc"`, integrator.json:2).
 * cfg->spp samples per pixel. Paths stop at vertex cfg->nrc_query_vertex
 * (vertex 1 = first hit), or where their spread calls for it
 * (AQUA_NRC_QUERY_SPREAD), and add throughput x cache; about
 * cfg->nrc_train_samples vertices of unbiased training paths become
 * training records, and the network takes ceil(records / cfg->batch_size)
 * Adam steps (at most cfg->training_iters when that is > 0) after the frame
 * is rendered. Positions are encoded relative to the scene's bounding box.
 * cfg->visualize_cache renders the cache at the first hit instead (no
 * training). Same rgb_out, flags and stats as aqua_render; the stats'
 * nrc_* fields are filled. */
AQUA_API aqua_status aqua_render_nrc(aqua_ctx* ctx, aqua_scene* scene, const aqua_integrator_cfg* cfg,
                                     const aqua_tuning* tuning, aqua_nrc* nrc, float* rgb_out, uint32_t flags,
                                     aqua_stats* stats);

/* aqua_render without any device allocation. No counterpart in the
 * reference: it exists for callers that may not let a library call
 * cudaMalloc — engines that hand out all device memory from their own arena
 * under a fixed budget, and hosts where the implicit device-wide
 * synchronisation of cudaMalloc/cudaFree would stall other GPU work.
 *
 * It renders like aqua_render (path integrator, same image bit for bit) but
 * keeps all scratch — path state, queues, film — in one static device array
 * of this library (about 17.3 MB, held by every GPU that loads the library
 * until the process exits). The scene must already be loaded and
 * rgb_out_device is a device buffer of width*height*3 floats owned by the
 * caller. Limits: at most aqua_render_noalloc_max_pixels() pixels (2^19),
 * else AQUA_ERR_INVALID_ARG before any device work.
 *
 * The first call on a device looks up the array's device address (a
 * one-time set-up per device); make that first call before any stream
 * capture. The address is kept for the life of the process: a device reset
 * (cudaDeviceReset) unloads the array, and the library must not be used on
 * that device afterwards. Every call shares the array and clears what it needs; calls
 * whose work overlaps on the GPU (other contexts or threads at the same
 * time) race on it and must be serialised by the caller. stats may be NULL;
 * its timing fields stay 0. */
AQUA_API aqua_status aqua_render_noalloc(aqua_ctx* ctx, aqua_scene* scene, const aqua_integrator_cfg* cfg,
                                         float* rgb_out_device, aqua_stats* stats);
AQUA_API uint64_t aqua_render_noalloc_max_pixels(void);

#ifdef __cplusplus
}
#endif

#endif /* AQUA_H */
