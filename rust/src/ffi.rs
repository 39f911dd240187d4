//! Raw binding of libaqua's C ABI (`include/aqua.h`), declaration for
//! declaration: the opaque handles, the `#[repr(C)]` structs field for field,
//! the constants and every entry point. This is the `src/ffi.rs` a
//! maintainer of the reference crate (`arukas`) adds; the reference's
//! `src/lib.rs` is empty, so nothing existing is replaced.
//!
//! `tests/test_integration_binding.py` parses this file and checks it
//! against the header (names, parameter and field types, pointer constness,
//! constant values); no Rust compiler exists where it was written.
#![allow(non_camel_case_types)]
use std::os::raw::{c_char, c_int};

#[repr(C)] pub struct aqua_ctx { _p: [u8; 0] }
#[repr(C)] pub struct aqua_scene { _p: [u8; 0] }
#[repr(C)] pub struct aqua_nrc { _p: [u8; 0] }

pub type aqua_status = c_int;
pub const AQUA_OK: aqua_status = 0;
pub const AQUA_ERR_INVALID_ARG: aqua_status = 1;
pub const AQUA_ERR_IO: aqua_status = 2;
pub const AQUA_ERR_PARSE: aqua_status = 3;
pub const AQUA_ERR_MISSING_ASSET: aqua_status = 4;
pub const AQUA_ERR_CUDA: aqua_status = 5;
pub const AQUA_ERR_OOM: aqua_status = 6;
pub const AQUA_ERR_TIMEOUT: aqua_status = 7;
pub const AQUA_ERR_UNSUPPORTED: aqua_status = 8;

pub const AQUA_VERSION: c_int = 300;  // compare with aqua_version() at start-up
pub const AQUA_NRC_QUERY_SPREAD: i32 = -1;
pub const AQUA_BVH_AUTO: i32 = -1;
pub const AQUA_BVH_FULL: i32 = 0;
pub const AQUA_BVH_QUANTIZED: i32 = 1;
pub const AQUA_DEVICE_HOST_ONLY: i32 = -2;
pub const AQUA_TRACE_DEVICE_PTRS: u32 = 1 << 0;
pub const AQUA_TRACE_ANY_HIT: u32 = 1 << 1;
pub const AQUA_TRACE_COUNT: u32 = 1 << 2;
pub const AQUA_INTEGRATOR_PATH: i32 = 0;
pub const AQUA_INTEGRATOR_NRC: i32 = 1;
pub const AQUA_KERNEL_WAVEFRONT: i32 = 0;
pub const AQUA_KERNEL_PERSISTENT: i32 = 1;
pub const AQUA_RENDER_DEVICE_FILM: u32 = 1 << 0;
pub const AQUA_RENDER_STAGE_TIMING: u32 = 1 << 1;
pub const AQUA_RENDER_COUNT: u32 = 1 << 2;
pub const AQUA_RENDER_ACCUMULATE: u32 = 1 << 3;
pub const AQUA_LIGHT_QUAD: i32 = 0;
pub const AQUA_LIGHT_POINT: i32 = 1;
pub const AQUA_LIGHT_TRIANGLE: i32 = 2;
pub const AQUA_NRC_PARAMS: usize = 20672;
pub const AQUA_NRC_INPUTS: usize = 64;
pub const AQUA_NRC_RAW: usize = 16;
pub const AQUA_NRC_DEVICE_PTRS: u32 = 1 << 0;
pub const AQUA_NRC_TIMING: u32 = 1 << 1;
pub const AQUA_NRC_KERNEL_AUTO: i32 = 0;
pub const AQUA_NRC_KERNEL_MMA_SYNC: i32 = 1;
pub const AQUA_NRC_KERNEL_TCGEN05: i32 = 2;

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_options { pub device: i32, pub verbose: i32, pub fail_alloc_after: u64 }

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_ray {
    pub ox: f32, pub oy: f32, pub oz: f32, pub tmin: f32,
    pub dx: f32, pub dy: f32, pub dz: f32, pub tmax: f32,
}

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_hit { pub t: f32, pub u: f32, pub v: f32, pub prim: i32 }

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_trace_counts { pub node_visits: u64, pub tri_tests: u64, pub kernel_ms: f64 }

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_integrator_cfg {
    pub r#type: i32, pub spp: i32, pub max_depth: i32, pub rr_depth: i32,
    pub batch_size: i32, pub training_iters: i32, pub learning_rate: f32,
    pub visualize_cache: i32, pub seed: u64, pub spp_offset: i32,
    pub nrc_train_samples: i32, pub nrc_query_vertex: i32, pub row_begin: i32, pub row_step: i32,
    pub reserved0: i32,
}

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_tuning {
    pub slots: i32, pub block_trace: i32, pub block_shade: i32, pub sort_by_material: i32,
    pub blocks_per_sm: i32, pub use_graph: i32, pub iters_per_graph: i32, pub replicas: i32,
    pub kernel: i32,
}

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_stats {
    pub paths: u64, pub ext_rays: u64, pub shadow_rays: u64, pub iterations: u64,
    pub device_ms: f64, pub trace_ms: f64, pub shadow_ms: f64, pub shade_ms: f64,
    pub trace_launches: u64, pub shadow_launches: u64, pub shade_launches: u64,
    pub total_launches: u64, pub node_visits: u64, pub tri_tests: u64,
    pub shadow_node_visits: u64, pub shadow_tri_tests: u64, pub nrc_queries: u64,
    pub nrc_train_records: u64, pub nrc_ms: f64, pub nrc_loss: f64,
}

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_scene_info {
    pub width: i32, pub height: i32,
    pub num_triangles: i32, pub num_materials: i32, pub num_lights: i32, pub num_textures: i32,
    pub num_meshes: i32, pub num_bvh_nodes: i32, pub bvh_depth: i32, pub max_leaf_size: i32,
    pub device_bytes: u64, pub upload_bytes: u64, pub env: [f32; 3], pub bvh_format: i32,
}

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_camera {
    pub width: i32, pub height: i32, pub fov_deg: f32, pub lens_radius: f32, pub focal: f32,
    pub pos: [f32; 3], pub right: [f32; 3], pub up: [f32; 3], pub back: [f32; 3],
}

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_material {
    pub base_color: [f32; 3], pub base_texture: i32, pub metallic: f32, pub roughness: f32,
    pub specular: f32, pub specular_tint: f32, pub sheen: f32, pub sheen_tint: f32,
    pub clearcoat: f32, pub clearcoat_roughness: f32, pub transmission: f32, pub ior: f32,
    pub reserved: [i32; 2],
}

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_light {
    pub r#type: i32, pub p0: [f32; 3], pub e1: [f32; 3], pub e2: [f32; 3],
    pub radiance: [f32; 3], pub pmf: f32,
}

#[repr(C)] #[derive(Clone, Copy)]
pub struct aqua_job {
    pub scene: *mut aqua_scene, pub width: i32, pub height: i32, pub spp: i32,
    pub max_depth: i32, pub seed: u64, pub rgb_out: *mut f32,
}

#[repr(C)] #[derive(Clone, Copy)]
pub struct aqua_batch_stats { pub device_ms: f64, pub paths: u64, pub job_ms: *mut f64 }

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct aqua_nrc_cfg {
    pub learning_rate: f32, pub beta1: f32, pub beta2: f32, pub eps: f32, pub seed: u64,
    pub bbox_min: [f32; 3], pub bbox_max: [f32; 3], pub ema_decay: f32, pub forward_kernel: i32,
}

extern "C" {
    // lifetime
    pub fn aqua_create(out: *mut *mut aqua_ctx, opt: *const aqua_options) -> aqua_status;
    pub fn aqua_destroy(ctx: *mut aqua_ctx);
    pub fn aqua_last_error(ctx: *const aqua_ctx) -> *const c_char;
    pub fn aqua_status_string(s: aqua_status) -> *const c_char;
    pub fn aqua_version() -> c_int;

    // scenes
    pub fn aqua_load_scene_json(ctx: *mut aqua_ctx, path: *const c_char, allow_missing: i32,
                                out: *mut *mut aqua_scene) -> aqua_status;
    pub fn aqua_make_procedural_scene(ctx: *mut aqua_ctx, config_id: i32, seed: u64, width: i32,
                                      height: i32, out: *mut *mut aqua_scene) -> aqua_status;
    pub fn aqua_scene_free(ctx: *mut aqua_ctx, scene: *mut aqua_scene) -> aqua_status;
    pub fn aqua_scene_set_resolution(ctx: *mut aqua_ctx, scene: *mut aqua_scene, width: i32,
                                     height: i32) -> aqua_status;
    pub fn aqua_scene_upload(ctx: *mut aqua_ctx, scene: *mut aqua_scene) -> aqua_status;
    pub fn aqua_scene_get_info(ctx: *mut aqua_ctx, scene: *const aqua_scene,
                               out: *mut aqua_scene_info) -> aqua_status;
    pub fn aqua_scene_export_triangles(ctx: *mut aqua_ctx, scene: *const aqua_scene, verts: *mut f32,
                                       uvs: *mut f32, mat: *mut i32, light: *mut i32) -> aqua_status;
    pub fn aqua_scene_export_camera(ctx: *mut aqua_ctx, scene: *const aqua_scene,
                                    out: *mut aqua_camera) -> aqua_status;
    pub fn aqua_scene_export_materials(ctx: *mut aqua_ctx, scene: *const aqua_scene,
                                       out: *mut aqua_material) -> aqua_status;
    pub fn aqua_scene_export_lights(ctx: *mut aqua_ctx, scene: *const aqua_scene,
                                    out: *mut aqua_light) -> aqua_status;
    pub fn aqua_scene_export_texture(ctx: *mut aqua_ctx, scene: *const aqua_scene, i: i32,
                                     width: *mut i32, height: *mut i32, rgba: *mut u8) -> aqua_status;
    pub fn aqua_scene_export_normals(ctx: *mut aqua_ctx, scene: *const aqua_scene, nrm: *mut f32,
                                     present: *mut i32) -> aqua_status;
    pub fn aqua_scene_export_bvh(ctx: *mut aqua_ctx, scene: *const aqua_scene, nodes: *mut f32,
                                 tri_order: *mut i32) -> aqua_status;
    pub fn aqua_scene_export_bvh_quantized(ctx: *mut aqua_ctx, scene: *const aqua_scene,
                                           nodes: *mut f32) -> aqua_status;
    pub fn aqua_scene_set_bvh_format(ctx: *mut aqua_ctx, scene: *mut aqua_scene, format: i32) -> aqua_status;

    // assets and images (host-only contexts too)
    pub fn aqua_decode_jpeg(ctx: *mut aqua_ctx, data: *const u8, n: usize, width: *mut i32,
                            height: *mut i32, rgb: *mut u8) -> aqua_status;
    pub fn aqua_convert_obj(ctx: *mut aqua_ctx, obj_path: *const c_char, out_dir: *const c_char,
                            scene_name: *const c_char, width: i32, height: i32, meshes: *mut i32,
                            triangles: *mut i32) -> aqua_status;
    pub fn aqua_write_image(ctx: *mut aqua_ctx, path: *const c_char, rgb: *const f32, width: i32,
                            height: i32) -> aqua_status;

    // integrator settings
    pub fn aqua_load_integrator_json(ctx: *mut aqua_ctx, path: *const c_char,
                                     out: *mut aqua_integrator_cfg) -> aqua_status;
    pub fn aqua_integrator_defaults(out: *mut aqua_integrator_cfg);
    pub fn aqua_tuning_defaults(out: *mut aqua_tuning);

    // the hot path
    pub fn aqua_trace(ctx: *mut aqua_ctx, scene: *mut aqua_scene, rays: *const aqua_ray, n: usize,
                      out: *mut aqua_hit, flags: u32, counts: *mut aqua_trace_counts) -> aqua_status;
    pub fn aqua_render(ctx: *mut aqua_ctx, scene: *mut aqua_scene, cfg: *const aqua_integrator_cfg,
                       tuning: *const aqua_tuning, rgb_out: *mut f32, flags: u32,
                       stats: *mut aqua_stats) -> aqua_status;
    pub fn aqua_autotune(ctx: *mut aqua_ctx, scene: *mut aqua_scene, cfg: *const aqua_integrator_cfg,
                         out: *mut aqua_tuning) -> aqua_status;
    pub fn aqua_render_batch(ctx: *mut aqua_ctx, jobs: *const aqua_job, n: usize,
                             tuning: *const aqua_tuning, stats: *mut aqua_batch_stats) -> aqua_status;
    pub fn aqua_autotune_batch(ctx: *mut aqua_ctx, jobs: *const aqua_job, n: usize,
                               out: *mut aqua_tuning) -> aqua_status;
    pub fn aqua_workspace_bytes(ctx: *const aqua_ctx) -> u64;
    pub fn aqua_render_noalloc(ctx: *mut aqua_ctx, scene: *mut aqua_scene,
                               cfg: *const aqua_integrator_cfg, rgb_out_device: *mut f32,
                               stats: *mut aqua_stats) -> aqua_status;
    pub fn aqua_render_noalloc_max_pixels() -> u64;

    // radiance cache
    pub fn aqua_nrc_defaults(cfg: *mut aqua_nrc_cfg);
    pub fn aqua_nrc_create(ctx: *mut aqua_ctx, cfg: *const aqua_nrc_cfg,
                           out: *mut *mut aqua_nrc) -> aqua_status;
    pub fn aqua_nrc_destroy(ctx: *mut aqua_ctx, nrc: *mut aqua_nrc) -> aqua_status;
    pub fn aqua_nrc_set_weights(ctx: *mut aqua_ctx, nrc: *mut aqua_nrc, w: *const f32) -> aqua_status;
    pub fn aqua_nrc_get_weights(ctx: *mut aqua_ctx, nrc: *mut aqua_nrc, w: *mut f32) -> aqua_status;
    pub fn aqua_nrc_get_gradients(ctx: *mut aqua_ctx, nrc: *mut aqua_nrc, g: *mut f32) -> aqua_status;
    pub fn aqua_nrc_encode(ctx: *mut aqua_ctx, nrc: *mut aqua_nrc, raw: *const f32, n: usize,
                           x: *mut u16, flags: u32) -> aqua_status;
    pub fn aqua_nrc_forward(ctx: *mut aqua_ctx, nrc: *mut aqua_nrc, x: *const u16, n: usize,
                            out: *mut f32, flags: u32) -> aqua_status;
    pub fn aqua_nrc_last_ms(ctx: *mut aqua_ctx, nrc: *mut aqua_nrc, ms: *mut f32) -> aqua_status;
    pub fn aqua_nrc_train_step(ctx: *mut aqua_ctx, nrc: *mut aqua_nrc, x: *const u16,
                               target: *const f32, n: usize, loss: *mut f64,
                               flags: u32) -> aqua_status;
    pub fn aqua_render_nrc(ctx: *mut aqua_ctx, scene: *mut aqua_scene, cfg: *const aqua_integrator_cfg,
                           tuning: *const aqua_tuning, nrc: *mut aqua_nrc, rgb_out: *mut f32,
                           flags: u32, stats: *mut aqua_stats) -> aqua_status;
}
