"""ctypes binding of libaqua (include/aqua.h).

This is the Python side of the same C ABI a Rust ``extern "C"`` crate binds:
the structures mirror the header field for field, every call checks its
aqua_status and raises AquaError with the library's message. There is no
fallback: if libaqua.so is missing the import fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libaqua.so")

# ---------------------------------------------------------------- status codes
OK = 0
ERR_INVALID_ARG = 1
ERR_IO = 2
ERR_PARSE = 3
ERR_MISSING_ASSET = 4
ERR_CUDA = 5
ERR_OOM = 6
ERR_TIMEOUT = 7
ERR_UNSUPPORTED = 8

TRACE_DEVICE_PTRS = 1
TRACE_ANY_HIT = 2
TRACE_COUNT = 4

RENDER_DEVICE_FILM = 1
RENDER_STAGE_TIMING = 2
RENDER_COUNT = 4
RENDER_ACCUMULATE = 8

INTEGRATOR_PATH = 0
INTEGRATOR_NRC = 1

LIGHT_QUAD = 0
LIGHT_POINT = 1
LIGHT_TRIANGLE = 2


class AquaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"aqua status {status}: {message}")
        self.status = status
        self.message = message


# ---------------------------------------------------------------- structures
class Options(C.Structure):
    _fields_ = [("device", C.c_int32), ("verbose", C.c_int32), ("fail_alloc_after", C.c_uint64)]


class Ray(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("ox", "oy", "oz", "tmin", "dx", "dy", "dz", "tmax")]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("u", C.c_float), ("v", C.c_float), ("prim", C.c_int32)]


class TraceCounts(C.Structure):
    _fields_ = [("node_visits", C.c_uint64), ("tri_tests", C.c_uint64), ("kernel_ms", C.c_double)]


class IntegratorCfg(C.Structure):
    _fields_ = [("type", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32), ("rr_depth", C.c_int32),
                ("batch_size", C.c_int32), ("training_iters", C.c_int32), ("learning_rate", C.c_float),
                ("visualize_cache", C.c_int32), ("seed", C.c_uint64), ("spp_offset", C.c_int32),
                ("nrc_train_samples", C.c_int32), ("nrc_query_vertex", C.c_int32), ("row_begin", C.c_int32),
                ("row_step", C.c_int32), ("reserved0", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("slots", "block_trace", "block_shade", "sort_by_material",
                                         "blocks_per_sm", "use_graph", "iters_per_graph", "replicas", "kernel")]


KERNEL_WAVEFRONT, KERNEL_PERSISTENT = 0, 1
BVH_AUTO, BVH_FULL, BVH_QUANTIZED = -1, 0, 1
NRC_QUERY_SPREAD = -1


class Stats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("ext_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("iterations", C.c_uint64), ("device_ms", C.c_double), ("trace_ms", C.c_double),
                ("shadow_ms", C.c_double), ("shade_ms", C.c_double), ("trace_launches", C.c_uint64),
                ("shadow_launches", C.c_uint64), ("shade_launches", C.c_uint64), ("total_launches", C.c_uint64),
                ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64), ("shadow_node_visits", C.c_uint64),
                ("shadow_tri_tests", C.c_uint64), ("nrc_queries", C.c_uint64), ("nrc_train_records", C.c_uint64),
                ("nrc_ms", C.c_double), ("nrc_loss", C.c_double)]


class SceneInfo(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("num_triangles", C.c_int32),
                ("num_materials", C.c_int32), ("num_lights", C.c_int32), ("num_textures", C.c_int32),
                ("num_meshes", C.c_int32), ("num_bvh_nodes", C.c_int32), ("bvh_depth", C.c_int32),
                ("max_leaf_size", C.c_int32), ("device_bytes", C.c_uint64), ("upload_bytes", C.c_uint64),
                ("env", C.c_float * 3), ("bvh_format", C.c_int32)]


class Camera(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("fov_deg", C.c_float), ("lens_radius", C.c_float),
                ("focal", C.c_float), ("pos", C.c_float * 3), ("right", C.c_float * 3), ("up", C.c_float * 3),
                ("back", C.c_float * 3)]


class Material(C.Structure):
    _fields_ = [("base_color", C.c_float * 3), ("base_texture", C.c_int32), ("metallic", C.c_float),
                ("roughness", C.c_float), ("specular", C.c_float), ("specular_tint", C.c_float),
                ("sheen", C.c_float), ("sheen_tint", C.c_float), ("clearcoat", C.c_float),
                ("clearcoat_roughness", C.c_float), ("transmission", C.c_float), ("ior", C.c_float),
                ("reserved", C.c_int32 * 2)]


class Light(C.Structure):
    _fields_ = [("type", C.c_int32), ("p0", C.c_float * 3), ("e1", C.c_float * 3), ("e2", C.c_float * 3),
                ("radiance", C.c_float * 3), ("pmf", C.c_float)]


class Job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32),
                ("max_depth", C.c_int32), ("seed", C.c_uint64), ("rgb_out", C.c_void_p)]


class BatchStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("paths", C.c_uint64), ("job_ms", C.POINTER(C.c_double))]


# Every symbol include/aqua.h declares: (name, restype, argtypes).
_P = C.c_void_p
SIGNATURES = [
    ("aqua_create", C.c_int, [C.POINTER(_P), C.POINTER(Options)]),
    ("aqua_destroy", None, [_P]),
    ("aqua_last_error", C.c_char_p, [_P]),
    ("aqua_status_string", C.c_char_p, [C.c_int]),
    ("aqua_version", C.c_int, []),
    ("aqua_load_scene_json", C.c_int, [_P, C.c_char_p, C.c_int32, C.POINTER(_P)]),
    ("aqua_make_procedural_scene", C.c_int, [_P, C.c_int32, C.c_uint64, C.c_int32, C.c_int32, C.POINTER(_P)]),
    ("aqua_scene_free", C.c_int, [_P, _P]),
    ("aqua_scene_set_resolution", C.c_int, [_P, _P, C.c_int32, C.c_int32]),
    ("aqua_scene_upload", C.c_int, [_P, _P]),
    ("aqua_scene_get_info", C.c_int, [_P, _P, C.POINTER(SceneInfo)]),
    ("aqua_scene_export_triangles", C.c_int, [_P, _P, _P, _P, _P, _P]),
    ("aqua_scene_export_camera", C.c_int, [_P, _P, C.POINTER(Camera)]),
    ("aqua_scene_export_materials", C.c_int, [_P, _P, _P]),
    ("aqua_scene_export_lights", C.c_int, [_P, _P, _P]),
    ("aqua_scene_export_texture", C.c_int, [_P, _P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P]),
    ("aqua_scene_export_bvh", C.c_int, [_P, _P, _P, _P]),
    ("aqua_scene_export_bvh_quantized", C.c_int, [_P, _P, _P]),
    ("aqua_scene_set_bvh_format", C.c_int, [_P, _P, C.c_int32]),
    ("aqua_load_integrator_json", C.c_int, [_P, C.c_char_p, C.POINTER(IntegratorCfg)]),
    ("aqua_integrator_defaults", None, [C.POINTER(IntegratorCfg)]),
    ("aqua_tuning_defaults", None, [C.POINTER(Tuning)]),
    ("aqua_trace", C.c_int, [_P, _P, _P, C.c_size_t, _P, C.c_uint32, C.POINTER(TraceCounts)]),
    ("aqua_render", C.c_int, [_P, _P, C.POINTER(IntegratorCfg), C.POINTER(Tuning), _P, C.c_uint32,
                              C.POINTER(Stats)]),
    ("aqua_autotune", C.c_int, [_P, _P, C.POINTER(IntegratorCfg), C.POINTER(Tuning)]),
    ("aqua_render_batch", C.c_int, [_P, _P, C.c_size_t, C.POINTER(Tuning), C.POINTER(BatchStats)]),
    ("aqua_autotune_batch", C.c_int, [_P, _P, C.c_size_t, C.POINTER(Tuning)]),
    ("aqua_workspace_bytes", C.c_uint64, [_P]),
    ("aqua_render_noalloc", C.c_int, [_P, _P, C.POINTER(IntegratorCfg), _P, C.POINTER(Stats)]),
    ("aqua_render_noalloc_max_pixels", C.c_uint64, []),
    ("aqua_nrc_defaults", None, [_P]),
    ("aqua_nrc_create", C.c_int, [_P, _P, C.POINTER(_P)]),
    ("aqua_nrc_destroy", C.c_int, [_P, _P]),
    ("aqua_nrc_set_weights", C.c_int, [_P, _P, _P]),
    ("aqua_nrc_get_weights", C.c_int, [_P, _P, _P]),
    ("aqua_nrc_get_gradients", C.c_int, [_P, _P, _P]),
    ("aqua_nrc_encode", C.c_int, [_P, _P, _P, C.c_size_t, _P, C.c_uint32]),
    ("aqua_nrc_forward", C.c_int, [_P, _P, _P, C.c_size_t, _P, C.c_uint32]),
    ("aqua_nrc_last_ms", C.c_int, [_P, _P, C.POINTER(C.c_float)]),
    ("aqua_scene_export_normals", C.c_int, [_P, _P, _P, C.POINTER(C.c_int32)]),
    ("aqua_decode_jpeg", C.c_int, [_P, _P, C.c_size_t, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P]),
    ("aqua_convert_obj", C.c_int, [_P, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int32, C.c_int32,
                                   C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("aqua_write_image", C.c_int, [_P, C.c_char_p, _P, C.c_int32, C.c_int32]),
    ("aqua_nrc_train_step", C.c_int, [_P, _P, _P, _P, C.c_size_t, C.POINTER(C.c_double), C.c_uint32]),
    ("aqua_render_nrc", C.c_int, [_P, _P, C.POINTER(IntegratorCfg), C.POINTER(Tuning), _P, _P, C.c_uint32,
                                  C.POINTER(Stats)]),
]

NRC_PARAMS = 20672


class NrcCfg(C.Structure):
    _fields_ = [("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("seed", C.c_uint64), ("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3),
                ("ema_decay", C.c_float), ("forward_kernel", C.c_int32)]


NRC_KERNEL_AUTO, NRC_KERNEL_MMA_SYNC, NRC_KERNEL_TCGEN05 = 0, 1, 2


class Nrc:
    """The radiance cache's network (weights + Adam state) on the context's device."""

    def __init__(self, ctx: "Context", **over):
        self.ctx = ctx
        cfg = NrcCfg()
        ctx.lib.aqua_nrc_defaults(C.byref(cfg))
        for k, v in over.items():
            if k in ("bbox_min", "bbox_max"):
                getattr(cfg, k)[:] = list(v)
            else:
                setattr(cfg, k, v)
        h = C.c_void_p()
        ctx._check(ctx.lib.aqua_nrc_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h.value

    def free(self):
        if self.handle:
            self.ctx._check(self.ctx.lib.aqua_nrc_destroy(self.ctx.handle, self.handle))
            self.handle = None

    def weights(self) -> np.ndarray:
        w = np.zeros(NRC_PARAMS, np.float32)
        self.ctx._check(self.ctx.lib.aqua_nrc_get_weights(self.ctx.handle, self.handle, _ptr(w)))
        return w

    def set_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == NRC_PARAMS
        self.ctx._check(self.ctx.lib.aqua_nrc_set_weights(self.ctx.handle, self.handle, _ptr(w)))

    def gradients(self) -> np.ndarray:
        g = np.zeros(NRC_PARAMS, np.float32)
        self.ctx._check(self.ctx.lib.aqua_nrc_get_gradients(self.ctx.handle, self.handle, _ptr(g)))
        return g

    def encode(self, raw: np.ndarray) -> np.ndarray:
        raw = np.ascontiguousarray(raw, np.float32).reshape(-1, 16)
        x = np.zeros((raw.shape[0], 64), np.uint16)
        self.ctx._check(self.ctx.lib.aqua_nrc_encode(self.ctx.handle, self.handle, _ptr(raw), raw.shape[0],
                                                     _ptr(x), 0))
        return x

    def forward_device(self, x_ptr: int, n: int, out_ptr: int) -> float:
        """Inference on device buffers (x: n x 64 bf16, out: n x 3 fp32);
        returns the kernel's device milliseconds (CUDA events)."""
        self.ctx._check(self.ctx.lib.aqua_nrc_forward(self.ctx.handle, self.handle, C.c_void_p(x_ptr), n,
                                                      C.c_void_p(out_ptr), 3))
        ms = C.c_float()
        self.ctx._check(self.ctx.lib.aqua_nrc_last_ms(self.ctx.handle, self.handle, C.byref(ms)))
        return ms.value

    def encode_device(self, raw_ptr: int, n: int, x_ptr: int):
        self.ctx._check(self.ctx.lib.aqua_nrc_encode(self.ctx.handle, self.handle, C.c_void_p(raw_ptr), n,
                                                     C.c_void_p(x_ptr), 1))

    def train_step_device(self, x_ptr: int, target_ptr: int, n: int) -> float:
        """One Adam step on device buffers (x: n x 64 bf16, target: n x 3
        fp32); returns the step's device milliseconds (CUDA events)."""
        self.ctx._check(self.ctx.lib.aqua_nrc_train_step(self.ctx.handle, self.handle, C.c_void_p(x_ptr),
                                                         C.c_void_p(target_ptr), n, None, 3))
        ms = C.c_float()
        self.ctx._check(self.ctx.lib.aqua_nrc_last_ms(self.ctx.handle, self.handle, C.byref(ms)))
        return ms.value

    def forward(self, x_bf16: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x_bf16, np.uint16).reshape(-1, 64)
        out = np.zeros((x.shape[0], 3), np.float32)
        self.ctx._check(self.ctx.lib.aqua_nrc_forward(self.ctx.handle, self.handle, _ptr(x), x.shape[0],
                                                      _ptr(out), 0))
        return out

    def train_step(self, x_bf16: np.ndarray, target: np.ndarray) -> float:
        x = np.ascontiguousarray(x_bf16, np.uint16).reshape(-1, 64)
        t = np.ascontiguousarray(target, np.float32).reshape(-1, 3)
        loss = C.c_double()
        self.ctx._check(self.ctx.lib.aqua_nrc_train_step(self.ctx.handle, self.handle, _ptr(x), _ptr(t),
                                                         x.shape[0], C.byref(loss), 0))
        return loss.value

_lib = None


def load_library(path: str = LIB_PATH):
    """Loads libaqua.so and declares every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with aqua-engine_gb300/build.py")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Scene:
    def __init__(self, ctx: "Context", handle: int):
        self.ctx = ctx
        self.handle = handle

    def free(self):
        if self.handle:
            self.ctx._check(self.ctx.lib.aqua_scene_free(self.ctx.handle, self.handle))
            self.handle = None

    def info(self) -> SceneInfo:
        i = SceneInfo()
        self.ctx._check(self.ctx.lib.aqua_scene_get_info(self.ctx.handle, self.handle, C.byref(i)))
        return i

    def set_resolution(self, w: int, h: int):
        self.ctx._check(self.ctx.lib.aqua_scene_set_resolution(self.ctx.handle, self.handle, w, h))

    def upload(self):
        self.ctx._check(self.ctx.lib.aqua_scene_upload(self.ctx.handle, self.handle))

    def triangles(self):
        n = self.info().num_triangles
        v = np.zeros((n, 9), np.float32)
        uv = np.zeros((n, 6), np.float32)
        m = np.zeros(n, np.int32)
        li = np.zeros(n, np.int32)
        self.ctx._check(self.ctx.lib.aqua_scene_export_triangles(self.ctx.handle, self.handle, _ptr(v), _ptr(uv),
                                                                 _ptr(m), _ptr(li)))
        return v, uv, m, li

    def normals(self):
        """(n, 9) float32 vertex normals per triangle, or None for a flat-shaded scene."""
        present = C.c_int32()
        self.ctx._check(self.ctx.lib.aqua_scene_export_normals(self.ctx.handle, self.handle, None,
                                                               C.byref(present)))
        if not present.value:
            return None
        out = np.zeros((self.info().num_triangles, 9), np.float32)
        self.ctx._check(self.ctx.lib.aqua_scene_export_normals(self.ctx.handle, self.handle, _ptr(out),
                                                               C.byref(present)))
        return out

    def camera(self) -> Camera:
        c = Camera()
        self.ctx._check(self.ctx.lib.aqua_scene_export_camera(self.ctx.handle, self.handle, C.byref(c)))
        return c

    def materials(self):
        n = self.info().num_materials
        arr = (Material * max(n, 1))()
        self.ctx._check(self.ctx.lib.aqua_scene_export_materials(self.ctx.handle, self.handle, arr))
        return list(arr)[:n]

    def lights(self):
        n = self.info().num_lights
        arr = (Light * max(n, 1))()
        self.ctx._check(self.ctx.lib.aqua_scene_export_lights(self.ctx.handle, self.handle, arr))
        return list(arr)[:n]

    def texture(self, i: int) -> np.ndarray:
        w, h = C.c_int32(), C.c_int32()
        self.ctx._check(self.ctx.lib.aqua_scene_export_texture(self.ctx.handle, self.handle, i, C.byref(w),
                                                               C.byref(h), None))
        a = np.zeros((h.value, w.value, 4), np.uint8)
        self.ctx._check(self.ctx.lib.aqua_scene_export_texture(self.ctx.handle, self.handle, i, None, None,
                                                               _ptr(a)))
        return a

    def bvh_quantized(self) -> np.ndarray:
        """The quantized copy of the BVH, 16 floats per node."""
        inf = self.info()
        nodes = np.zeros((inf.num_bvh_nodes, 16), np.float32)
        self.ctx._check(self.ctx.lib.aqua_scene_export_bvh_quantized(self.ctx.handle, self.handle, _ptr(nodes)))
        return nodes

    def set_bvh_format(self, fmt: int):
        self.ctx._check(self.ctx.lib.aqua_scene_set_bvh_format(self.ctx.handle, self.handle, fmt))

    def bvh(self):
        """(nodes, tri_order): the four-wide BVH, 32 floats per node."""
        inf = self.info()
        nodes = np.zeros((inf.num_bvh_nodes, 32), np.float32)
        order = np.zeros(inf.num_triangles, np.int32)
        self.ctx._check(self.ctx.lib.aqua_scene_export_bvh(self.ctx.handle, self.handle, _ptr(nodes), _ptr(order)))
        return nodes, order


class Context:
    def __init__(self, device: int = -1, fail_alloc_after: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        opt = Options(device, 0, fail_alloc_after)
        st = self.lib.aqua_create(C.byref(h), C.byref(opt))
        if st != OK:
            raise AquaError(st, self.lib.aqua_last_error(None).decode())
        self.handle = h

    def _check(self, st: int):
        if st != OK:
            raise AquaError(st, self.lib.aqua_last_error(self.handle).decode("utf-8", "replace"))

    def close(self):
        if self.handle:
            self.lib.aqua_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # scenes
    def procedural(self, config: int, seed: int = 0, width: int = 0, height: int = 0) -> Scene:
        h = C.c_void_p()
        self._check(self.lib.aqua_make_procedural_scene(self.handle, config, seed, width, height, C.byref(h)))
        return Scene(self, h.value)

    def load_scene(self, path: str, allow_missing: bool = False) -> Scene:
        h = C.c_void_p()
        self._check(self.lib.aqua_load_scene_json(self.handle, path.encode(), 1 if allow_missing else 0,
                                                  C.byref(h)))
        return Scene(self, h.value)

    def integrator(self, path: str | None = None, **over) -> IntegratorCfg:
        c = IntegratorCfg()
        if path is None:
            self.lib.aqua_integrator_defaults(C.byref(c))
        else:
            self._check(self.lib.aqua_load_integrator_json(self.handle, path.encode(), C.byref(c)))
        for k, v in over.items():
            setattr(c, k, v)
        return c

    @staticmethod
    def tuning(**over) -> Tuning:
        t = Tuning()
        load_library().aqua_tuning_defaults(C.byref(t))
        for k, v in over.items():
            setattr(t, k, v)
        return t

    # hot path
    def trace(self, scene: Scene, rays: np.ndarray, any_hit: bool = False, count: bool = False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        out = np.zeros((n, 4), np.float32)
        cnt = TraceCounts()
        flags = (TRACE_ANY_HIT if any_hit else 0) | (TRACE_COUNT if count else 0)
        self._check(self.lib.aqua_trace(self.handle, scene.handle, _ptr(rays), n, _ptr(out), flags, C.byref(cnt)))
        t = out[:, 0].copy()
        u = out[:, 1].copy()
        v = out[:, 2].copy()
        prim = out[:, 3].copy().view(np.int32)
        return t, u, v, prim, cnt

    def render(self, scene: Scene, cfg: IntegratorCfg, tuning: Tuning | None = None, flags: int = 0,
               out: np.ndarray | None = None):
        inf = scene.info()
        if out is None:
            out = np.zeros((inf.height, inf.width, 3), np.float32)
        st = Stats()
        self._check(self.lib.aqua_render(self.handle, scene.handle, C.byref(cfg),
                                         C.byref(tuning) if tuning is not None else None, _ptr(out), flags,
                                         C.byref(st)))
        return out, st

    def render_nrc(self, scene: Scene, cfg: IntegratorCfg, nrc: "Nrc", tuning: Tuning | None = None, flags: int = 0,
                   out: np.ndarray | None = None, dev_ptr: int | None = None):
        """One frame of the cached renderer (host film, or a device film with dev_ptr)."""
        st = Stats()
        if dev_ptr is not None:
            target = C.c_void_p(dev_ptr)
            flags |= RENDER_DEVICE_FILM
        else:
            inf = scene.info()
            if out is None:
                out = np.zeros((inf.height, inf.width, 3), np.float32)
            target = _ptr(out)
        self._check(self.lib.aqua_render_nrc(self.handle, scene.handle, C.byref(cfg),
                                             C.byref(tuning) if tuning is not None else None, nrc.handle, target,
                                             flags, C.byref(st)))
        return out, st

    def render_device(self, scene: Scene, cfg: IntegratorCfg, dev_ptr: int, tuning: Tuning | None = None,
                      flags: int = 0):
        st = Stats()
        self._check(self.lib.aqua_render(self.handle, scene.handle, C.byref(cfg),
                                         C.byref(tuning) if tuning is not None else None, C.c_void_p(dev_ptr),
                                         flags | RENDER_DEVICE_FILM, C.byref(st)))
        return st

    def autotune(self, scene: Scene, cfg: IntegratorCfg) -> Tuning:
        t = Tuning()
        self._check(self.lib.aqua_autotune(self.handle, scene.handle, C.byref(cfg), C.byref(t)))
        return t

    def render_batch(self, jobs, tuning: Tuning | None = None):
        """jobs: list of (scene, width, height, spp, max_depth, seed, device_ptr).
        Returns (BatchStats, per-job completion ms)."""
        arr = (Job * len(jobs))()
        for i, (sc, w, h, spp, depth, seed, ptr) in enumerate(jobs):
            arr[i] = Job(sc.handle, w, h, spp, depth, seed, ptr)
        job_ms = (C.c_double * max(len(jobs), 1))()
        st = BatchStats(0.0, 0, job_ms)
        self._check(self.lib.aqua_render_batch(self.handle, arr, len(jobs),
                                               C.byref(tuning) if tuning is not None else None, C.byref(st)))
        return st, np.array(job_ms[:len(jobs)])

    def autotune_batch(self, jobs) -> Tuning:
        arr = (Job * len(jobs))()
        for i, (sc, w, h, spp, depth, seed, ptr) in enumerate(jobs):
            arr[i] = Job(sc.handle, w, h, spp, depth, seed, ptr)
        t = Tuning()
        self._check(self.lib.aqua_autotune_batch(self.handle, arr, len(jobs), C.byref(t)))
        return t

    def decode_jpeg(self, data: bytes) -> np.ndarray:
        """JPEG bytes -> (h, w, 3) uint8 RGB, row 0 at the top."""
        buf = np.frombuffer(data, np.uint8)
        w, h = C.c_int32(), C.c_int32()
        self._check(self.lib.aqua_decode_jpeg(self.handle, _ptr(buf), buf.size, C.byref(w), C.byref(h), None))
        out = np.zeros((h.value, w.value, 3), np.uint8)
        self._check(self.lib.aqua_decode_jpeg(self.handle, _ptr(buf), buf.size, C.byref(w), C.byref(h), _ptr(out)))
        return out

    def convert_obj(self, obj_path: str, out_dir: str, scene_name: str = "scene.json", width: int = 512,
                    height: int = 512):
        """OBJ + MTL -> BSON meshes + scene JSON in out_dir; returns (meshes, triangles)."""
        m, t = C.c_int32(), C.c_int32()
        self._check(self.lib.aqua_convert_obj(self.handle, obj_path.encode(), out_dir.encode(), scene_name.encode(),
                                              width, height, C.byref(m), C.byref(t)))
        return m.value, t.value

    def write_image(self, path: str, rgb: np.ndarray, width: int, height: int):
        rgb = np.ascontiguousarray(rgb, np.float32)
        assert rgb.size == width * height * 3
        self._check(self.lib.aqua_write_image(self.handle, path.encode(), _ptr(rgb), width, height))

    def workspace_bytes(self) -> int:
        return int(self.lib.aqua_workspace_bytes(self.handle))
