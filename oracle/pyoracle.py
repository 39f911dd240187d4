"""ctypes wrapper of liboracle.so (test infrastructure only: used by tests/,
the smoke check and the benchmark's CPU baseline, never by the library).

`OracleScene.from_aqua(scene)` snapshots a libaqua scene through the C ABI's
export calls (triangles, BVH, materials, lights, textures, camera) so the
oracle sees exactly the data the device renders.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "aqua-engine_gb300"))
import aqua  # noqa: E402
import importlib.util  # noqa: E402

_spec = importlib.util.spec_from_file_location("aqua_oracle_build", os.path.join(HERE, "build.py"))
_oracle_build = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(_oracle_build)
_build = _oracle_build.build


class OrcScene(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("n_nodes", C.c_int32), ("tri_order", C.c_void_p), ("verts", C.c_void_p),
                ("uvs", C.c_void_p), ("tri_mat", C.c_void_p), ("tri_light", C.c_void_p), ("n_tris", C.c_int32),
                ("mats", C.c_void_p), ("n_mats", C.c_int32), ("lights", C.c_void_p), ("n_lights", C.c_int32),
                ("tex_rgba", C.c_void_p), ("tex_w", C.c_void_p), ("tex_h", C.c_void_p), ("n_tex", C.c_int32),
                ("cam", aqua.Camera), ("env", C.c_float * 3), ("nrm", C.c_void_p), ("qnodes", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.orc_trace_bvh_f32.argtypes = [P, P, C.c_int64, C.c_int, P, P, C.c_int]
        L.orc_trace_brute_f32.argtypes = [P, P, C.c_int64, C.c_int, P, C.c_int]
        L.orc_trace_brute_f64.argtypes = [P, P, C.c_int64, P, C.c_int]
        L.orc_render.argtypes = [P, C.c_int, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_int,
                                 C.c_int64, C.c_int64, P, P]
        L.orc_render.restype = C.c_int
        L.orc_render_cached.argtypes = [P, C.c_int, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                        C.c_int, C.c_int64, C.c_int64, C.c_int32, P, P, P]
        L.orc_render_cached.restype = C.c_int
        L.orc_render_pixels.argtypes = [P, C.c_int, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                        C.c_int, P, C.c_int64, P, P]
        L.orc_render_pixels.restype = C.c_int
        L.orc_bsdf_eval.argtypes = [P, C.c_int, P, P, C.c_int64, P, P]
        L.orc_bsdf_sample.argtypes = [P, C.c_int, P, P, C.c_int64, P]
        L.orc_srgb_to_linear.argtypes = [C.c_double]
        L.orc_srgb_to_linear.restype = C.c_double
        L.orc_pcg32_first.argtypes = [C.c_uint64, C.c_uint64, P, C.c_int]
        L.orc_pcg32_first.restype = C.c_uint32
        L.orc_mlp_forward.argtypes = [P, P, C.c_int64, C.c_int, P]
        L.orc_mlp_forward_f64.argtypes = [P, P, C.c_int64, C.c_int, P]
        L.orc_mlp_grad.argtypes = [P, P, P, C.c_int64, C.c_int, P, P]
        L.orc_nrc_encode.argtypes = [P, C.c_int64, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleScene:
    """Host snapshot of a scene in the oracle's layout (keeps arrays alive)."""

    def __init__(self):
        self.keep = []
        self.s = OrcScene()

    @classmethod
    def from_aqua(cls, scene) -> "OracleScene":
        o = cls()
        info = scene.info()
        verts, uvs, mat, light = scene.triangles()
        nodes, order = scene.bvh()
        mats = (aqua.Material * max(info.num_materials, 1))(*scene.materials())
        lights = (aqua.Light * max(info.num_lights, 1))(*scene.lights())
        texs = [np.ascontiguousarray(scene.texture(i)) for i in range(info.num_textures)]
        tex_ptrs = (C.c_void_p * max(len(texs), 1))(*[t.ctypes.data for t in texs])
        tw = np.array([t.shape[1] for t in texs] or [0], np.int32)
        th = np.array([t.shape[0] for t in texs] or [0], np.int32)
        o.keep = [verts, uvs, mat, light, nodes, order, mats, lights, texs, tex_ptrs, tw, th]
        s = o.s
        s.nodes, s.n_nodes = _p(nodes).value, nodes.shape[0]
        s.tri_order = _p(order).value
        s.verts, s.uvs, s.tri_mat, s.tri_light = _p(verts).value, _p(uvs).value, _p(mat).value, _p(light).value
        s.n_tris = verts.shape[0]
        s.mats, s.n_mats = C.cast(mats, C.c_void_p).value, info.num_materials
        s.lights, s.n_lights = C.cast(lights, C.c_void_p).value, info.num_lights
        s.tex_rgba, s.tex_w, s.tex_h, s.n_tex = C.cast(tex_ptrs, C.c_void_p).value, _p(tw).value, _p(th).value, len(texs)
        s.cam = scene.camera()
        for i in range(3):
            s.env[i] = info.env[i]
        if info.bvh_format == aqua.BVH_QUANTIZED:  # walk the nodes the device walks
            q = scene.bvh_quantized()
            o.keep.append(q)
            s.qnodes = _p(q).value
        nrm = scene.normals()
        if nrm is not None:
            o.keep.append(nrm)
            s.nrm = _p(nrm).value
        o.verts = verts
        o.width, o.height = info.width, info.height
        return o

    def set_resolution(self, w: int, h: int):
        self.s.cam.width = w
        self.s.cam.height = h
        self.width, self.height = w, h

    # -- traversal ---------------------------------------------------------
    def trace_bvh_f32(self, rays: np.ndarray, any_hit: bool = False, threads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.zeros((rays.shape[0], 4), np.float32)
        counts = np.zeros((rays.shape[0], 2), np.uint32)
        lib().orc_trace_bvh_f32(C.byref(self.s), _p(rays), rays.shape[0], int(any_hit), _p(hits), _p(counts),
                                threads)
        return hits[:, 0].copy(), hits[:, 1].copy(), hits[:, 2].copy(), hits[:, 3].copy().view(np.int32), counts

    def trace_brute_f32(self, rays: np.ndarray, any_hit: bool = False, threads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.zeros((rays.shape[0], 4), np.float32)
        lib().orc_trace_brute_f32(C.byref(self.s), _p(rays), rays.shape[0], int(any_hit), _p(hits), threads)
        return hits[:, 0].copy(), hits[:, 1].copy(), hits[:, 2].copy(), hits[:, 3].copy().view(np.int32)

    def trace_brute_f64(self, rays: np.ndarray, threads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.zeros((rays.shape[0], 4), np.float64)
        lib().orc_trace_brute_f64(C.byref(self.s), _p(rays), rays.shape[0], _p(hits), threads)
        return hits[:, 0].copy(), hits[:, 1].copy(), hits[:, 2].copy(), hits[:, 3].astype(np.int64)

    # -- rendering ---------------------------------------------------------
    def render(self, spp: int, max_depth: int, seed: int = 0, precision: int = 64, rr_depth: int = 3,
               spp_offset: int = 0, threads: int = 0, pixel_begin: int = 0, pixel_end: int | None = None,
               query_depth: int = -1, cache_rgb=None):
        n = self.width * self.height
        out = np.zeros((self.height, self.width, 3), np.float32)
        stats = np.zeros(3, np.float64)
        pe = n if pixel_end is None else pixel_end
        cache = None if cache_rgb is None else np.ascontiguousarray(cache_rgb, np.float32)
        r = lib().orc_render_cached(C.byref(self.s), precision, spp, spp_offset, max_depth, rr_depth, seed,
                                    threads, pixel_begin, pe, query_depth,
                                    None if cache is None else _p(cache), _p(out), _p(stats))
        if r != 0:
            raise RuntimeError("orc_render rejected its arguments")
        return out, stats

    def render_pixels(self, pixels, spp: int, max_depth: int, seed: int = 0, precision: int = 64,
                      rr_depth: int = 3, spp_offset: int = 0, threads: int = 0):
        """Renders the listed pixel indices; returns (len(pixels) x 3, stats)."""
        px = np.ascontiguousarray(pixels, np.uint32)
        out = np.zeros((px.shape[0], 3), np.float32)
        stats = np.zeros(3, np.float64)
        r = lib().orc_render_pixels(C.byref(self.s), precision, spp, spp_offset, max_depth, rr_depth, seed, threads,
                                    _p(px), px.shape[0], _p(out), _p(stats))
        if r != 0:
            raise RuntimeError("orc_render_pixels rejected its arguments")
        return out, stats

    def render_rows(self, rows, spp: int, max_depth: int, **kw):
        """Renders whole image rows; returns (len(rows) x width x 3, stats)."""
        rows = np.asarray(rows, np.int64)
        px = (rows[:, None] * self.width + np.arange(self.width)[None, :]).reshape(-1)
        out, st = self.render_pixels(px, spp, max_depth, **kw)
        return out.reshape(rows.shape[0], self.width, 3), st


def bsdf_eval(mat, wo, wi, front: bool = True):
    """f (n x 3) and pdf (n) of the Principled BSDF for direction pairs in the
    local frame; mat is an aqua.Material."""
    wo = np.ascontiguousarray(wo, np.float64).reshape(-1, 3)
    wi = np.ascontiguousarray(wi, np.float64).reshape(-1, 3)
    wo = np.broadcast_to(wo, wi.shape).copy() if wo.shape[0] == 1 else wo
    f = np.zeros(wi.shape, np.float64)
    p = np.zeros(wi.shape[0], np.float64)
    lib().orc_bsdf_eval(C.byref(mat), int(front), _p(wo), _p(wi), wi.shape[0], _p(f), _p(p))
    return f, p


def bsdf_sample(mat, wo, u, front: bool = True):
    """Sampled directions (n x 3) for n x 3 uniform numbers."""
    u = np.ascontiguousarray(u, np.float64).reshape(-1, 3)
    wo = np.ascontiguousarray(wo, np.float64).reshape(-1, 3)
    wo = np.broadcast_to(wo, u.shape).copy() if wo.shape[0] == 1 else wo
    wi = np.zeros(u.shape, np.float64)
    lib().orc_bsdf_sample(C.byref(mat), int(front), _p(wo), _p(u), u.shape[0], _p(wi))
    return wi


def srgb_to_linear(c: float) -> float:
    return lib().orc_srgb_to_linear(c)


def pcg32_sequence(initstate: int, initseq: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().orc_pcg32_first(initstate, initseq, _p(out), n)
    return out


NRC_PARAMS = 20672


def mlp_forward(w: np.ndarray, x: np.ndarray, emulate_bf16: bool = True) -> np.ndarray:
    w = np.ascontiguousarray(w, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 64)
    out = np.zeros((x.shape[0], 3), np.float32)
    lib().orc_mlp_forward(_p(w), _p(x), x.shape[0], int(emulate_bf16), _p(out))
    return out


def mlp_forward_f64(w: np.ndarray, x: np.ndarray, emulate_bf16: bool = False) -> np.ndarray:
    w = np.ascontiguousarray(w, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 64)
    out = np.zeros((x.shape[0], 3), np.float64)
    lib().orc_mlp_forward_f64(_p(w), _p(x), x.shape[0], int(emulate_bf16), _p(out))
    return out


def mlp_grad(w: np.ndarray, x: np.ndarray, target: np.ndarray, emulate_bf16: bool = True):
    w = np.ascontiguousarray(w, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 64)
    t = np.ascontiguousarray(target, np.float32).reshape(-1, 3)
    g = np.zeros(NRC_PARAMS, np.float64)
    loss = C.c_double()
    lib().orc_mlp_grad(_p(w), _p(x), _p(t), x.shape[0], int(emulate_bf16), _p(g), C.byref(loss))
    return g, loss.value


def nrc_encode(raw: np.ndarray, bmin, bmax) -> np.ndarray:
    raw = np.ascontiguousarray(raw, np.float32).reshape(-1, 16)
    bmin = np.ascontiguousarray(bmin, np.float32)
    bmax = np.ascontiguousarray(bmax, np.float32)
    x = np.zeros((raw.shape[0], 64), np.float32)
    lib().orc_nrc_encode(_p(raw), raw.shape[0], _p(bmin), _p(bmax), _p(x))
    return x


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    b = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def bf16_bits(a: np.ndarray) -> np.ndarray:
    return (bf16_round(a).view(np.uint32) >> 16).astype(np.uint16)


def bf16_to_float(bits: np.ndarray) -> np.ndarray:
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32)


def rel_mse(x: np.ndarray, ref: np.ndarray) -> float:
    """mean over pixels and channels of (x - r)^2 / (r^2 + 1e-2)."""
    x = x.astype(np.float64)
    r = ref.astype(np.float64)
    return float(np.mean((x - r) ** 2 / (r * r + 1e-2)))
