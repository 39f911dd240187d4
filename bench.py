"""Benchmark of the light-transport hot path.

Workload (one "step"): the procedural Cornell box with GGX materials
(roughness U[0.05,0.8], metallic {0,1} from seed 0), 1024 x 1024, 1024 spp,
max depth 8, per-pixel PCG32 streams, fp32 film — 1,073,741,824 camera paths
rendered by the wavefront kernels. Metric: Mpaths/s (higher is better).

Arms:
  default            libaqua on cuda:<local rank>; one JSON line from rank 0.
  --impl reference   the reference has no runnable CPU path (src/lib.rs is
                     empty), so the arm times the CPU oracle port (same
                     estimator, FP32, all host threads) on a bounded sample of
                     the same workload.

Under torchrun (--gpus N > 1) every rank renders its own replica of the
workload (the path shards by pixel with no exchange step), timing is the max
over ranks and `value` is the sum of all ranks' paths over that time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "aqua-engine_gb300"))

WORKLOAD = {"workload": "cornell-ggx-1024x1024-1024spp-depth8", "scene": "procedural Cornell box, GGX, seed 0",
            "width": 1024, "height": 1024, "spp": 1024, "max_depth": 8, "rr_depth": 3, "film": "fp32"}
METRIC = "Mpaths/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def cpu_sample_run(threads: int, target_s: float, seed: int = 0):
    """Oracle port (FP32, `threads` host threads) on every k-th row of the
    workload's image at full spp, k chosen for about target_s seconds, so the
    sample covers the image uniformly (walls, boxes, light and floor in their
    proportions); returns (Mpaths/s, seconds, description). The scene and its
    BVH come from libaqua's host-only loader; only the rendering is timed,
    and it is the oracle's."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import aqua
    import pyoracle

    hctx = aqua.Context(device=-2)
    scene = hctx.procedural(2, seed=0, width=WORKLOAD["width"], height=WORKLOAD["height"])
    orc = pyoracle.OracleScene.from_aqua(scene)
    W, H = WORKLOAD["width"], WORKLOAD["height"]
    kw = dict(seed=seed, precision=32, rr_depth=WORKLOAD["rr_depth"], threads=threads)
    # calibrate on 8 evenly spaced rows, then take every k-th row
    cal = list(range(H // 16, H, H // 8))
    t0 = time.perf_counter()
    orc.render_rows(cal, WORKLOAD["spp"], WORKLOAD["max_depth"], **kw)
    per_row = max(time.perf_counter() - t0, 1e-3) / len(cal)
    step = max(1, int(np.ceil(H * per_row / target_s)))
    rows = list(range(step // 2, H, step))
    t0 = time.perf_counter()
    _, st = orc.render_rows(rows, WORKLOAD["spp"], WORKLOAD["max_depth"], **kw)
    dt = time.perf_counter() - t0
    paths = float(st[0])
    scene.free()
    hctx.close()
    return paths / dt / 1e6, dt, f"one row in every {step} of the {W}x{H} image ({len(rows)} rows of {W} pixels, " \
                                  f"{WORKLOAD['spp']} spp each: {int(paths)} paths, {dt:.1f} s); scene and BVH " \
                                  f"built by libaqua's host-only loader, rendering by the oracle"


NRC_WORKLOAD = {"workload": "interior-1920x1080-1spp-per-frame-cache-vs-plain",
                "scene": "synthetic interior: 153 meshes, 1.15M triangles, 8 textures 2048^2, 16 quad lights, seed 0",
                "width": 1920, "height": 1080, "max_depth": 8, "rr_depth": 3, "frame_spp": 1,
                "train_records_per_frame": 65536, "batch": 16384, "learning_rate": 1e-2, "query_vertex": -1,
                "burn_in_frames": 16, "target_relmse": 1e-3, "ema_decay": 0.0, "plain_spp_per_call": 16,
                "reference_spp": 65536, "reference_rows": "rows 8, 24, ..., 1064 (every 16th row, 67 rows)",
                "error_rows": "the reference's rows: relMSE over every 16th row, an unbiased estimate of the "
                              "whole image's relMSE",
                "note": "cached renderer: 1 spp per 1920x1080 frame, online training on 65,536 records per frame "
                        "(Adam, lr 1e-2), queried where the path spread first exceeds 0.01 x the first-hit "
                        "footprint, at vertex >= 2 (query_vertex -1; fixed vertices 2..5 measured 0.67-0.87x), "
                        "frames after the burn-in averaged; plain: the wavefront path tracer at 16 spp per call; both render whole frames "
                        "and are timed by wall clock per call (error evaluation excluded)"}
REF_ROW_BEGIN, REF_ROW_STEP = 8, 16

_NRC_REF = {}


def nrc_reference(ctx, scene, W):
    """65,536-spp plain reference of every 16th row (row subset render, the
    same random-number streams as whole frames), cached per process."""
    import aqua
    import numpy as np

    key = (W["width"], W["height"], W["reference_spp"], W["max_depth"])
    if key not in _NRC_REF:
        rows = len(range(REF_ROW_BEGIN, W["height"], REF_ROW_STEP))
        acc = np.zeros((rows, W["width"], 3), np.float32)
        chunk = W["reference_spp"] // 16
        t0 = time.perf_counter()
        for k in range(16):
            ctx.render(scene, ctx.integrator(spp=chunk, max_depth=W["max_depth"], rr_depth=W["rr_depth"],
                                             seed=424242, spp_offset=k * chunk, row_begin=REF_ROW_BEGIN,
                                             row_step=REF_ROW_STEP), out=acc, flags=aqua.RENDER_ACCUMULATE)
        _NRC_REF[key] = (acc.astype(np.float64) / W["reference_spp"], time.perf_counter() - t0)
    return _NRC_REF[key]


def run_nrc_metric(ctx, budget_s: float = 90.0, runs: int = 3, overrides: dict | None = None):
    """Time to relMSE 1e-3 against a 65,536-spp plain reference, for the plain
    wavefront path tracer and for the cached renderer at 1 spp per 1080p
    frame (online training included in its time); `runs` runs per arm with
    different seeds, medians reported. Wall clock per render call; the error
    evaluation between calls (a device-to-host copy of the reference rows)
    is excluded."""
    import aqua
    import numpy as np
    import torch

    W = dict(NRC_WORKLOAD, **(overrides or {}))
    scene = ctx.procedural(3, seed=0, width=W["width"], height=W["height"])
    ref, t_ref = nrc_reference(ctx, scene, W)
    rows = torch.arange(REF_ROW_BEGIN, W["height"], REF_ROW_STEP, device="cuda")

    def rel_mse(film_rows, n):
        x = film_rows.double().cpu().numpy() / n
        return float(np.mean((x - ref) ** 2 / (ref * ref + 1e-2)))

    film = torch.zeros((W["height"], W["width"], 3), dtype=torch.float32, device="cuda")
    plain_runs, cached_runs = [], []
    for run in range(runs):
        # Plain: plain_spp_per_call spp per call, running sum on the device.
        film.zero_()
        torch.cuda.synchronize()
        spp, t, t_hit, e, curve = 0, 0.0, None, 1.0, []
        k = W["plain_spp_per_call"]
        while t < budget_s:
            t0 = time.perf_counter()
            ctx.render_device(scene, ctx.integrator(spp=k, max_depth=W["max_depth"], rr_depth=W["rr_depth"],
                                                    seed=7 + run, spp_offset=spp), film.data_ptr(),
                              flags=aqua.RENDER_ACCUMULATE)
            t += time.perf_counter() - t0
            spp += k
            e = rel_mse(film[rows], spp)
            if spp % 512 == 0:
                curve.append((spp, round(t, 3), e))
            if e <= W["target_relmse"]:
                t_hit = t
                break
        plain_runs.append({"time_s": t_hit, "spp": spp, "relmse": e, "curve": curve[-4:]})

        # Cached: 1 spp per frame with online training; frames after the
        # burn-in are summed on the device.
        net = aqua.Nrc(ctx, seed=1 + run, learning_rate=W["learning_rate"], ema_decay=W["ema_decay"])
        scratch = torch.zeros_like(film)
        film.zero_()
        torch.cuda.synchronize()
        frames, used, t, t_hit, e, curve, nrc_ms = 0, 0, 0.0, None, 1.0, [], 0.0
        while t < budget_s:
            burn = frames < W["burn_in_frames"]
            cfg = ctx.integrator(type=aqua.INTEGRATOR_NRC, spp=W["frame_spp"], max_depth=W["max_depth"],
                                 rr_depth=W["rr_depth"], seed=1000 * (run + 1) + frames,
                                 nrc_query_vertex=W["query_vertex"], nrc_train_samples=W["train_records_per_frame"],
                                 batch_size=W["batch"], training_iters=0)
            t0 = time.perf_counter()
            _, st = ctx.render_nrc(scene, cfg, net, dev_ptr=(scratch if burn else film).data_ptr(),
                                   flags=0 if burn else aqua.RENDER_ACCUMULATE)
            t += time.perf_counter() - t0
            nrc_ms += st.nrc_ms
            frames += 1
            if burn:
                continue
            used += 1
            if used % 16 == 0:
                e = rel_mse(film[rows], used * W["frame_spp"])
                if used % 256 == 0:
                    curve.append((frames, round(t, 3), e))
                if e <= W["target_relmse"]:
                    t_hit = t
                    break
        net.free()
        cached_runs.append({"time_s": t_hit, "frames": frames, "relmse": e, "mlp_ms_total": round(nrc_ms, 1),
                            "ms_per_frame": 1e3 * t / max(frames, 1), "curve": curve[-4:]})
    scene.free()

    def med(xs):
        xs = [x for x in xs if x is not None]
        return statistics.median(xs) if len(xs) == len(plain_runs) else None

    tp = med([r["time_s"] for r in plain_runs])
    tc = med([r["time_s"] for r in cached_runs])
    return {"config": W, "runs": runs, "reference_s": round(t_ref, 2),
            "plain": {"time_s_median": tp, "runs": plain_runs},
            "cached": {"time_s_median": tc, "runs": cached_runs},
            "time_ratio_cached_over_plain": (tc / tp) if (tc and tp) else None,
            "budget_s_per_run": budget_s}


def measure_l2_copy_gbs(device: int) -> dict:
    """L2-resident copy bandwidth: two buffers that fit in the 129 MB L2
    copied back and forth (read + write bytes), best of 20, CUDA events."""
    import torch

    best = {}
    for mb in (8, 16, 32):
        n = mb * (1 << 20) // 2
        a = torch.ones(n, dtype=torch.bfloat16, device=f"cuda:{device}")
        b = torch.empty_like(a)
        for _ in range(5):
            b.copy_(a)
        torch.cuda.synchronize()
        times = []
        for _ in range(20):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(10):
                b.copy_(a)
                a.copy_(b)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
        best[mb] = 20 * 2 * a.numel() * 2 / min(times) / 1e9
    return {"gbs": max(best.values()), "by_buffer_mb": best}


INTERIOR_WORKLOAD = {"workload": "interior-1920x1080-256spp-depth8", "width": 1920, "height": 1080, "spp": 256,
                     "max_depth": 8, "scene": "synthetic interior: 153 meshes, 1.15M triangles, 8 textures, "
                                              "16 quad lights, seed 0"}
SPHERES_WORKLOAD = {"workload": "sphere-field-1024x1024-64spp-depth8", "width": 1024, "height": 1024, "spp": 64,
                    "max_depth": 8, "scene": "random-sphere field: 4.0M triangles, seed 0"}
# DRAM bytes (read + write) of one full-queue k_trace_ext launch from ncu
# captures of these scenes, and the rays that launch traced.
TRACE_TRAFFIC = {
    "cornell": {"bytes": 849.785e6, "rays": 16777216,
                "source": "ncu capture of the first k_trace_ext launch of a 16-spp Cornell GGX 1024x1024 render at "
                          "the default queue depth (16 replicas: 16,777,216 camera rays; 604.5 MB read + 245.3 MB "
                          "written)"},
    "interior": {"bytes": 1212.296e6, "rays": 16588800,
                 "source": "ncu capture of the first k_trace_ext launch of a 16-spp 1080p interior render at the "
                           "default queue depth (8 replicas: 16,588,800 camera rays; 918.3 MB read + 293.9 MB "
                           "written; bounce-ray launches cost up to 1.4x more per ray)"},
    "spheres": {"bytes": 1943.945e6, "rays": 16777216,
                "source": "ncu capture of the first k_trace_ext launch of a 16-spp sphere-field render at the "
                          "default queue depth (16 replicas: 16,777,216 camera rays; 1668.6 MB read + 275.4 MB "
                          "written)"},
}


# Algorithmic bytes of k_shade: per shaded path it reads the queue entry
# (4 B), path state and throughput (32), hit (16), direction (16), triangle
# (48) and material (32) and writes the continued or restarted path (ray,
# throughput, state: 64) and its next-queue entry (4); per next-event
# estimate it writes a shadow record (48).
SHADE_BYTES_PER_PATH = 4 + 32 + 16 + 16 + 48 + 32 + 64 + 4
SHADOW_RECORD_BYTES = 48
# DRAM bytes of one full-queue k_shade launch from an ncu capture.
SHADE_TRAFFIC = {
    "cornell": {"bytes": 2636.587e6, "paths": 16777216,
                "source": "ncu capture of the first k_shade launch of a 16-spp Cornell GGX 1024x1024 render at the "
                          "default queue depth (16,777,216 camera-ray hits; 1162.1 MB read + 1474.5 MB written)"},
}


def trace_roofline(ctx, scene, cfg, film_ptr, hbm_peak, peak_src, l2_gbs, count_spp, traffic=None):
    """Roofline of k_trace_ext on one scene: algorithmic bytes per ray from a
    counting pass at count_spp (node visits x NODE_BYTES + triangle tests x
    48 + 48 B of ray and hit), times the rays per launch of a full render,
    over the mean launch time from CUDA events around every 8th launch of
    that render (RENDER_STAGE_TIMING; an extra render outside the timed
    steps)."""
    import aqua

    ccfg = ctx.integrator(spp=count_spp, max_depth=cfg.max_depth, rr_depth=cfg.rr_depth, seed=cfg.seed)
    cst = ctx.render_device(scene, ccfg, film_ptr, flags=aqua.RENDER_COUNT)
    bytes_per_ray = (cst.node_visits * NODE_BYTES + cst.tri_tests * 48) / max(cst.ext_rays, 1) + 48
    st = ctx.render_device(scene, cfg, film_ptr, flags=aqua.RENDER_STAGE_TIMING)
    rays_per_launch = st.ext_rays / max(st.iterations, 1)
    avg_launch_s = st.trace_ms * 1e-3 / max(st.trace_launches, 1)
    achieved = bytes_per_ray * rays_per_launch / avg_launch_s / 1e9
    out = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
           "peak_source": peak_src, "kernel": "k_trace_ext (closest-hit BVH traversal)",
           "bytes_per_ray": bytes_per_ray, "rays_per_launch": rays_per_launch,
           "avg_launch_us": avg_launch_s * 1e6, "frac_of_l2_copy": achieved / l2_gbs if l2_gbs else None,
           "node_visits_per_ray": cst.node_visits / max(cst.ext_rays, 1),
           "tri_tests_per_ray": cst.tri_tests / max(cst.ext_rays, 1), "counting_spp": count_spp,
           "traffic": None}
    if traffic:
        per_ray = traffic["bytes"] / traffic["rays"]
        out["traffic"] = per_ray * rays_per_launch
        out["traffic_note"] = (f"ncu DRAM bytes of a full-queue launch ({traffic['rays']} rays) scaled to this "
                               f"launch's mean ray count; {traffic['source']}")
        out["dram_gbs"] = out["traffic"] / avg_launch_s / 1e9
        out["dram_frac"] = out["dram_gbs"] / hbm_peak
    return out


def run_scene_metric(ctx, config_id: int, W: dict, hbm_peak: float, peak_src: str, l2_gbs: float,
                     warmup: int = 1, steps: int = 2, traffic=None):
    """Plain path tracing of one procedural scene (one step = the whole
    image), with the traversal roofline of that workload."""
    import torch

    scene = ctx.procedural(config_id, seed=0, width=W["width"], height=W["height"])
    film = torch.zeros(W["width"] * W["height"] * 3, dtype=torch.float32, device="cuda")
    cfg = ctx.integrator(spp=W["spp"], max_depth=W["max_depth"], rr_depth=3, seed=1)
    torch.cuda.synchronize()
    for _ in range(warmup):
        ctx.render_device(scene, cfg, film.data_ptr())
    ms, paths, rays = 0.0, 0, 0
    for _ in range(steps):
        torch.cuda.nvtx.range_push(f"scene{config_id}_step")
        st = ctx.render_device(scene, cfg, film.data_ptr())
        torch.cuda.nvtx.range_pop()
        ms += st.device_ms
        paths += st.paths
        rays += st.ext_rays + st.shadow_rays
    roof = trace_roofline(ctx, scene, cfg, film.data_ptr(), hbm_peak, peak_src, l2_gbs, count_spp=16,
                          traffic=traffic)
    info = scene.info()
    scene.free()
    return {"config": dict(W, triangles=info.num_triangles, bvh_nodes=info.num_bvh_nodes,
                           scene_device_mb=round(info.device_bytes / 1e6, 1)),
            "value": paths / (ms * 1e-3) / 1e6, "unit": "Mpaths/s", "mrays_per_s": rays / (ms * 1e-3) / 1e6,
            "ms_per_step": ms / steps, "steps": steps, "warmup": warmup, "roofline": roof}


NRC_INFER_WORKLOAD = {"workload": "nrc-inference-16777216-rows", "rows": 1 << 24,
                      "network": "64 -> 5 x 64 (ReLU) -> 3, bf16 operands, fp32 accumulation",
                      "inputs": "encoded from uniform random vertex features (positions in the unit box, "
                                "unit directions and normals, albedos), seed 21"}
NODE_BYTES = 112  # a four-wide node visit reads seven 16-byte words (its counts word is not read)
NRC_FLOP_PER_ROW = 2 * (5 * 64 * 64 + 3 * 64)  # 41,344 useful multiply-adds x 2
NRC_BYTES_PER_ROW = 128 + 12                   # bf16 input row + fp32 output


def run_nrc_inference_metric(ctx, bf16_peak: float, peak_src: str, warmup: int = 3, steps: int = 10,
                             rows: int = NRC_INFER_WORKLOAD["rows"]):
    """The cache's inference kernels alone on 16.8M encoded rows (2.1 GB of
    input, > L2): rows/s and the tensor roofline of the tcgen05 kernel, with
    the mma.sync kernel beside it. Device time from CUDA events on the
    library's stream."""
    import torch
    import aqua

    W = dict(NRC_INFER_WORKLOAD)
    n = W["rows"] = rows
    W["workload"] = f"nrc-inference-{rows}-rows"
    g = torch.Generator(device="cuda").manual_seed(21)
    raw = torch.rand((n, 16), generator=g, device="cuda", dtype=torch.float32)
    for sl in (slice(3, 6), slice(6, 9)):
        v = raw[:, sl] * 2 - 1
        raw[:, sl] = v / v.norm(dim=1, keepdim=True).clamp_min(1e-6)
    x = torch.empty((n, 64), dtype=torch.int16, device="cuda")
    out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    res = {}
    for name, kern in (("tcgen05", aqua.NRC_KERNEL_TCGEN05), ("mma_sync", aqua.NRC_KERNEL_MMA_SYNC)):
        net = aqua.Nrc(ctx, seed=3, bbox_min=[0, 0, 0], bbox_max=[1, 1, 1], forward_kernel=kern)
        net.encode_device(raw.data_ptr(), n, x.data_ptr())
        for _ in range(warmup):
            net.forward_device(x.data_ptr(), n, out.data_ptr())
        ms = [net.forward_device(x.data_ptr(), n, out.data_ptr()) for _ in range(steps)]
        net.free()
        t = sum(ms) / len(ms) * 1e-3
        res[name] = {"rows_per_s": n / t, "ms_per_launch": t * 1e3, "tflops": n * NRC_FLOP_PER_ROW / t / 1e12,
                     "gbs": n * NRC_BYTES_PER_ROW / t / 1e9}
    del raw, x, out
    tc = res["tcgen05"]
    return {"config": W, "unit": "Grows/s", "value": tc["rows_per_s"] / 1e9,
            "mma_sync_value": res["mma_sync"]["rows_per_s"] / 1e9, "steps": steps, "warmup": warmup,
            "kernels": res,
            "roofline": {"bound": "tensor", "achieved": tc["tflops"], "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": tc["tflops"] / bf16_peak, "peak_source": peak_src,
                         "kernel": "k_nrc_forward_tc (tcgen05 MLP inference)",
                         "flop_per_row": NRC_FLOP_PER_ROW, "hbm_bytes_per_row": NRC_BYTES_PER_ROW,
                         "hbm_gbs": tc["gbs"]}}


NRC_TRAIN_FLOP_PER_ROW = 3 * NRC_FLOP_PER_ROW  # forward + activation gradients + weight gradients


def run_nrc_training_metric(ctx, peak: float, peak_src: str, warmup: int = 5, steps: int = 20,
                            batches=(16384, 262144)):
    """One Adam step of the cache network (tcgen05 forward, backward and
    weight gradients, Adam) on `batch` device rows of random encoded inputs
    and targets: rows/s and the tensor roofline of the whole step (useful
    MLP FLOPs / step time / sustained bf16 peak). 16,384 rows is the cached
    renderer's batch; the larger batch shows the step when it is not
    launch-latency bound. Device time from CUDA events (AQUA_NRC_TIMING)."""
    import torch
    import aqua

    out = {}
    for batch in batches:
        g = torch.Generator(device="cuda").manual_seed(33)
        raw = torch.rand((batch, 16), generator=g, device="cuda", dtype=torch.float32)
        x = torch.empty((batch, 64), dtype=torch.int16, device="cuda")
        tgt = torch.rand((batch, 3), generator=g, device="cuda", dtype=torch.float32)
        net = aqua.Nrc(ctx, seed=4, bbox_min=[0, 0, 0], bbox_max=[1, 1, 1])
        net.encode_device(raw.data_ptr(), batch, x.data_ptr())
        for _ in range(warmup):
            net.train_step_device(x.data_ptr(), tgt.data_ptr(), batch)
        ms = [net.train_step_device(x.data_ptr(), tgt.data_ptr(), batch) for _ in range(steps)]
        net.free()
        t = statistics.median(ms) * 1e-3
        tflops = batch * NRC_TRAIN_FLOP_PER_ROW / t / 1e12
        out[str(batch)] = {"ms_per_step": t * 1e3, "rows_per_s": batch / t, "tflops": tflops,
                           "frac": tflops / peak}
        del raw, x, tgt
    big = out[str(batches[-1])]
    return {"config": {"workload": "nrc-train-step", "batches": list(batches),
                       "step": "forward (tcgen05) + backward (tcgen05) + weight gradients (tcgen05) + Adam",
                       "flop_per_row": NRC_TRAIN_FLOP_PER_ROW},
            "unit": "Mrows/s", "value": big["rows_per_s"] / 1e6, "steps": steps, "warmup": warmup, "by_batch": out,
            "roofline": {"bound": "tensor", "achieved": big["tflops"], "peak": peak, "unit": "TFLOP/s",
                         "frac": big["frac"], "peak_source": peak_src,
                         "kernel": f"one training step at {batches[-1]} rows (4 launches + weight packing)"}}


BATCH_WORKLOAD = {"workload": "batch-64-jobs-4-scenes",
                  "scenes": ["Cornell Lambert (36 tris)", "Cornell GGX (36 tris)",
                             "synthetic interior (1.15M tris, 8 textures)", "random-sphere field (4.0M tris)"],
                  "jobs": 64, "resolutions": [128, 256, 512, 1024], "spp_range": [16, 1024],
                  "spp_distribution": "log-uniform, seed 5", "max_depth": 8}


def run_batch_metric(ctx, warmup: int = 1, steps: int = 2, spp_div: int = 1):
    """64 jobs over 4 seeded scenes in one persistent launch per step:
    aggregate Mpaths/s and per-job completion latency p50/p99."""
    import numpy as np
    import torch

    W = BATCH_WORKLOAD
    t0 = time.perf_counter()
    scenes = [ctx.procedural(c, seed=0) for c in (1, 2, 3, 5)]
    t_scenes = time.perf_counter() - t0
    rng = np.random.default_rng(5)
    specs = []
    for i in range(W["jobs"]):
        res = int(rng.choice(W["resolutions"]))
        spp = int(round(np.exp(rng.uniform(np.log(16), np.log(1024)))))
        specs.append((int(rng.integers(0, 4)), res, res, max(1, spp // spp_div), W["max_depth"], 1000 + i))
    bufs = [torch.empty(r * r * 3, dtype=torch.float32, device="cuda") for (_, r, _, _, _, _) in specs]
    jobs = [(scenes[s], w, h, spp, d, seed, b.data_ptr()) for (s, w, h, spp, d, seed), b in zip(specs, bufs)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tune = ctx.autotune_batch(jobs)
    t_tune = time.perf_counter() - t0
    for _ in range(warmup):
        ctx.render_batch(jobs, tune)
    ms, paths, lat = 0.0, 0, []
    for _ in range(steps):
        torch.cuda.nvtx.range_push("batch_step")
        st, job_ms = ctx.render_batch(jobs, tune)
        torch.cuda.nvtx.range_pop()
        ms += st.device_ms
        paths += st.paths
        lat.extend(job_ms.tolist())
    for s in scenes:
        s.free()
    return {"config": W, "value": paths / (ms * 1e-3) / 1e6, "unit": "Mpaths/s", "ms_per_batch": ms / steps,
            "paths_per_batch": paths // steps, "job_latency_ms": {"p50": float(np.percentile(lat, 50)),
                                                                   "p99": float(np.percentile(lat, 99))},
            "tuning": {"block": tune.block_trace, "blocks_per_sm": tune.blocks_per_sm, "graph": tune.use_graph},
            "autotune_s": round(t_tune, 2), "scene_build_s": round(t_scenes, 2), "steps": steps, "warmup": warmup}


def run_reference(args, world, rank, pg):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample_run(threads, 1.0)
    vals, secs = [], []
    desc = ""
    for _ in range(args.steps):
        v, dt, desc = cpu_sample_run(threads, 10.0)
        vals.append(v)
        secs.append(dt)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (procedural scene, seeded)", "config": dict(WORKLOAD, parallelism="cpu threads"),
            "cpu_baseline": {"value": value, "unit": "Mpaths/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference crate has no implementation (src/lib.rs is empty); this arm times the CPU "
                    "oracle port of the same estimator; the scene and BVH are built by libaqua's host-only loader "
                    "(untimed) and only the rendering, the oracle's, is timed"}
    print(json.dumps(line), flush=True)


def run_gpu(args, world, rank, local, pg):
    import aqua

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    ctx = aqua.Context(device=local)
    scene = ctx.procedural(2, seed=0, width=WORKLOAD["width"], height=WORKLOAD["height"])
    info = scene.info()
    cfg = ctx.integrator(spp=WORKLOAD["spp"], max_depth=WORKLOAD["max_depth"], rr_depth=WORKLOAD["rr_depth"],
                         seed=1)
    tune = ctx.tuning()
    import torch

    torch.cuda.set_device(local)
    film = torch.zeros(info.width * info.height * 3, dtype=torch.float32, device=f"cuda:{local}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")  # > 129 MB L2
    torch.cuda.synchronize()

    # Untimed counting pass: node visits and triangle tests of this exact
    # workload (deterministic, so every timed step repeats them).
    cst = ctx.render_device(scene, cfg, film.data_ptr(), tune, flags=aqua.RENDER_COUNT)
    for _ in range(args.warmup):
        ctx.render_device(scene, cfg, film.data_ptr(), tune)

    barrier(pg)
    torch.cuda.synchronize()
    steps = []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_push("timed_step")
            steps.append(ctx.render_device(scene, cfg, film.data_ptr(), tune))
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    barrier(pg)
    ws_mb = ctx.workspace_bytes() / 1e6  # this workload's wavefront state, before the side runs grow it
    dev_ms = sum(s.device_ms for s in steps)
    ms_max = max_over_ranks(pg, dev_ms)
    paths = sum(s.paths for s in steps)
    all_paths = sum_over_ranks(pg, paths)
    value = all_paths / (ms_max * 1e-3) / 1e6

    # Rooflines of the two largest stages. Launch times come from one more
    # render of the same step with CUDA events around every 8th iteration's
    # launches (RENDER_STAGE_TIMING), run after the timed steps so the events
    # do not stretch them; `roofline` is the stage with the larger sampled time.
    flush.zero_()
    torch.cuda.synchronize()
    staged = ctx.render_device(scene, cfg, film.data_ptr(), tune, flags=aqua.RENDER_STAGE_TIMING)
    iters = max(staged.iterations, 1)
    rays_per_launch = staged.ext_rays / iters
    # Closest-hit traversal (k_trace_ext).
    ext = cst.ext_rays
    bytes_step = cst.node_visits * NODE_BYTES + cst.tri_tests * 48 + ext * (32 + 16)
    bytes_per_launch = bytes_step / max(cst.trace_launches, 1)
    avg_launch_s = staged.trace_ms * 1e-3 / max(staged.trace_launches, 1)
    achieved = bytes_per_launch / avg_launch_s / 1e9
    if args.traffic_per_launch > 0:
        traffic = args.traffic_per_launch
    else:  # the ncu DRAM bytes per ray of a full-queue launch, scaled to this launch's mean ray count
        tc = TRACE_TRAFFIC["cornell"]
        traffic = tc["bytes"] / tc["rays"] * rays_per_launch
    trace_roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                  "traffic": traffic, "rays_per_launch": rays_per_launch, "peak_source": peak_src,
                  "traffic_note": "ncu DRAM bytes per ray of a full-queue launch scaled to this launch's mean ray "
                                  "count; " + TRACE_TRAFFIC["cornell"]["source"],
                  "kernel": "k_trace_ext (closest-hit BVH traversal)",
                  "bytes_per_launch": bytes_per_launch, "avg_launch_us": avg_launch_s * 1e6,
                  "sampled_ms": staged.trace_ms,
                  "note": f"algorithmic bytes = node visits x {NODE_BYTES} B (four-wide node: six box words and the "
                          "child links) + triangle tests x 48 B + 48 B per ray; the Cornell BVH (8 nodes) is "
                          "cache-resident (L1/L2), so the algorithmic rate can pass the HBM copy rate while DRAM "
                          "traffic stays far below it"}
    # Shading (k_shade).
    sh_per_launch = staged.shadow_rays / iters
    shade_bytes = rays_per_launch * SHADE_BYTES_PER_PATH + sh_per_launch * SHADOW_RECORD_BYTES
    shade_s = staged.shade_ms * 1e-3 / max(staged.shade_launches, 1)
    shade_gbs = shade_bytes / shade_s / 1e9
    st_tr = SHADE_TRAFFIC.get("cornell")
    shade_roof = {"bound": "hbm", "achieved": shade_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": shade_gbs / hbm_peak,
                  "traffic": st_tr["bytes"] / st_tr["paths"] * rays_per_launch if st_tr else None,
                  "traffic_note": "ncu DRAM bytes per path of a full-queue launch scaled to this launch's mean path "
                                  "count; " + st_tr["source"] if st_tr else None,
                  "paths_per_launch": rays_per_launch, "peak_source": peak_src,
                  "kernel": "k_shade (emission, next-event estimation, BSDF sampling, roulette, path restart)",
                  "bytes_per_launch": shade_bytes, "avg_launch_us": shade_s * 1e6, "sampled_ms": staged.shade_ms,
                  "note": f"algorithmic bytes = {SHADE_BYTES_PER_PATH} B per shaded path (queue entry, path state, "
                          "hit, direction, triangle, material read; path state and next-queue entry written) + "
                          f"{SHADOW_RECORD_BYTES} B per shadow record written"}
    for r in (trace_roof, shade_roof):  # DRAM rate implied by the traffic figure
        if r["traffic"]:
            r["dram_gbs"] = r["traffic"] / (r["avg_launch_us"] * 1e-6) / 1e9
            r["dram_frac"] = r["dram_gbs"] / hbm_peak
    roofline = shade_roof if staged.shade_ms >= staged.trace_ms else trace_roof

    # End to end through the C ABI with host buffers: scene upload from
    # pinned host memory + render + film download every step, over the same
    # step count as `value` and with the same L2 flush before each step
    # (outside the timed stretch).
    host_film = None
    barrier(pg)
    e2e_s, e2e_paths = 0.0, 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        scene.upload()
        host_film, st = ctx.render(scene, cfg, tune, out=host_film)
        e2e_s += time.perf_counter() - t0
        e2e_paths += st.paths
    e2e_s = max_over_ranks(pg, e2e_s)
    e2e_value = sum_over_ranks(pg, e2e_paths) / e2e_s / 1e6

    l2 = measure_l2_copy_gbs(local)
    for r in (trace_roof, shade_roof):
        r["l2_copy_gbs"] = l2["gbs"]
        r["frac_of_l2_copy"] = r["achieved"] / l2["gbs"]
    interior = spheres = None
    if rank == 0 and not args.no_interior:
        interior = run_scene_metric(ctx, 3, INTERIOR_WORKLOAD, hbm_peak, peak_src, l2["gbs"],
                                    traffic=TRACE_TRAFFIC.get("interior"))
        spheres = run_scene_metric(ctx, 5, SPHERES_WORKLOAD, hbm_peak, peak_src, l2["gbs"],
                                   traffic=TRACE_TRAFFIC.get("spheres"))
    nrc = None
    if rank == 0 and not args.no_nrc and not args.no_nrc_time:
        nrc = run_nrc_metric(ctx, args.nrc_budget, args.nrc_runs)
    batch = None
    if rank == 0 and not args.no_batch:
        batch = run_batch_metric(ctx, spp_div=args.batch_spp_div)
        if args.batch_spp_div != 1:
            batch["config"] = dict(batch["config"], spp_divided_by=args.batch_spp_div)
    nrc_inf = None
    if rank == 0 and not args.no_nrc:
        bf16_peak = peaks.get("bf16_tflops", 1900.0)
        nrc_inf = run_nrc_inference_metric(ctx, bf16_peak, "measured (burst)" if "bf16_tflops" in peaks else "fallback",
                                           rows=args.nrc_rows)

    nrc_train = None
    if rank == 0 and not args.no_nrc:
        sus = peaks.get("bf16_tflops_sustained", 1700.0)
        nrc_train = run_nrc_training_metric(ctx, sus, "measured (sustained)" if "bf16_tflops_sustained" in peaks
                                            else "fallback")

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt, desc = cpu_sample_run(threads, args.cpu_seconds)
        cpu = {"value": v, "unit": "Mpaths/s", "cores": threads, "kind": "port", "sample": desc}

    gpu_launches = sum(s.total_launches for s in steps)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (procedural Cornell box, seeded)",
                "config": dict(WORKLOAD, parallelism=f"replicas x{world}",
                               l2="256 MB buffer zeroed before every timed step; wavefront state "
                                  f"{ws_mb:.0f} MB > 129 MB L2"),
                "mrays_per_s": sum_over_ranks(pg, sum(s.ext_rays + s.shadow_rays for s in steps)) /
                               (ms_max * 1e-3) / 1e6,
                "wall_s": wall, "clocks": clk.summary(), "roofline": roofline,
                "stage_rooflines": {"k_trace_ext": trace_roof, "k_shade": shade_roof}, "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": "Mpaths/s", "steps": args.steps,
                        "timing": "wall clock per step around scene upload + aqua_render + film download, "
                                  "L2 flushed before each step outside the timed stretch",
                        "h2d_bytes_per_step": int(info.upload_bytes),
                        "d2h_bytes_per_step": int(info.width * info.height * 12)},
                "gpu_launches": gpu_launches,
                "interior": interior,
                "sphere_field": spheres,
                "nrc_time_to_relmse": nrc,
                "nrc_inference": nrc_inf,
                "nrc_training": nrc_train,
                "batch": batch,
                "stage_ms_sampled": {"trace": staged.trace_ms, "shade": staged.shade_ms, "shadow": staged.shadow_ms,
                                     "note": "device ms of every 8th iteration's launches of one render of the "
                                             "step (RENDER_STAGE_TIMING), i.e. about 1/8 of each stage's time"}}
        print(json.dumps(line), flush=True)
    scene.free()
    ctx.close()


def run_profile_scene(args):
    """Profiling hook: one render of one procedural scene at its workload's
    resolution (config 2: the headline workload, 3: the interior, 5: the
    sphere field) with --spp samples, after 2 warm-up renders, inside the NVTX
    range "profile_scene". Prints nothing; for ncu captures on a small case."""
    import torch
    import aqua

    W = {2: WORKLOAD, 3: INTERIOR_WORKLOAD, 5: SPHERES_WORKLOAD}[args.profile_scene]
    ctx = aqua.Context(device=0)
    scene = ctx.procedural(args.profile_scene, seed=0, width=W["width"], height=W["height"])
    film = torch.zeros(W["width"] * W["height"] * 3, dtype=torch.float32, device="cuda")
    cfg = ctx.integrator(spp=args.spp or 4, max_depth=W["max_depth"], rr_depth=3, seed=1)
    for _ in range(2):
        ctx.render_device(scene, cfg, film.data_ptr())
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("profile_scene")
    ctx.render_device(scene, cfg, film.data_ptr())
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    scene.free()
    ctx.close()


def run_profile_cache_frame(args):
    """Profiling hook: the cached renderer on the config-4 workload (interior
    1920x1080, 1 spp per frame, online training): 20 warm-up frames, then one
    frame inside the NVTX range "cache_frame"; prints the frame's wall and
    network times."""
    import torch
    import aqua

    W = NRC_WORKLOAD
    ctx = aqua.Context(device=0)
    scene = ctx.procedural(3, seed=0, width=W["width"], height=W["height"])
    film = torch.zeros((W["height"], W["width"], 3), dtype=torch.float32, device="cuda")
    net = aqua.Nrc(ctx, seed=1, learning_rate=W["learning_rate"])
    cfg = lambda f: ctx.integrator(type=aqua.INTEGRATOR_NRC, spp=W["frame_spp"], max_depth=W["max_depth"],
                                   rr_depth=W["rr_depth"], seed=1000 + f, nrc_query_vertex=W["query_vertex"],
                                   nrc_train_samples=W["train_records_per_frame"], batch_size=W["batch"],
                                   training_iters=0)
    for f in range(20):
        ctx.render_nrc(scene, cfg(f), net, dev_ptr=film.data_ptr())
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("cache_frame")
    t0 = time.perf_counter()
    _, st = ctx.render_nrc(scene, cfg(20), net, dev_ptr=film.data_ptr())
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    torch.cuda.nvtx.range_pop()
    log(json.dumps({"frame_ms": wall * 1e3, "device_ms": st.device_ms, "nrc_ms": st.nrc_ms,
                    "iterations": st.iterations, "launches": st.total_launches, "queries": st.nrc_queries,
                    "records": st.nrc_train_records}))
    net.free()
    scene.free()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="aqua", choices=["aqua", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=13.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-nrc", action="store_true", help="skip both radiance-cache measurements")
    ap.add_argument("--no-nrc-time", action="store_true", help="skip the cached-vs-plain time-to-relMSE measurement")
    ap.add_argument("--nrc-rows", type=int, default=NRC_INFER_WORKLOAD["rows"],
                    help="rows of the cache-inference measurement (smaller only for profiling captures)")
    ap.add_argument("--nrc-budget", type=float, default=90.0, help="seconds per run and arm of that measurement")
    ap.add_argument("--nrc-runs", type=int, default=3, help="runs per arm of that measurement (median reported)")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-job batched-serving measurement")
    ap.add_argument("--batch-spp-div", type=int, default=1,
                    help="divide every batch job's spp by this (profiling captures only)")
    ap.add_argument("--no-interior", action="store_true", help="skip the 1080p interior measurement")
    # dram__bytes_read.sum + dram__bytes_write.sum of one full-queue
    # k_trace_ext launch (1M rays) of this workload, from `ncu --set full`
    # (40.53 MB read + 3.00 MB written, iteration 2 of a 16-spp render); every
    # launch of the step has the same queue size until the last samples drain.
    ap.add_argument("--traffic-per-launch", type=float, default=0.0,
                    help="DRAM bytes per k_trace_ext launch (default: the ncu figure per ray x rays per launch)")
    ap.add_argument("--spp", type=int, default=0,
                    help="samples per pixel of the workload (default 1024; smaller only for profiling captures)")
    ap.add_argument("--profile-scene", type=int, default=0, choices=[0, 2, 3, 5],
                    help="profiling hook: render one scene once (with --spp) and exit")
    ap.add_argument("--profile-cache-frame", action="store_true",
                    help="profiling hook: one cached-renderer frame of the config-4 workload, then exit")
    ap.add_argument("--profile-train", type=int, default=0,
                    help="profiling hook: time cache training steps on this many rows and exit")
    args = ap.parse_args()
    if args.profile_scene:
        run_profile_scene(args)
        return
    if args.profile_cache_frame:
        run_profile_cache_frame(args)
        return
    if args.profile_train:
        import aqua

        ctx = aqua.Context(device=0)
        r = run_nrc_training_metric(ctx, 1700.0, "fallback", warmup=2, steps=3, batches=(args.profile_train,))
        log(json.dumps(r["by_batch"]))
        ctx.close()
        return
    if args.spp > 0 and args.spp != WORKLOAD["spp"]:
        WORKLOAD["spp"] = args.spp
        WORKLOAD["workload"] = f"cornell-ggx-1024x1024-{args.spp}spp-depth8"
    if args.warmup < 3:
        log("warning: fewer than 3 warm-up steps")
    world, rank, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    else:
        run_gpu(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
