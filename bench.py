#!/usr/bin/env python
"""Benchmark: ms/frame of voxelize + mipmap + cone-trace at 1920x1080 with a
256^3 grid (6-direction anisotropic RGBA8 mips, 9 diffuse + 1 specular + 1
shadow cone per pixel) on a seeded synthetic scene: a closed box room (10
triangles) plus a noise-displaced geodesic icosphere of frequency 158
(499,280 triangles), one point light.

One step = one Renderer::render() frame.  ``value`` is the device time of
the voxelize + mip + trace stages (the metric's stages; the G-buffer raster is
reported next to it and included in ``ms_per_step``), timed with CUDA events
recorded on the renderer's stream; L2 is flushed (256 MB write) between timed
frames.  ``e2e`` is the same frame through the public C ABI as a user drives
it: host-side camera/model/light setup, render, and the read-back of the RGBA8
frame into pinned host memory, wall-clock timed.

``--impl reference`` times the CPU restatement of the reference's algorithm
(the oracle's FP32 instantiation, every host thread) on the same workload:
the reference itself is an OpenGL program that cannot run on these machines.

Multi-GPU: the path has no exchange step; N ranks render N independent
replicas of the frame (weak scaling), no collective on the data path.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/frame 1080p@256³ (voxelize+mip+trace)"
UNIT = "ms/frame"
WIDTH, HEIGHT, GRID = 1920, 1080, 256
SCENE_SEED = 2000
CPU_WARMUP_ROW_STRIDE = 64   # warm-up frames of the CPU arm trace every 64th row only
# Texture fetches per pixel of this frame that the texture-unit tracer
# issues, counted by the instrumented oracle (oracle.trace_stats over every
# 32nd row; checked by tests/test_scenes.py::test_bench_frame_work): 251.2
# cone-march steps per pixel by the reference's sample rule (778.9
# quadrilinear fetches: 3 per step, +1 level-0 fetch below lod 1); the engine
# skips the steps beyond the grid (exact early exit), the empty steps (exact
# empty-space skip), the maps whose anisotropic weight is exactly 0, and
# reads packed alpha-only chains for the shadow cones: 265.6 two-level
# (quadrilinear) and 83.5 one-level (trilinear) RGBA8 fetches per pixel when
# every pixel marches all its cones (far_share 0).  With shared far fields
# (far_share 1, the default: groups of 4x2 pixels march their diffuse cones
# after the first step once), counted over whole groups: 58.1 two-level and
# 25.9 one-level fetches per pixel.
TRACE_FETCHES_PER_PIXEL_REF = 778.9
TRACE_FETCH_QUAD_PER_PIXEL = 58.14
TRACE_FETCH_TRI_PER_PIXEL = 25.88
TRACE_FETCH_QUAD_PER_PIXEL_NOSHARE = 265.6
TRACE_FETCH_TRI_PER_PIXEL_NOSHARE = 83.5
INSTANCE_RECORD_BYTES = 144   # one per queued model (DevInstance)
STATUS_BYTES = 48             # per-frame status read back with the frame


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples around the timed region.

    The sampler starts before the warm-up and waits for nvidia-smi's first
    line (its start-up takes longer than a short timed region), then polls
    every ``interval_ms``; ``start()`` and
    ``stop()`` mark the timed region on the host clock, and the summary keeps
    the samples that arrived inside it (plus one polling interval after it,
    the sample taken while its last frame ran)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, interval_ms: int = 20):
        self.gpu = gpu_index
        self.interval = interval_ms
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            deadline = time.perf_counter() + 5.0   # first line before the warm-up starts
            while not self.lines and self.proc.poll() is None and time.perf_counter() < deadline:
                time.sleep(0.005)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def start(self):
        self.t0 = time.perf_counter()

    def stop(self):
        self.t1 = time.perf_counter()

    def __exit__(self, *a):
        if self.proc is not None:
            if self.t1 is not None:  # let the sample that covers the region's end arrive
                time.sleep(max(0.0, self.t1 + 3 * self.interval / 1000.0 - time.perf_counter()))
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lo = self.t0 if self.t0 is not None else float("-inf")
        hi = self.t1 + self.interval / 1000.0 if self.t1 is not None else float("inf")
        for t, ln in list(self.lines):
            if not lo <= t <= hi:
                continue
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm),
               "interval_ms": self.interval}
        if self.t0 is not None and self.t1 is not None:
            out["region_ms"] = round((self.t1 - self.t0) * 1000.0, 1)
        return out


def _scene():
    from voxel_cone_tracing_gb300 import scenes
    return scenes.scene_sphere(seed=SCENE_SEED, width=WIDTH, height=HEIGHT)


def _oracle_params(threads):
    from oracle import oracle as O
    return O.Params(grid_res=GRID, width=WIDTH, height=HEIGHT, threads=threads)


def cpu_frame_ms(scene, threads, row_stride=1):
    """FP32 CPU restatement of the frame: voxelize + mip + cone trace (of
    every row_stride-th pixel row; 1 = the whole frame).  -> (voxelize + mip
    + trace ms, per-stage ms)."""
    from oracle import oracle as O
    ms = O.time_frame(scene, _oracle_params(threads), row_stride)
    return ms[0] + ms[1] + ms[3], ms


CPU_SAMPLE = (f"FP32 C++ restatement of the whole frame: voxelize + mip of the {GRID}^3 grid and the cone trace "
              f"of all {WIDTH}x{HEIGHT} pixels, every step; host threads over triangle chunks, voxel slabs and "
              "32-pixel runs")


def bench_config(sampler: str, parallelism: str) -> dict:
    """The workload description both arms print (same keys, same workload)."""
    return {"workload": "room + displaced icosphere (499,290 triangles), 1920x1080, 256^3 aniso RGBA8, "
                        "9 diffuse + 1 specular + 1 shadow cone", "grid": GRID, "width": WIDTH, "height": HEIGHT,
            "triangles": 499290, "voxelizer": "reference raster 2x", "sampler": sampler,
            "l2": "flushed between timed frames (256 MB write)" if sampler == "texture unit" else "n/a (CPU)",
            "parallelism": parallelism}


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    scene = _scene()
    assert scene.n_tris == 499290
    for _ in range(max(args.warmup, 0)):
        cpu_frame_ms(scene, threads, CPU_WARMUP_ROW_STRIDE)
    vals, stages = [], []
    for _ in range(args.steps):
        v, ms = cpu_frame_ms(scene, threads, 1)
        vals.append(v)
        stages.append(ms)
    value = statistics.mean(vals)
    frame = statistics.mean(float(sum(st)) for st in stages)  # + the G-buffer raster
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(frame, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config("FP32 software", f"host threads x{threads}"),
        "stages_ms": {k: round(statistics.mean(st[i] for st in stages), 2)
                      for k, i in (("voxelize", 0), ("mipmap", 1), ("gbuffer", 2), ("trace", 3))},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": CPU_SAMPLE},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is an OpenGL 4.5 program (GLSL in the GL driver); no graphics stack exists on this "
                "box, so its algorithm is timed as the project's CPU restatement; warm-up frames trace every "
                f"{CPU_WARMUP_ROW_STRIDE}th row only",
    }
    print(json.dumps(line))
    return 0


def mlp_leg(r, R, scene, ids, stream, flush, steps, plain_stages, per_pixel_trace_ms=None):
    """Learned diffuse term: train on this frame's scene (2^24 cone-traced
    surface samples, 1000 Adam steps of 2^18), then time frames that
    evaluate the network instead of the nine diffuse cones (the judge checks
    1/256 of the pixels against their cones every frame), and compare the
    frame with the cone-traced one (RGBA8, PSNR).  Then move the light (as
    the injection leg does) and the camera, and report the network's PSNR
    against the cones there and what the judge decides."""
    import numpy as np
    import torch

    def frame(lights=None, view=None):
        if view is not None:
            r.set_camera_transform(view, scene.proj)
        for mid in ids:
            r.queue_model(mid)
        for l in (scene.lights if lights is None else lights):
            r.queue_point_light(l)
        r.render()

    def psnr(a, b):
        mse = float(np.mean((a[..., :3] - b[..., :3]) ** 2))
        return round(10 * np.log10(1.0 / mse), 2) if mse > 0 else None

    r.set_diffuse_mode(R.DIFFUSE_CONES)
    frame()
    ref = r.read_frame().astype(np.float64) / 255.0
    rep = r.mlp_train(R.mlp_desc())
    r.set_diffuse_mode(R.DIFFUSE_MLP)
    for _ in range(3):
        frame()
    r.synchronize()
    stages = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        frame()
        r.synchronize()
        stages.append(r.stage_times())
    got = r.read_frame().astype(np.float64) / 255.0
    judge = r.mlp_judge()
    # the same frames with the mma.sync warp-tile forward in place of the
    # warp-specialised tcgen05 one (the default)
    r.mlp_set_tensor_kernels(False)
    for _ in range(2):
        frame()
    sync_stages = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        frame()
        r.synchronize()
        sync_stages.append(r.stage_times())
    r.mlp_set_tensor_kernels(True)
    # generalisation: the light moved, then the camera moved
    moved = scene.lights.copy()
    moved["position"] = scene.lights["position"] + (0.06, 0.0, -0.03)
    from voxel_cone_tracing_gb300 import scenes as S
    view2 = S.look_at((0.12, 0.05, 0.48), (0.0, -0.05, -0.2))
    out = {}
    for name, kw in (("light_moved", dict(lights=moved)), ("camera_moved", dict(view=view2))):
        r.set_diffuse_mode(R.DIFFUSE_CONES)
        frame(**kw)
        cones = r.read_frame().astype(np.float64) / 255.0
        r.set_mlp_judge(0)
        r.set_diffuse_mode(R.DIFFUSE_MLP)
        frame(**kw)
        net = r.read_frame().astype(np.float64) / 255.0
        r.set_mlp_judge(8, 40.0)
        frame(**kw)
        j = r.mlp_judge()
        out[name] = {"psnr_db_vs_cones": psnr(net, cones), "judge_psnr_db": round(j["last_psnr_db"], 2),
                     "judge_fell_back": j["diffuse_mode"] == R.DIFFUSE_CONES}
    r.set_camera_transform(scene.view, scene.proj)
    r.set_diffuse_mode(R.DIFFUSE_CONES)
    trace_mlp = statistics.mean(s["trace"] for s in stages)
    trace_cones = statistics.mean(s["trace"] for s in plain_stages)
    value = statistics.mean(s["voxelize"] + s["mipmap"] + s["trace"] for s in stages)
    res = {"value": round(value, 4), "unit": UNIT, "trace_ms": round(trace_mlp, 4),
           "infer_ms": round(statistics.mean(s["infer"] for s in stages), 4),
           "forward": "tcgen05, warp-specialised",
           "trace_ms_mma_sync_forward": round(statistics.mean(s["trace"] for s in sync_stages), 4),
           "trace_ms_cones": round(trace_cones, 4), "trace_speedup": round(trace_cones / trace_mlp, 3),
           "psnr_db_vs_cones": psnr(got, ref),
           "judge": {"stride": judge["stride"], "min_psnr_db": judge["min_psnr_db"],
                     "last_psnr_db": round(judge["last_psnr_db"], 2), "fallbacks": judge["fallbacks"]},
           "after_training": out,
           "train": {"samples": rep["n_samples"], "steps": rep["steps"], "loss_first": rep["loss_first"],
                     "loss_last": rep["loss_last"], "ms_samples": round(rep["ms_samples"], 2),
                     "ms_train": round(rep["ms_train"], 2)}}
    if per_pixel_trace_ms:
        res["trace_ms_cones_per_pixel"] = round(per_pixel_trace_ms, 4)
        res["trace_speedup_vs_per_pixel_cones"] = round(per_pixel_trace_ms / trace_mlp, 3)
    return res


def per_pixel_leg(R, torch, scene, steps, flush):
    """The bench frame with every pixel marching all of its cones
    (far_share 0, the reference's rule): the exact-rule tracer's stages."""
    r = R.Renderer(WIDTH, HEIGHT, grid_res=GRID, far_share=0)
    ids = R.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    stream = torch.cuda.Stream()
    r.set_stream(stream.cuda_stream)
    for _ in range(3):
        R.queue_scene(r, scene, ids)
        r.render()
    r.synchronize()
    stages = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        R.queue_scene(r, scene, ids)
        r.render()
        r.synchronize()
        stages.append(r.stage_times())
    r.close()
    mean = lambda key: statistics.mean(st[key] for st in stages)  # noqa: E731
    return {"workload": "bench frame, every pixel marching all its cones (far_share 0)", "unit": UNIT,
            "value": round(mean("voxelize") + mean("mipmap") + mean("trace"), 4),
            "stages_ms": {k: round(mean(k), 4) for k in ("voxelize", "mipmap", "gbuffer", "trace")},
            "fetches": {"two_level_per_pixel": TRACE_FETCH_QUAD_PER_PIXEL_NOSHARE,
                        "one_level_per_pixel": TRACE_FETCH_TRI_PER_PIXEL_NOSHARE}}


def precision_leg(R, torch, steps, flush_mb=256):
    """Precision workload: 512^3 grid with RGBA16F maps (radiance clamped to
    [0, 16]), the conservative (exact SAT) voxelizer, 1,997,514 triangles
    (room + 4 displaced icospheres + 32 cuboids), 1080p.  Per-stage device
    times of `steps` frames (L2 flushed between frames); the per-stage error
    against the FP64 oracle is checked by tests/test_gpu_hdr.py."""
    from voxel_cone_tracing_gb300 import scenes
    scene = scenes.scene_hdr(width=WIDTH, height=HEIGHT)
    r = R.Renderer(WIDTH, HEIGHT, grid_res=512, storage=R.STORAGE_RGBA16F, radiance_max=scenes.HDR_RADIANCE_MAX,
                   vox_mode=R.VOX_CONSERVATIVE)
    ids = R.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    stream = torch.cuda.Stream()
    r.set_stream(stream.cuda_stream)
    flush = torch.empty(flush_mb << 20, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        R.queue_scene(r, scene, ids)
        r.render()
    r.synchronize()
    stages = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        R.queue_scene(r, scene, ids)
        r.render()
        r.synchronize()
        stages.append(r.stage_times())
    mean = lambda k: statistics.mean(st[k] for st in stages)  # noqa: E731
    out = {"workload": f"{scene.name} ({scene.n_tris} triangles), {WIDTH}x{HEIGHT}, 512^3 aniso RGBA16F, "
                       "radiance [0,16], conservative SAT voxelizer, 9 diffuse + 1 specular + 1 shadow cone",
           "value": round(mean("voxelize") + mean("mipmap") + mean("trace"), 4), "unit": UNIT,
           "stages_ms": {k: round(mean(k), 4) for k in ("voxelize", "mipmap", "gbuffer", "trace", "total")},
           "steps": steps, "gpu_launches": int(sum(st["kernel_launches"] for st in stages))}
    r.close()
    return out


def overlap_leg(R, torch, scene, steps, flush):
    """The bench frame with the G-buffer raster on a second stream beside
    voxelize and mipmap (vct_config.overlap_raster = 1): a shorter frame,
    but the overlapped stages slow each other down."""
    r = R.Renderer(WIDTH, HEIGHT, grid_res=GRID, overlap_raster=1)
    ids = R.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    stream = torch.cuda.Stream()
    r.set_stream(stream.cuda_stream)
    for _ in range(3):
        R.queue_scene(r, scene, ids)
        r.render()
    r.synchronize()
    stages, frame_ms = [], []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        R.queue_scene(r, scene, ids)
        r.render()
        e.record(stream)
        r.synchronize()
        stages.append(r.stage_times())
        frame_ms.append(s.elapsed_time(e))
    r.close()
    mean = lambda key: statistics.mean(st[key] for st in stages)  # noqa: E731
    return {"workload": "bench frame, G-buffer raster beside voxelize and mipmap", "unit": UNIT,
            "value": round(mean("voxelize") + mean("mipmap") + mean("trace"), 4),
            "frame_ms": round(statistics.mean(frame_ms), 4),
            "stages_ms": {k: round(mean(k), 4) for k in ("voxelize", "mipmap", "gbuffer", "trace")}}


def injection_leg(R, torch, scene, steps, flush):
    """Deferred light injection on the bench frame: the light moves every
    frame, the geometry does not, so frames after the first skip
    voxelization and light level 0 from the attribute grids."""
    r = R.Renderer(WIDTH, HEIGHT, grid_res=GRID)
    ids = R.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    r.set_light_injection(True)
    stream = torch.cuda.Stream()
    r.set_stream(stream.cuda_stream)
    base = scene.lights[0]

    def frame(k):
        for mid in ids:
            r.queue_model(mid)
        light = base.copy()
        light["position"] = base["position"] + (0.02 * (k % 5), 0.0, -0.01 * (k % 3))
        r.queue_point_light(light)
        r.render()

    frame(0)
    first = r.stage_times()
    for k in range(3):
        frame(k + 1)
    stages = []
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        frame(k + 4)
        r.synchronize()
        stages.append(r.stage_times())
    r.close()
    mean = lambda key: statistics.mean(st[key] for st in stages)  # noqa: E731
    return {"workload": "bench frame, light moved every frame, geometry fixed", "unit": UNIT,
            "value": round(mean("voxelize") + mean("mipmap") + mean("trace"), 4),
            "inject_ms": round(mean("voxelize"), 4), "voxelized_frames": sum(int(st["voxelized"]) for st in stages),
            "first_frame_voxelize_ms": round(first["voxelize"], 4),
            "stages_ms": {k: round(mean(k), 4) for k in ("voxelize", "mipmap", "gbuffer", "trace")}}


def batch_leg(R, torch, steps, rank=0, world=1, pg=None):
    """Batched workload: 64 seeded scenes of uneven size (grids 32^3-256^3,
    990-865k triangles, frames 256^2-1920x1080, 9 or 6 diffuse cones), one
    frame of all of them per step: every stage pass one launch over all
    scenes (the trace may be one launch per scene, if the autotuner finds
    that faster; `one_launch_per_stage` times the single-launch trace too),
    the frame captured once in a CUDA graph and replayed, launch shapes
    chosen by the autotuner, shared far fields as a Renderer's default.  Compared with the same 64 scenes rendered one after another by
    64 Renderers (same settings) on one stream.  With N ranks
    the scenes are split between them by cost (no data moves between
    GPUs); times are the max over ranks."""
    from voxel_cone_tracing_gb300 import replicas, scenes
    all_items = scenes.batch_scenes()
    items = replicas.my_scenes(all_items, rank, world)
    stream = torch.cuda.Stream()
    b = R.Batch(items, use_graph=True)
    b.set_stream(stream.cuda_stream)
    b.render()
    b.synchronize()
    tune = b.autotune(frames=2)
    for _ in range(2):
        b.render()
    b.synchronize()
    dev, wall, stages = [], [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        b.render()
        b.synchronize()
        wall.append((time.perf_counter() - t0) * 1e3)
        st = b.stage_times()
        stages.append(st)
        dev.append(st["total"])
    launches = stages[-1]["kernel_launches"]
    # the same batch with every stage one launch (the trace one CTA per tile
    # of every scene) instead of the tuned trace form
    b.shape = dict(b.shape, trace_per_scene=0, trace_ctas_per_sm=0)
    for _ in range(2):
        b.render()
    b.synchronize()
    one = []
    for _ in range(steps):
        b.render()
        b.synchronize()
        one.append(b.stage_times())
    one_launch = {"shape": b.shape, "value": round(statistics.mean(t["total"] for t in one), 3),
                  "trace_ms": round(statistics.mean(t["trace"] for t in one), 3),
                  "kernel_launches_per_frame": one[-1]["kernel_launches"]}
    b.close()
    # the same scenes, one Renderer each, rendered one after another
    rs = []
    for s, w, h, g, c in items:
        r = R.Renderer(w, h, grid_res=g, cone_set=c)
        ids = R.load_scene(r, s)
        r.set_voxel_view_dir(7, 0.0)
        r.set_stream(stream.cuda_stream)
        rs.append((r, s, ids))
    for r, s, ids in rs:
        R.queue_scene(r, s, ids)
        r.render()
    torch.cuda.synchronize()
    seq_wall, seq_dev, seq_launches, seq_stages = [], [], 0, []
    for _ in range(steps):
        t0 = time.perf_counter()
        for r, s, ids in rs:
            R.queue_scene(r, s, ids)
            r.render()
        for r, _, _ in rs:
            r.synchronize()
        seq_wall.append((time.perf_counter() - t0) * 1e3)
        sts = [r.stage_times() for r, _, _ in rs]
        seq_dev.append(sum(t["total"] for t in sts))
        seq_stages.append({k: sum(t[k] for t in sts) for k in ("voxelize", "mipmap", "gbuffer", "trace")})
        seq_launches = sum(t["kernel_launches"] for t in sts)
    for r, _, _ in rs:
        r.close()
    mean = lambda k: statistics.mean(st[k] for st in stages)  # noqa: E731
    dev_ms = replicas.job_time(statistics.mean(dev), pg, "cuda" if pg else None)
    seq_ms = replicas.job_time(statistics.mean(seq_wall), pg, "cuda" if pg else None)
    wall_ms = replicas.job_time(statistics.mean(wall), pg, "cuda" if pg else None)
    items = all_items
    return {"workload": f"{len(items)} scenes, {sum(it[0].n_tris for it in items)} triangles, "
                        f"{sum(it[1] * it[2] for it in items) / 1e6:.1f} Mpx per frame, grids 32^3-256^3, "
                        "6-9 diffuse cones", "unit": "ms/batch frame",
            "value": round(dev_ms, 3), "wall_ms": round(wall_ms, 3), "ranks": world,
            "stages_ms": {k: round(mean(k), 3) for k in ("voxelize", "mipmap", "gbuffer", "trace")},
            "kernel_launches_per_frame": launches, "autotune": tune, "one_launch_per_stage": one_launch,
            "sequential_renderers": {"device_ms": round(statistics.mean(seq_dev), 3),
                                     "stages_ms": {k: round(statistics.mean(s[k] for s in seq_stages), 3)
                                                   for k in ("voxelize", "mipmap", "gbuffer", "trace")},
                                     "wall_ms": round(statistics.mean(seq_wall), 3),
                                     "kernel_launches_per_frame": seq_launches},
            "speedup_wall": round(seq_ms / wall_ms, 3)}


def run_ours(args):
    rank, world, local = _dist()
    import numpy as np
    import torch

    import __graft_entry__ as ge
    from voxel_cone_tracing_gb300 import renderer as R

    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (the engine has no CPU path)")
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    ge.build()
    scene = _scene()
    r = R.Renderer(WIDTH, HEIGHT, grid_res=GRID)
    ids = R.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)  # the UI sets 7 unless the voxel view is on (main.cpp:300)
    stream = torch.cuda.Stream()
    r.set_stream(stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def frame():
        R.queue_scene(r, scene, ids)
        r.render()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stages = []
    with ClockSampler(local) as clk:
        for _ in range(max(args.warmup, 3)):
            frame()
        r.synchronize()
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        clk.start()
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()          # L2 flush, outside the timed pair
            starts[k].record(stream)
            frame()
            ends[k].record(stream)
            r.synchronize()
            stages.append(r.stage_times())
        torch.cuda.synchronize()
        clk.stop()
    if pg:
        pg.barrier()
    frame_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    vmt = [st["voxelize"] + st["mipmap"] + st["trace"] for st in stages]
    value = statistics.mean(vmt)
    ms_step = statistics.mean(frame_ms)
    if pg:
        t = torch.tensor([value, ms_step], device="cuda", dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        value, ms_step = float(t[0]), float(t[1])
    mean = lambda k: statistics.mean(st[k] for st in stages)  # noqa: E731

    # ---- end to end through the public API, host buffers -----------------
    host = torch.empty((HEIGHT, WIDTH, 4), dtype=torch.uint8, pin_memory=True).numpy()
    view, proj = np.asarray(scene.view, np.float32), np.asarray(scene.proj, np.float32)
    e2e_steps = args.steps
    r.synchronize()
    e2e_each = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        r.set_camera_transform(view, proj)
        for mid, model in zip(ids, scene.models):
            r.set_model_transform(mid, model)
        R.queue_scene(r, scene, ids)
        r.render()
        r.read_frame(R.FRAME_RGBA8, out=host)
        e2e_each.append((time.perf_counter() - t0) * 1000.0)
    # median over the steps: one host hiccup (another process, a page fault)
    # does not move it; the mean is reported beside it
    e2e_ms = statistics.median(e2e_each)
    e2e_mean = statistics.mean(e2e_each)
    h2d = len(ids) * INSTANCE_RECORD_BYTES  # lights and camera travel as kernel parameters
    d2h = WIDTH * HEIGHT * 4 + STATUS_BYTES

    # ---- roofline of the dominant kernel (cone trace) ----------------------
    # The trace reads its texels through the texture unit from L1 (the chain
    # fits in L2 and neighbouring cones share cache lines): its bound is the
    # texture unit's filtering rate, measured here on this device by
    # vct_measure_texture_rate (two-level and one-level 3D RGBA8 fetches,
    # every lane fetching, L1-resident).  The trace's fetches are counted by
    # the instrumented oracle; a one-level fetch is charged rate_quad/rate_tri
    # of a two-level one.  HBM is reported beside it.
    probe = {k: R.measure_texture_rate(k) for k in (0, 1, 2)}
    rate_quad, rate_tri = probe[0]["fetches_per_s"], probe[1]["fetches_per_s"]
    px = WIDTH * HEIGHT
    n_quad, n_tri = TRACE_FETCH_QUAD_PER_PIXEL * px, TRACE_FETCH_TRI_PER_PIXEL * px
    trace_ms = mean("trace")
    q_equiv = n_quad + n_tri * rate_quad / rate_tri
    achieved_tex = q_equiv / (trace_ms * 1e-3) / 1e9
    floor_ms = (n_quad / rate_quad + n_tri / rate_tri) * 1e3
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_clock_hz = (clk.summary().get("sm_mhz") or 2070.0) * 1e6
    per_clk_sm = lambda rate: round(rate / sm_clock_hz / sms, 3)  # noqa: E731
    peak, peak_kind = _peaks()
    nmaps_levels = sum((GRID >> l) ** 3 for l in range(1, 7)) * 6
    trace_bytes = px * (32 + 4) + (GRID ** 3 + nmaps_levels) * 4
    achieved_hbm = trace_bytes / (trace_ms * 1e-3) / 1e9
    traffic, tex_pct = None, None
    tp = os.path.join(ROOT, "profiles", "trace_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            prof = json.load(f)
        traffic, tex_pct = prof.get("dram_bytes_per_launch"), prof.get("tex_pipe_pct_of_peak")

    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(ms_step, 4), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config("texture unit", f"replicas x{world}"),
        "stages_ms": {"voxelize": round(mean("voxelize"), 4), "mipmap": round(mean("mipmap"), 4),
                      "gbuffer": round(mean("gbuffer"), 4), "trace": round(trace_ms, 4),
                      "frame": round(ms_step, 4)},
        "e2e": {"value": round(e2e_ms, 4), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "statistic": "median of per-step host wall times", "mean": round(e2e_mean, 4)},
        "gpu_launches": int(sum(st["kernel_launches"] for st in stages)),
        "roofline": {"kernel": "k_trace_share", "bound": "tex", "achieved": round(achieved_tex, 2),
                     "peak": round(rate_quad / 1e9, 2), "unit": "Gfetch/s", "frac": round(achieved_tex * 1e9 / rate_quad, 4),
                     "traffic": traffic, "peak_source": "measured in this run (vct_measure_texture_rate)",
                     "fetches": {"two_level_per_pixel": TRACE_FETCH_QUAD_PER_PIXEL,
                                 "one_level_per_pixel": TRACE_FETCH_TRI_PER_PIXEL,
                                 "per_pixel_cones": {"two_level_per_pixel": TRACE_FETCH_QUAD_PER_PIXEL_NOSHARE,
                                                     "one_level_per_pixel": TRACE_FETCH_TRI_PER_PIXEL_NOSHARE},
                                 "reference_rule_per_pixel": TRACE_FETCHES_PER_PIXEL_REF,
                                 "two_level_equivalents_per_frame": round(q_equiv),
                                 "unit": "3D RGBA8 texture fetches (achieved/peak in two-level equivalents)"},
                     "fetch_floor_ms": round(floor_ms, 4),
                     "probe": {"two_level_per_clk_per_sm": per_clk_sm(rate_quad),
                               "one_level_per_clk_per_sm": per_clk_sm(rate_tri),
                               "mip_integer_lod_per_clk_per_sm": per_clk_sm(probe[2]["fetches_per_s"]),
                               "sms": sms, "sm_mhz": sm_clock_hz / 1e6},
                     "trace_two_level_equivalents_per_clk_per_sm": per_clk_sm(q_equiv / (trace_ms * 1e-3)),
                     "ncu_tex_pipe_pct_of_peak": tex_pct,
                     "hbm": {"achieved": round(achieved_hbm, 2), "peak": peak, "unit": "GB/s",
                             "frac": round(achieved_hbm / peak, 5), "peak_source": peak_kind,
                             "algorithmic_bytes": trace_bytes}},
        "clocks": clk.summary(),
    }
    line["per_pixel_cones"] = per_pixel_leg(R, torch, scene, min(args.steps, 20), flush)
    if not args.no_mlp:
        line["mlp"] = mlp_leg(r, R, scene, ids, stream, flush, min(args.steps, 20), stages,
                              line["per_pixel_cones"]["stages_ms"]["trace"])
    line["overlap_raster"] = overlap_leg(R, torch, scene, min(args.steps, 20), flush)
    line["injection"] = injection_leg(R, torch, scene, min(args.steps, 20), flush)
    if not args.no_precision:
        line["precision"] = precision_leg(R, torch, min(args.steps, 20))
    if not args.no_batch:
        line["batch"] = batch_leg(R, torch, min(max(args.steps, 3), 10), rank, world, pg)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, ms = cpu_frame_ms(scene, threads, 1)
        line["cpu_baseline"] = {"value": round(v, 2), "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": CPU_SAMPLE + " (one frame)",
                                "stages_ms": {"voxelize": round(ms[0], 2), "mipmap": round(ms[1], 2),
                                              "trace": round(ms[3], 2)}}
    if rank == 0:
        print(json.dumps(line))
    r.close()
    if pg:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mlp", action="store_true", help="skip the learned-diffuse leg")
    ap.add_argument("--no-precision", action="store_true", help="skip the 512^3 RGBA16F HDR leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-scene batched leg")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
