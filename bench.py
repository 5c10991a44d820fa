#!/usr/bin/env python3
"""Headline benchmark: frames/s of the fixed-function pipeline on one GB300.

Workload (default `batch`): 256 independent frames per step — sides log-uniform 64-1024,
triangle counts log-uniform 100-200k, each a lit UV sphere or a textured frame with ~30 %
clipped triangles (p = 1/2), with its own modelview, lights and 256x256 mipmapped texture —
rendered by one batched pipeline run (mtgl_batch_render: persistent tile kernel over all
frames, CUDA graph replay), and compared with the plain per-frame path on the same frames.
Other workloads: `textured` (1920x1080, 100k clip-straddling triangles, 512^2 trilinear
texture, 8 point lights, EXP fog), `rop` (1920x1080, 1M small blended triangles with
alpha, stencil and depth tests), `sphere` (800x600 lit UV sphere), `serve` (Poisson
requests at 2,000/s against 32 resident scenes through the C serving loop). Seeded
synthetic inputs (mytinygl_gb300/workloads.py), no dataset.

Lines printed (one JSON object each, rank 0 only):
  value        frames/s with inputs resident in device memory, timed with CUDA events on
               the stream the work runs on (the batch's, or the context's for single
               frames); L2 is flushed (a 256 MiB write on that stream) before every step.
  e2e          the same frames through the public C ABI with host inputs (client vertex
               arrays copied host->device every step) and every colour buffer read back,
               timed on the host clock; for the batch, with three steps in flight (three
               sets of contexts taking turns) and, as `sequential_value`, one at a time.
  roofline     the tile raster/ROP kernel (K4): compulsory bytes per launch over its mean
               launch time (CUDA events inside the library), against the measured HBM copy peak.
  cpu_baseline the CPU oracle (a restatement of MyTinyGL's renderer) on all host cores, one
               context per thread, on a bounded sample of the same workload.
--impl reference times that CPU implementation as the measured arm.
Several GPUs run independent replicas (one process per GPU, no collective on the data path).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

from mytinygl_gb300 import gl as G  # noqa: E402
from mytinygl_gb300 import workloads as W  # noqa: E402

WORKLOADS = {
    "textured": dict(builder=W.textured_scene, full_tris=100_000, name="textured_clip_fog_1920x1080_100k",
                     desc="1920x1080, 100k triangles (~30% clipped), 512^2 trilinear texture, 8 point lights, EXP fog"),
    "rop": dict(builder=W.rop_scene, full_tris=1_000_000, name="rop_blend_stencil_1920x1080_1M",
                desc="1920x1080, 1M small triangles, blend + alpha test + stencil INCR + depth LEQUAL, no depth writes"),
    "sphere": dict(builder=W.sphere_scene, full_tris=1984, name="sphere_lit_800x600_1984",
                   desc="800x600 UV sphere (1,984 triangles), directional light, GL_LESS, back-face culling"),
}
WORKLOADS["batch"] = dict(builder=None, full_tris=None, name="uneven_batch_256_frames",
                          desc=("256 independent frames, sides log-uniform 64-1024, triangles log-uniform "
                                "100-200k, each a lit UV sphere or a clip-straddling textured frame (p=1/2) "
                                "with its own modelview, lights and 256^2 mipmapped texture; seed 3"))
WORKLOADS["serve"] = dict(builder=None, full_tris=None, name="serve_32_scenes_poisson_2000",
                          desc=("serving loop: 32 resident scenes (1k-500k triangles like the textured frame, "
                                "256^2-2048^2 mipmapped textures), Poisson arrivals at 2,000 req/s, resolution "
                                "uniform over 256^2, 512^2, 1280x720, 1920x1080, modelview from the request "
                                "seed, 40 GiB framebuffer + pipeline-scratch budget"))
REC_BYTES = 224  # triangle record written by the setup kernel, read by the tile kernel
BATCH_FRAMES = 256  # frames per step of the batch workload (--frames changes it for profiling)
E2E_SETS = 3  # context sets the end-to-end batch measurement keeps in flight


class Timings(ctypes.Structure):
    _fields_ = [("vertex_ms", ctypes.c_double), ("setup_ms", ctypes.c_double), ("bin_ms", ctypes.c_double),
                ("tile_ms", ctypes.c_double), ("passes", ctypes.c_uint64)]


def bind_extras(lib):
    L = lib.lib
    L.mtgl_set_profiling.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.mtgl_set_profiling.restype = ctypes.c_int
    L.mtgl_get_timings.argtypes = [ctypes.c_void_p, ctypes.POINTER(Timings)]
    L.mtgl_get_timings.restype = ctypes.c_int
    L.mtgl_cuda_stream.argtypes = [ctypes.c_void_p]
    L.mtgl_cuda_stream.restype = ctypes.c_void_p
    L.mtgl_set_option.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    L.mtgl_set_option.restype = ctypes.c_int


MTGL_OPT_DEPTH_REJECTION = 1


def covered_fragments(lib, scene, fs):
    """Covered fragments of one frame (the F the reference runs through its per-pixel
    pipeline), counted in an untimed frame with the tile kernel's depth rejection off."""
    ctx = lib.context(scene.width, scene.height)
    lib.lib.mtgl_set_option(ctx.handle, MTGL_OPT_DEPTH_REJECTION, 0)
    scene.play(ctx, 0, fs)
    ctx.glFinish()
    lib.lib.mtgl_reset_stats(ctx.handle)
    scene.play(ctx, fs)
    frags = get_stats(ctx)["fragments"]
    ctx.destroy()
    return frags


def get_stats(ctx):
    s = G.Stats()
    assert ctx.glib.lib.mtgl_get_stats(ctx.handle, ctypes.byref(s)) == 0
    return {k: int(getattr(s, k)) for k, _ in G.Stats._fields_}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(workload):
    """DRAM bytes per K4 launch from the committed ncu summary, if one exists for the workload."""
    path = os.path.join(REPO, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and parts[0] == workload and parts[1] == "k_tile":
            return float(parts[2])
    return None


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def scene_bytes(scene, start):
    """Bytes of client arrays the frame part passes by pointer (host->device per frame)."""
    total = 0
    for name, args in scene.cmds[start:]:
        for a in args:
            if isinstance(a, np.ndarray) and name.endswith("Pointer"):
                total += a.nbytes
    return total


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, device="cuda"):
    """The largest x over the ranks of the process group (x itself without one)."""
    import torch

    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(units, seconds, device="cuda"):
    """Whole-job throughput of replicas: each of the world's ranks processes `units` in its
    own `seconds`; the job takes as long as its slowest rank."""
    import torch

    world = 1
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        world = torch.distributed.get_world_size()
    return world * units / max_over_ranks(seconds, device)


def run_ours(args, spec):
    import torch

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import mytinygl_gb300 as M

    M.build()
    lib = M.library()
    bind_extras(lib)

    # ---- device-resident frames (value)
    scene = spec["builder"](use_vbo=True)
    fs = W.frame_start(scene)
    ctx = lib.context(scene.width, scene.height)
    scene.play(ctx, 0, fs)
    for _ in range(args.warmup):
        scene.play(ctx, fs)
        ctx.glFinish()
    stream_ptr = ctx.glib.lib.mtgl_cuda_stream(ctx.handle)
    ext = torch.cuda.ExternalStream(stream_ptr)
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ctx.glib.lib.mtgl_reset_stats(ctx.handle)
    ctx.glib.lib.mtgl_set_profiling(ctx.handle, 1)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ctx.glFinish()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for i in range(args.steps):
            with torch.cuda.stream(ext):
                flush_buf.zero_()
                starts[i].record(ext)
            scene.play(ctx, fs)
            ctx.glFlush()
            ends[i].record(ext)
        ctx.glFinish()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(step_ms)
    st = get_stats(ctx)
    tm = Timings()
    ctx.glib.lib.mtgl_get_timings(ctx.handle, ctypes.byref(tm))
    ctx.glib.lib.mtgl_set_profiling(ctx.handle, 0)
    fps = job_rate(args.steps, total_ms / 1e3)
    tested_per_frame = st["fragments"] / args.steps
    ctx.destroy()
    frags_per_frame = covered_fragments(lib, scene, fs)

    # ---- roofline of K4 (tile raster/ROP)
    peak, peak_src = measured_peaks()
    npix = scene.width * scene.height
    tex_bytes = 0
    for name, a in scene.cmds:
        if name == "glTexImage2D":
            w, h = int(a[3]), int(a[4])
            tex_bytes += 4 * (w * h + (w // 2) * (h // 2))
    rec = st["setup_triangles"] / args.steps
    pairs = st["bin_entries"] / args.steps
    k4_bytes = npix * 9 + pairs * 4 + rec * REC_BYTES + tex_bytes
    k4_ms = tm.tile_ms / max(1, tm.passes)
    achieved = k4_bytes / (k4_ms / 1e3) / 1e9 if k4_ms > 0 else None
    traffic = ncu_traffic(spec["name"])

    # ---- end to end through the C ABI with client arrays and readback (e2e)
    escene = spec["builder"](use_vbo=False)
    efs = W.frame_start(escene)
    ectx = lib.context(escene.width, escene.height)
    escene.play(ectx, 0, efs)
    host = torch.empty((escene.height, escene.width), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    for _ in range(args.warmup):
        escene.play(ectx, efs)
        ectx.read(color=True, depth=False, stencil=False)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        escene.play(ectx, efs)
        ectx.glib.lib.mtgl_read_framebuffer(ectx.handle, host.ctypes.data, None, None)
    e2e_s = time.perf_counter() - t0
    ectx.destroy()
    e2e_fps = job_rate(args.steps, e2e_s)
    h2d = scene_bytes(escene, efs)
    d2h = escene.width * escene.height * 4

    out = {
        "metric": "frames/s",
        "value": round(fps, 3),
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded; mytinygl_gb300/workloads.py)",
        "config": {"workload": spec["name"], "description": spec["desc"], "width": scene.width,
                   "height": scene.height, "input_triangles": int(st["input_triangles"] / args.steps),
                   "setup_triangles": int(rec), "bin_entries": int(pairs), "tile": 16,
                   "l2": "flushed before every timed frame (256 MiB write on the renderer's stream)",
                   "parallelism": f"replicas x{world}"},
        "fragments_per_s": round(frags_per_frame * fps, 1),
        "fragments_per_frame": int(frags_per_frame),
        "depth_tested_fragments_per_frame": int(tested_per_frame),
        "triangles_per_s": round(st["input_triangles"] / args.steps * fps, 1),
        "phase_ms": {"vertex": round(tm.vertex_ms / max(1, tm.passes), 4),
                     "setup": round(tm.setup_ms / max(1, tm.passes), 4),
                     "bin": round(tm.bin_ms / max(1, tm.passes), 4),
                     "tile": round(k4_ms, 4)},
        "wall_ms_per_step": round(wall * 1e3 / args.steps, 4),
        "roofline": {"kernel": "k_tile (K4 tile raster/ROP)", "bound": "hbm",
                     "achieved": round(achieved, 2) if achieved else None, "peak": peak,
                     "peak_source": f"{peak_src} (HBM copy)", "unit": "GB/s",
                     "frac": round(achieved / peak, 5) if achieved else None,
                     "algorithmic_bytes_per_launch": int(k4_bytes),
                     "traffic": traffic},
        "e2e": {"value": round(e2e_fps, 3), "unit": "frames/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(st["kernel_launches"]),
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(spec, args.cpu_seconds)
    if world > 1:
        torch.distributed.destroy_process_group()
    return out if rank == 0 else None


def tex_bytes_of(scene):
    n = 0
    for name, a in scene.cmds:
        if name == "glTexImage2D":
            w, h = int(a[3]), int(a[4])
            n += 4 * (w * h + (w // 2) * (h // 2))
    return n


def setup_batch_frames(lib, scenes):
    ctxs, streams = [], []
    for sc in scenes:
        c = lib.context(sc.width, sc.height)
        k = W.frame_start(sc)
        sc.play(c, 0, k)
        ctxs.append(c)
        streams.append(sc.stream(k))
    for c in ctxs:
        c.glFinish()
    return ctxs, G.PreparedStreams(lib, ctxs, streams)


def run_batch(args, spec):
    """The uneven-batch workload: 256 frames of different sizes and loads per step.

    value: frames/s of the batched path (one mtgl_batch_render of all frames per step,
    replayed from its CUDA graph), CUDA events on the batch's stream around the submission,
    L2 flushed before each step. batched_wall / plain_wall: the same frames on the host
    clock through the batched path and through the plain per-frame path (glFinish on each
    context), GL calls replayed natively (mtgl_play_many) in both."""
    import torch

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import mytinygl_gb300 as M

    M.build()
    lib = M.library()
    bind_extras(lib)
    scenes = W.uneven_batch(BATCH_FRAMES)
    ctxs, streams = setup_batch_frames(lib, scenes)
    npix = sum(sc.width * sc.height for sc in scenes)
    tris = sum(W.scene_triangles(sc) for sc in scenes)
    batch = lib.batch()
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ext = torch.cuda.ExternalStream(batch.stream)
    for _ in range(args.warmup):
        streams.play()
        batch.render(ctxs)
        batch.wait()
    batch.reset_stats()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for i in range(args.steps):
            streams.play()  # host: each frame's GL calls queue its pass
            with torch.cuda.stream(ext):
                flush_buf.zero_()
                starts[i].record(ext)
            batch.render(ctxs)
            ends[i].record(ext)
        batch.wait()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    total_ms = sum(s_.elapsed_time(e) for s_, e in zip(starts, ends))
    bst = batch.stats()
    fps = job_rate(args.steps * BATCH_FRAMES, total_ms / 1e3)

    # host clock, outside the clock sampler (its NVML queries stall the driver): the batched
    # path and the plain per-frame path (each frame's pass flushed on its own context, as
    # one frame per pipeline run; glFinish per frame, or glFlush per frame and one glFinish
    # per step, whichever is faster)
    wall_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(wall_steps):
        streams.play()
        batch.render(ctxs)
    batch.wait()
    batched_wall_fps = job_rate(wall_steps * BATCH_FRAMES, time.perf_counter() - t0)
    for c in ctxs:
        c.glFinish()
    plain_fps = {}
    for mode in ("finish", "flush"):
        t0 = time.perf_counter()
        for _ in range(max(1, wall_steps // 2)):
            for c, b in zip(ctxs, streams._bufs):
                lib.lib.mtgl_play(c.handle, b, len(b))
                c.glFinish() if mode == "finish" else c.glFlush()
            for c in ctxs:
                c.glFinish()
        plain_fps[mode] = job_rate(max(1, wall_steps // 2) * BATCH_FRAMES, time.perf_counter() - t0)
    plain_best = max(plain_fps.values())

    # per-phase device time from a profiled run without the graph (K4 roofline)
    pbatch = lib.batch(use_graph=0)
    streams.play()
    pbatch.render(ctxs)
    pbatch.wait()
    pbatch.profile(True)
    for _ in range(3):
        streams.play()
        pbatch.render(ctxs)
    tm = pbatch.timings()
    pst = pbatch.stats()
    pbatch.destroy()
    passes = max(1, tm["passes"])
    k4_ms = tm["tile_ms"] / passes
    rec = bst["setup_triangles"] / max(1, bst["batches"])
    pairs = bst["bin_entries"] / max(1, bst["batches"])
    tex = sum(tex_bytes_of(sc) for sc in scenes)
    k4_bytes = npix * 9 + pairs * 4 + rec * REC_BYTES + tex
    peak, peak_src = measured_peaks()
    achieved = k4_bytes / (k4_ms / 1e3) / 1e9 if k4_ms > 0 else None

    # fragments per batch with depth rejection off (untimed)
    frags = 0
    for c, sc in zip(ctxs, scenes):
        frags += covered_fragments(lib, sc, W.frame_start(sc))

    # e2e: each step replays every frame's GL calls with client vertex arrays (staged and
    # sent host->device that step) and copies every colour buffer back into page-locked host
    # memory (mtgl_batch_render_read). Sequential: one step at a time. In flight: E2E_SETS
    # sets of contexts and executors take turns (triple buffering), so one step's host work
    # (playing the GL calls, submitting) overlaps the others' copies and device work, as a
    # renderer feeding frames continuously would run.
    escenes = W.uneven_batch(BATCH_FRAMES, use_vbo=False)
    e_steps = max(E2E_SETS, min(args.steps, 20))

    def e2e_set():
        c, st = setup_batch_frames(lib, escenes)
        hs = [torch.empty((sc.height, sc.width), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
              for sc in escenes]
        return c, st, lib.batch(), hs

    sets = [e2e_set() for _ in range(E2E_SETS)]
    for ectxs, estreams, ebatch, hosts in sets:
        for _ in range(args.warmup):
            estreams.play()
            ebatch.render(ectxs, colors=hosts)
            ebatch.wait()
    ectxs, estreams, ebatch, hosts = sets[0]
    for c in ectxs:
        c.reset_stats()
    estreams.play()
    ebatch.render(ectxs, colors=hosts)
    ebatch.wait()
    h2d = sum(c.stats()["staged_bytes"] for c in ectxs)
    t0 = time.perf_counter()
    for _ in range(e_steps):
        estreams.play()
        ebatch.render(ectxs, colors=hosts)
        ebatch.wait()
    e2e_seq_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for k in range(e_steps):
        ectxs, estreams, ebatch, hosts = sets[k % E2E_SETS]
        ebatch.wait()  # this set's previous step has landed
        estreams.play()
        ebatch.render(ectxs, colors=hosts)
    for _, _, ebatch, _ in sets:
        ebatch.wait()
    e2e_s = time.perf_counter() - t0
    e2e_fps = job_rate(e_steps * BATCH_FRAMES, e2e_s)
    e2e_seq_fps = job_rate(e_steps * BATCH_FRAMES, e2e_seq_s)
    for ectxs, _, ebatch, _ in sets:
        ebatch.destroy()
        for c in ectxs:
            c.destroy()
    batch.destroy()
    for c in ctxs:
        c.destroy()

    out = {
        "metric": "frames/s",
        "value": round(fps, 2),
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded; mytinygl_gb300/workloads.py uneven_batch)",
        "config": {"workload": spec["name"] if BATCH_FRAMES == 256 else f"uneven_batch_{BATCH_FRAMES}_frames",
                   "description": spec["desc"], "frames_per_step": BATCH_FRAMES,
                   "pixels_per_step": npix, "input_triangles_per_step": tris,
                   "setup_triangles_per_step": int(rec), "bin_entries_per_step": int(pairs),
                   "tile": bst["tile_size"], "persistent_ctas": bst["ctas"],
                   "record_capacity": bst["record_capacity"], "pair_capacity": bst["pair_capacity"],
                   "graph_replays": bst["graph_replays"], "graph_captures": bst["graph_captures"],
                   "l2": "flushed before every timed step (256 MiB write on the batch stream)",
                   "parallelism": f"replicas x{world}"},
        "batched_wall_frames_per_s": round(batched_wall_fps, 2),
        "plain_wall_frames_per_s": round(plain_best, 2),
        "plain_wall_frames_per_s_by_sync": {k: round(v, 2) for k, v in plain_fps.items()},
        "batched_vs_plain_wall": round(batched_wall_fps / plain_best, 3),
        "fragments_per_s": round(frags * fps / BATCH_FRAMES, 1),
        "fragments_per_step": int(frags),
        "triangles_per_s": round(tris * fps / BATCH_FRAMES, 1),
        "phase_ms": {"vertex": round(tm["vertex_ms"] / passes, 4), "setup": round(tm["setup_ms"] / passes, 4),
                     "bin": round(tm["bin_ms"] / passes, 4), "tile": round(k4_ms, 4)},
        "wall_ms_per_step": round(wall * 1e3 / args.steps, 4),
        "roofline": {"kernel": "k_tile (K4 tile raster/ROP, persistent over all frames)", "bound": "hbm",
                     "achieved": round(achieved, 2) if achieved else None, "peak": peak,
                     "peak_source": f"{peak_src} (HBM copy)", "unit": "GB/s",
                     "frac": round(achieved / peak, 5) if achieved else None,
                     "algorithmic_bytes_per_launch": int(k4_bytes), "traffic": ncu_traffic(spec["name"])},
        "e2e": {"value": round(e2e_fps, 2), "unit": "frames/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(npix * 4), "steps_in_flight": E2E_SETS,
                "sequential_value": round(e2e_seq_fps, 2),
                "note": "host clock; GL calls replayed with client arrays every step (their staged bytes are "
                        "h2d), every colour buffer copied to page-locked host memory"},
        "gpu_launches": int(bst["kernel_launches"]),
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_batch_baseline(args.cpu_seconds)
    if world > 1:
        torch.distributed.destroy_process_group()
    return out if rank == 0 else None


def _serve_requests(trace, base, outs=None):
    reqs = (G.Request * len(trace))()
    for i, (t, sc, w, h, mv) in enumerate(trace):
        r = reqs[i]
        r.scene, r.width, r.height = sc, w, h
        r.modelview[:] = [float(v) for v in mv]
        r.arrival = base + t
        r.color = outs(i, w, h) if outs else None
    return reqs


def _latency_summary(reqs):
    lat = np.array([r.finished - r.arrival for r in reqs if r.status == 0]) * 1e3
    ok = [r for r in reqs if r.status == 0]
    span = max(r.finished for r in ok) - min(r.arrival for r in ok)
    return {"p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
            "mean_ms": round(float(lat.mean()), 3), "max_ms": round(float(lat.max()), 3),
            "completed": len(ok), "failed": len(reqs) - len(ok),
            "frames_per_s": round(len(ok) / span, 2), "span_s": span,
            "mean_batch": round(float(np.mean([r.batch_size for r in ok])), 2)}


def run_serve(args, spec):
    """The serving workload: a Poisson trace replayed against the C serving loop.

    value: frames/s completed over the trace (first arrival to last completion), frames
    left in device framebuffers; latency = completion - arrival on the server clock.
    e2e: a shorter trace at the same rate with every frame read back into page-locked
    host buffers (a ring larger than the requests that can be in flight)."""
    import torch

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    import mytinygl_gb300 as M

    M.build()
    lib = M.library()
    scenes = W.serve_scenes(32)
    ctxs = []
    srv = lib.server(executors=2, max_batch=64)
    for sc in scenes:
        c = lib.context(sc.width, sc.height)
        k = W.frame_start(sc)
        sc.play(c, 0, k)
        c.glFinish()
        ctxs.append(c)
        srv.add_scene(c, sc.stream(k), W.scene_triangles(sc))
    rate = 2000.0
    # warm-up: capacities learned, graphs captured, framebuffer pool filled
    for i in range(args.warmup):
        warm = W.serve_trace(0.5, rate, seed=100 + i)
        srv.run_trace(_serve_requests(warm, srv.now() + 0.01))
    trace = W.serve_trace(args.serve_seconds, rate, seed=6)
    reqs = _serve_requests(trace, srv.now() + 0.05)
    with ClockSampler(local) as clocks:
        st0 = srv.stats()
        srv.run_trace(reqs)
        st1 = srv.stats()
    summ = _latency_summary(reqs)
    served_fps = job_rate(summ["completed"], summ["span_s"])
    busy = st1["busy_seconds"] - st0["busy_seconds"]
    batches = st1["batches"] - st0["batches"]
    # the rated load saturates the GPU: latency there is mostly queueing. Latency below
    # saturation, at 70 % of the throughput just measured, on a shorter trace:
    sub_rate = round(0.7 * summ["frames_per_s"], 1)
    sub = W.serve_trace(min(20.0, args.serve_seconds), sub_rate, seed=8)
    sreqs = _serve_requests(sub, srv.now() + 0.05)
    srv.run_trace(sreqs)
    ssumm = _latency_summary(sreqs)

    # e2e: every frame read back into a ring of page-locked buffers per resolution
    ring = 4 * 64 + 32  # more than executors x max_batch requests can be in flight
    pinned = {}
    for w, h in W.SERVE_RESOLUTIONS:
        pinned[(w, h)] = [torch.empty(w * h, dtype=torch.int32, pin_memory=True) for _ in range(ring)]
    count = {}

    def out_for(i, w, h):
        j = count.get((w, h), 0)
        count[(w, h)] = j + 1
        return pinned[(w, h)][j % ring].data_ptr()

    etrace = W.serve_trace(min(10.0, args.serve_seconds), rate, seed=7)
    ereqs = _serve_requests(etrace, srv.now() + 0.05, out_for)
    srv.run_trace(ereqs)
    esumm = _latency_summary(ereqs)
    e2e_fps = job_rate(esumm["completed"], esumm["span_s"])
    d2h = sum(w * h * 4 for _, _, w, h, _ in etrace) / max(1, len(etrace))
    srv.destroy()
    for c in ctxs:
        c.destroy()
    out = {
        "metric": "frames/s", "value": round(served_fps, 2), "unit": "frames/s", "n_gpus": world,
        "steps": len(reqs), "warmup": args.warmup, "ms_per_step": summ["mean_ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; mytinygl_gb300/workloads.py serve_scenes / serve_trace)",
        "config": {"workload": spec["name"], "description": spec["desc"], "offered_rate": rate,
                   "duration_s": args.serve_seconds, "requests": len(reqs), "executors": 2, "max_batch": 64,
                   "memory_budget_gib": 40, "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": summ["p50_ms"], "p99": summ["p99_ms"], "mean": summ["mean_ms"],
                       "max": summ["max_ms"]},
        "served": summ, "batches": batches,
        "below_saturation": {"offered_rate": sub_rate, "duration_s": min(20.0, args.serve_seconds),
                             "latency_ms": {"p50": ssumm["p50_ms"], "p99": ssumm["p99_ms"]},
                             "frames_per_s": ssumm["frames_per_s"], "mean_batch": ssumm["mean_batch"]},
        "gpu_busy_fraction": round(busy / max(1e-9, max(r.finished for r in reqs) - min(r.arrival for r in reqs)), 3),
        "deferred_for_budget": st1["deferred_for_budget"] - st0["deferred_for_budget"],
        "peak_gib_admitted": round(st1["peak_bytes_admitted"] / 2**30, 3),
        "e2e": {"value": round(e2e_fps, 2), "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(d2h), "latency_ms": {"p50": esumm["p50_ms"], "p99": esumm["p99_ms"]}},
        "gpu_launches": int(st1["kernel_launches"] - st0["kernel_launches"]), "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        times = cpu_serve_sample(_oracle_lib(), args.cpu_seconds, threads)
        out["cpu_baseline"] = {"value": round(threads / statistics.mean(times), 4), "unit": "frames/s",
                               "cores": threads, "kind": "port",
                               "sample": (f"{len(times)} requests of the trace, each frame on its own oracle "
                                          f"context, {threads} threads; frames/s = threads / mean frame time")}
    if world > 1:
        torch.distributed.destroy_process_group()
    return out if rank == 0 else None


def cpu_serve_sample(lib, seconds, threads):
    """Oracle frames of serving requests, concurrently on `threads` cores: each request's scene
    is set up on a context of the request's size (untimed), then its frame is timed. Takes
    requests of the trace in order until about `seconds` of work per thread is done."""
    scenes = W.serve_scenes(32)
    trace = W.serve_trace(60.0, 2000.0, seed=6)
    lock = threading.Lock()
    state = {"next": 0, "times": [], "spent": 0.0}

    def work(_):
        while True:
            with lock:
                if state["spent"] >= seconds * threads or state["next"] >= len(trace):
                    return
                i = state["next"]
                state["next"] += 1
            _, sc, w, h, mv = trace[i]
            scene = scenes[sc]
            k = W.frame_start(scene)
            c = lib.context(w, h)
            scene.play(c, 0, k)
            c.glViewport(0, 0, w, h)
            c.glMatrixMode(G.GL_MODELVIEW)
            c.glLoadMatrixf(np.asarray(mv, np.float32))
            t0 = time.perf_counter()
            scene.play(c, k)
            dt = time.perf_counter() - t0
            c.destroy()
            with lock:
                state["times"].append(dt)
                state["spent"] += dt
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, range(threads)))
    return state["times"]


def cpu_batch_frames(lib, scenes, threads):
    """Render each scene once on the oracle, one context per thread; returns wall seconds."""
    def one(sc):
        c = lib.context(sc.width, sc.height)
        sc.play(c)
        c.destroy()
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(one, scenes))
    return time.perf_counter() - t0


def cpu_batch_sample(seconds):
    """Frames of the uneven batch whose oracle time fits the budget: every k-th frame."""
    scenes = W.uneven_batch(BATCH_FRAMES, use_vbo=False)
    tris = [W.scene_triangles(sc) for sc in scenes]
    per_tri = 2.5e-6  # conservative CPU seconds per input triangle per thread
    threads = os.cpu_count() or 1
    k = 1
    while k < BATCH_FRAMES and sum(tris[::k]) * per_tri / threads > seconds:
        k *= 2
    return scenes[::k], k, threads


def cpu_batch_baseline(seconds):
    lib = _oracle_lib()
    sample, k, threads = cpu_batch_sample(seconds)
    wall = cpu_batch_frames(lib, sample, threads)
    return {"value": round(len(sample) / wall, 4), "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": (f"every {k}th frame of the 256-frame batch ({len(sample)} frames, whole frames), "
                       f"one oracle context per frame on {threads} threads"), "wall_s": round(wall, 2)}


def _oracle_lib():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True, capture_output=True)
    return G.load(os.path.join(REPO, "oracle", "_build", "libmtgl_oracle.so"))


def cpu_frame_time(lib, spec, ntri, reps):
    scene = spec["builder"](use_vbo=False, ntri=ntri) if spec["name"] != WORKLOADS["sphere"]["name"] else \
        spec["builder"](use_vbo=False)
    fs = W.frame_start(scene)
    ctx = lib.context(scene.width, scene.height)
    scene.play(ctx, 0, fs)
    t0 = time.perf_counter()
    for _ in range(reps):
        scene.play(ctx, fs)
    dt = time.perf_counter() - t0
    ctx.destroy()
    return dt / reps


def cpu_baseline(spec, seconds):
    """The oracle on every host core, one context per thread (the reference keeps one current
    context per thread, gl_api.c:14-23), each rendering a sample of the frame's triangles."""
    lib = _oracle_lib()
    threads = os.cpu_count() or 1
    full = spec["full_tris"]
    sample = min(full, 500)
    t1 = cpu_frame_time(lib, spec, sample, 1)
    per_tri = t1 / sample
    # about `seconds` of work per thread in total, at least one render each
    sample = int(min(full, max(100, (seconds / 3.0) / max(per_tri, 1e-9))))
    reps = 3 if sample < full else max(1, int(seconds / max(t1 * full / 500, 1e-6)))
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        times = list(ex.map(lambda _: cpu_frame_time(lib, spec, sample, reps), range(threads)))
    wall = time.perf_counter() - t0
    frame_s = statistics.median(times) * (full / sample)
    return {"value": round(threads / frame_s, 5), "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": (f"first {sample} of {full} triangles of the same frame, {reps} renders per context, "
                       f"{threads} contexts on {threads} threads; frame time scaled by {full}/{sample}"),
            "wall_s": round(wall, 2)}


def run_reference(args, spec):
    world, rank, local = dist_init()
    if rank != 0:
        return None
    lib = _oracle_lib()
    if spec is WORKLOADS["serve"]:
        threads = os.cpu_count() or 1
        budget = 120.0 / max(1, args.steps + args.warmup)
        cpu_serve_sample(lib, min(2.0, budget), threads)  # warm-up
        times = cpu_serve_sample(lib, budget * (args.steps / max(1, args.steps)), threads)
        fps = threads / statistics.mean(times)
        desc = (f"{len(times)} requests of the trace in order, each frame rendered on its own oracle context "
                f"(scene set-up untimed), {threads} threads at once; frames/s = threads / mean frame time")
        return {"impl": "reference", "metric": "frames/s", "value": round(fps, 4), "unit": "frames/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(statistics.mean(times) * 1e3, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded; mytinygl_gb300/workloads.py serve_scenes / serve_trace)",
                "config": {"workload": spec["name"], "description": spec["desc"]},
                "latency_ms": {"p50": round(float(np.percentile(times, 50)) * 1e3, 3),
                               "p99": round(float(np.percentile(times, 99)) * 1e3, 3)},
                "cpu_baseline": {"value": round(fps, 4), "unit": "frames/s", "cores": threads, "kind": "port",
                                 "sample": desc},
                "e2e": {"value": round(fps, 4), "unit": "frames/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
    if spec is WORKLOADS["batch"]:
        sample, k, threads = cpu_batch_sample(120.0 / max(1, args.steps + args.warmup))
        for _ in range(args.warmup):
            cpu_batch_frames(lib, sample, threads)
        walls = [cpu_batch_frames(lib, sample, threads) for _ in range(args.steps)]
        fps = len(sample) / statistics.median(walls)
        desc = (f"every {k}th frame of the 256-frame batch ({len(sample)} whole frames) per step, one oracle "
                f"context per frame on {threads} threads")
        return {"impl": "reference", "metric": "frames/s", "value": round(fps, 5), "unit": "frames/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(statistics.median(walls) * 1e3, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded; mytinygl_gb300/workloads.py uneven_batch)",
                "config": {"workload": spec["name"], "description": spec["desc"]},
                "cpu_baseline": {"value": round(fps, 5), "unit": "frames/s", "cores": threads, "kind": "port",
                                 "sample": desc},
                "e2e": {"value": round(fps, 5), "unit": "frames/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
    threads = os.cpu_count() or 1
    full = spec["full_tris"]
    sample = min(full, 500)
    t1 = cpu_frame_time(lib, spec, sample, 1)
    budget = 120.0 / max(1, args.steps + args.warmup)  # whole run within a couple of minutes
    sample = int(min(full, max(100, budget / max(t1 / sample, 1e-9))))
    step = lambda: list(cf.ThreadPoolExecutor(threads).map(lambda _: cpu_frame_time(lib, spec, sample, 1),
                                                           range(threads)))
    for _ in range(args.warmup):
        step()
    per = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        per.append(statistics.median(step()))
    wall = time.perf_counter() - t0
    frame_s = statistics.median(per) * (full / sample)
    fps = threads / frame_s
    desc = (f"first {sample} of {full} triangles of the frame per context, {threads} contexts on {threads} "
            f"threads per step; frame time scaled by {full}/{sample}")
    return {"impl": "reference", "metric": "frames/s", "value": round(fps, 5), "unit": "frames/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(wall * 1e3 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; mytinygl_gb300/workloads.py)",
            "config": {"workload": spec["name"], "description": spec["desc"]},
            "cpu_baseline": {"value": round(fps, 5), "unit": "frames/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": round(fps, 5), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="batch")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline work per thread")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="serving trace length (workload serve)")
    ap.add_argument("--frames", type=int, default=256, help="frames per step of the batch workload")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)  # at least three untimed warm-up steps
    global BATCH_FRAMES
    BATCH_FRAMES = args.frames
    spec = WORKLOADS[args.workload]
    if args.impl == "reference":
        out = run_reference(args, spec)
    elif args.workload == "batch":
        out = run_batch(args, spec)
    elif args.workload == "serve":
        out = run_serve(args, spec)
    else:
        out = run_ours(args, spec)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
