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
  roofline_stages  the same for each pipeline stage (vertex, setup, binning, tile), and K4's
               issue-slot fraction (ncu warp instructions per launch over SMs x 4 x clock x time).
  parity       the timed frames read back and compared with the CPU oracle rendering the same
               inputs: colour max error and mismatching-pixel fraction, depth and stencil
               mismatches (serving: a seeded sample of requests, colour only).
  cpu_baseline the CPU oracle (a restatement of MyTinyGL's renderer) on all host cores, one
               context per thread, on a bounded sample of the same workload; also on one
               thread and built with MyTinyGL's shipped flags, with the CPU model.
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
REC_BYTES = 240  # triangle record written by the setup kernel, read by the tile kernel
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


POST_VERTEX_BYTES = 48  # post-transform vertex written by K1, read by K2
REC_BOX_BYTES = 80      # record words binning reads: screen vertices, box, area, edge differences
PAIR_BYTES = 8          # (tile, record) pair written by binning


def ncu_instructions(workload):
    """Warp instructions per K4 launch (smsp__inst_executed.sum) from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "ncu_k4_instructions.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and parts[0] == workload and parts[1] == "k_tile":
            return float(parts[2])
    return None


def stage_rooflines(workload, vertices, vertex_bytes, rec, pairs, npix, tex, phase_ms, peak, sms, sm_mhz):
    """Per-stage HBM fractions from each stage's compulsory bytes (inputs read once, outputs
    written once) over its measured time, and K4's issue-slot fraction: warp instructions
    per launch (ncu) over the issue slots of its measured time (SMs x 4 schedulers x clock).
      K1 vertex:  attribute bytes read + vertices x 48 (post-transform vertex written)
      K2 setup:   vertices x 48 (read once) + records x 224 (written)
      K3 binning: records x 80 (box and edge words read) + pairs x 8 (written)
      K4 tile:    pixels x 9 + pairs x 4 + records x 224 + texture bytes"""
    stages = {
        "k1_vertex": (vertex_bytes + vertices * POST_VERTEX_BYTES, phase_ms.get("vertex")),
        "k2_setup": (vertices * POST_VERTEX_BYTES + rec * REC_BYTES, phase_ms.get("setup")),
        "k3_bin": (rec * REC_BOX_BYTES + pairs * PAIR_BYTES, phase_ms.get("bin")),
        "k4_tile": (npix * 9 + pairs * 4 + rec * REC_BYTES + tex, phase_ms.get("tile")),
    }
    out = {}
    for k, (b, ms) in stages.items():
        gbs = b / (ms / 1e3) / 1e9 if ms else None
        out[k] = {"algorithmic_bytes": int(b), "ms": ms, "achieved_gbs": round(gbs, 2) if gbs else None,
                  "frac": round(gbs / peak, 5) if gbs else None}
    inst = ncu_instructions(workload)
    t4 = phase_ms.get("tile")
    if inst and t4 and sm_mhz:
        slots = sms * 4 * sm_mhz * 1e6 * t4 / 1e3
        out["k4_tile"]["issue"] = {"warp_instructions": int(inst), "issue_slots": int(slots),
                                   "frac": round(inst / slots, 4),
                                   "how": "ncu smsp__inst_executed.sum per launch (profiles/ncu_k4_instructions.txt) "
                                          "over SMs x 4 schedulers x median SM clock x measured K4 time"}
    return out


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


PARITY_TOLERANCE = "depth and stencil bit-exact (NaN payloads aside), RGBA8 colour within 1 LSB per channel"


def frame_buffers(scene):
    """Buffers the frame part of a scene clears (a frame played again on a context leaves only
    these defined as the frame alone would)."""
    bits = 0
    for name, a in scene.cmds[W.frame_start(scene):]:
        if name == "glClear":
            bits |= int(a[0])
    return {"color": bool(bits & G.GL_COLOR_BUFFER_BIT), "depth": bool(bits & G.GL_DEPTH_BUFFER_BIT),
            "stencil": bool(bits & G.GL_STENCIL_BUFFER_BIT)}


class Parity:
    """Oracle-versus-GPU statistics over many frames: colour max error and mismatching-pixel
    fraction, depth and stencil mismatches, glGetError agreement."""

    def __init__(self):
        self.lock = threading.Lock()
        self.frames = self.pixels = self.color_px = self.color_bad = 0
        self.color_max = 0
        self.depth_bad = self.stencil_bad = self.error_bad = 0
        self.buffers = set()
        self.worst = None

    def add(self, want, got, buffers, name=""):
        """want/got: (colour u32, depth f32 or None, stencil u8 or None, gl error or None)."""
        cmax = cbad = dbad = sbad = 0
        npx = int(want[0].size)
        if buffers.get("color") and want[0] is not None and got[0] is not None:
            a = want[0].view(np.uint8).reshape(*want[0].shape, 4).astype(np.int16)
            b = got[0].view(np.uint8).reshape(*got[0].shape, 4).astype(np.int16)
            d = np.abs(a - b).max(axis=-1)
            cmax = int(d.max()) if d.size else 0
            cbad = int((d > 0).sum())
        if buffers.get("depth") and want[1] is not None and got[1] is not None:
            same = (want[1].view(np.uint32) == got[1].view(np.uint32)) | (np.isnan(want[1]) & np.isnan(got[1]))
            dbad = int((~same).sum())
        if buffers.get("stencil") and want[2] is not None and got[2] is not None:
            sbad = int((want[2] != got[2]).sum())
        with self.lock:
            self.frames += 1
            self.pixels += npx
            self.buffers |= {k for k, v in buffers.items() if v}
            if buffers.get("color"):
                self.color_px += npx
            self.color_bad += cbad
            if cmax > self.color_max:
                self.worst = name
            self.color_max = max(self.color_max, cmax)
            self.depth_bad += dbad
            self.stencil_bad += sbad
            if want[3] is not None and got[3] is not None and int(want[3]) != int(got[3]):
                self.error_bad += 1

    def summary(self):
        ok = (self.color_max <= 1 and self.depth_bad == 0 and self.stencil_bad == 0 and self.error_bad == 0
              and self.frames > 0)
        return {"frames_compared": self.frames, "pixels_compared": self.pixels,
                "buffers": sorted(self.buffers), "color_max_err": self.color_max,
                "color_mismatch_frac": round(self.color_bad / max(1, self.color_px), 9),
                "depth_mismatches": self.depth_bad, "stencil_mismatches": self.stencil_bad,
                "gl_error_mismatches": self.error_bad, "worst_color_frame": self.worst,
                "tolerance": PARITY_TOLERANCE, "pass": ok,
                "against": "CPU oracle (restatement of MyTinyGL's renderer, pinned bit-exact to the reference "
                           "build and its golden fixtures), same seeded inputs"}


def gpu_frame(ctx, buffers=None):
    c, d, s = ctx.read()
    return c, d, s, ctx.glGetError()


def oracle_frame(lib, scene):
    c = lib.context(scene.width, scene.height)
    try:
        scene.play(c)
        col, dep, st = c.read()
        return col, dep, st, c.glGetError()
    finally:
        c.destroy()


def oracle_parity(scenes, gpu_frames, threads=None):
    """Each scene rendered whole on the CPU oracle (one context per thread) and compared with the
    GPU's frame of it. Untimed: this is the checker, not the baseline."""
    lib = _oracle_lib()
    threads = threads or os.cpu_count() or 1
    par = Parity()
    t0 = time.perf_counter()

    def one(i):
        par.add(oracle_frame(lib, scenes[i]), gpu_frames[i], frame_buffers(scenes[i]), scenes[i].name)

    # largest frames first, so the threads finish together
    order = sorted(range(len(scenes)), key=lambda i: -W.scene_triangles(scenes[i]) - scenes[i].width * scenes[i].height)
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(one, order))
    out = par.summary()
    out["oracle_wall_s"] = round(time.perf_counter() - t0, 2)
    return out



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
    gpu_out = gpu_frame(ctx) if not args.no_parity else None  # the last timed frame
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
        "config": single_config(spec, scene, world),
        "pipeline": {"setup_triangles": int(rec), "bin_entries": int(pairs), "tile": 16},
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
    out["roofline_stages"] = stage_rooflines(
        spec["name"], st["vertices"] / args.steps, st["vertex_bytes"] / args.steps, rec, pairs, npix, tex_bytes,
        out["phase_ms"], peak, torch.cuda.get_device_properties(local).multi_processor_count,
        out["clocks"].get("sm_mhz"))
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(spec, args.cpu_seconds)
    if rank == 0 and gpu_out is not None:
        out["parity"] = oracle_parity([scene], [gpu_out])
    if world > 1:
        torch.distributed.destroy_process_group()
    return out if rank == 0 else None


L2_NOTE = "GPU arm: L2 flushed before every timed step (256 MiB write on the rendering stream)"


def single_config(spec, scene, world):
    """The workload keys of a single-frame line (the same in both arms)."""
    return {"workload": spec["name"], "description": spec["desc"], "width": scene.width, "height": scene.height,
            "input_triangles": W.scene_triangles(scene), "l2": L2_NOTE, "parallelism": f"replicas x{world}"}


def batch_config(spec, scenes, world):
    return {"workload": spec["name"] if len(scenes) == 256 else f"uneven_batch_{len(scenes)}_frames",
            "description": spec["desc"], "frames_per_step": len(scenes),
            "pixels_per_step": sum(sc.width * sc.height for sc in scenes),
            "input_triangles_per_step": sum(W.scene_triangles(sc) for sc in scenes), "l2": L2_NOTE,
            "parallelism": f"replicas x{world}"}


def serve_config(spec, args, requests, world):
    return {"workload": spec["name"], "description": spec["desc"], "offered_rate": args.serve_rate,
            "duration_s": args.serve_seconds, "requests": requests, "memory_budget_gib": 40,
            "parallelism": f"replicas x{world}"}


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
    # the frames of the last timed step, for the parity check against the oracle
    gpu_frames = [gpu_frame(c) for c in ctxs] if not args.no_parity else None

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
        "config": batch_config(spec, scenes, world),
        "pipeline": {"setup_triangles_per_step": int(rec), "bin_entries_per_step": int(pairs),
                     "tile": bst["tile_size"], "persistent_ctas": bst["ctas"],
                     "record_capacity": bst["record_capacity"], "pair_capacity": bst["pair_capacity"],
                     "graph_replays": bst["graph_replays"], "graph_captures": bst["graph_captures"]},
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
    nb = max(1, bst["batches"])
    out["roofline_stages"] = stage_rooflines(
        out["config"]["workload"], bst["vertices"] / nb, bst["vertex_bytes"] / nb, rec, pairs, npix, tex,
        out["phase_ms"], peak, torch.cuda.get_device_properties(local).multi_processor_count,
        out["clocks"].get("sm_mhz"))
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_batch_baseline(args.cpu_seconds)
    if rank == 0 and gpu_frames is not None:
        out["parity"] = oracle_parity(scenes, gpu_frames)
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
    rate = args.serve_rate
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

    # parity: a seeded sample of the timed trace's requests, served again as one burst with
    # their colour read back, against the oracle rendering the same calls
    psample = []
    if not args.no_parity:
        pick = np.random.default_rng(61).choice(len(trace), size=min(SERVE_PARITY_REQUESTS, len(trace)),
                                                replace=False)
        psample = [trace[int(i)] for i in sorted(pick)]
        pouts = [np.zeros((h, w), np.uint32) for _, _, w, h, _ in psample]
        preqs = _serve_requests([(0.0,) + tuple(r[1:]) for r in psample], srv.now() + 0.01,
                                lambda i, w, h: pouts[i].ctypes.data)
        srv.run_trace(preqs)
        pfailed = sum(1 for r in preqs if r.status != 0)
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
        "config": serve_config(spec, args, len(reqs), world),
        "pipeline": {"executors": 2, "max_batch": 64},
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
    if rank == 0 and psample:
        out["parity"] = serve_parity(scenes, psample, pouts)
        out["parity"]["gpu_failed_requests"] = pfailed
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        times = cpu_serve_sample(_oracle_lib(), args.cpu_seconds, threads)
        times1 = cpu_serve_sample(_oracle_lib(), min(args.cpu_seconds, 10.0), 1)
        times_s = cpu_serve_sample(_oracle_lib(shipped=True), args.cpu_seconds, threads)
        out["cpu_baseline"] = {"value": round(threads / statistics.mean(times), 4), "unit": "frames/s",
                               "cores": threads, "kind": "port", "cpu_model": cpu_model(), "build": STRICT_BUILD,
                               "sample": (f"{len(times)} requests of the trace, each frame on its own oracle "
                                          f"context, {threads} threads; frames/s = threads / mean frame time"),
                               "one_thread": {"value": round(1.0 / statistics.mean(times1), 4), "unit": "frames/s",
                                              "cores": 1, "sample": f"{len(times1)} requests of the trace in order"},
                               "shipped_flags": {"value": round(threads / statistics.mean(times_s), 4),
                                                 "unit": "frames/s", "cores": threads, "build": SHIPPED_BUILD,
                                                 "sample": f"{len(times_s)} requests of the trace in order"},
                               "vs_reference": PORT_VS_REFERENCE}
    if world > 1:
        torch.distributed.destroy_process_group()
    return out if rank == 0 else None


SERVE_PARITY_REQUESTS = 16


def serve_oracle_frame(lib, scene, w, h, mv):
    """A serving request rendered on the oracle: the scene's resident part on a context of the
    request's size, then the request's viewport and modelview, then the frame part."""
    c = lib.context(w, h)
    try:
        k = W.frame_start(scene)
        scene.play(c, 0, k)
        c.glViewport(0, 0, w, h)
        c.glMatrixMode(G.GL_MODELVIEW)
        c.glLoadMatrixf(np.asarray(mv, np.float32))
        scene.play(c, k)
        col, _, _ = c.read(depth=False, stencil=False)
        return col, None, None, None
    finally:
        c.destroy()


def serve_parity(scenes, sample, colours):
    """Served colour of each sampled request against the oracle (the server reads back colour
    only). Untimed checker."""
    lib = _oracle_lib()
    par = Parity()
    t0 = time.perf_counter()

    def one(i):
        _, sc, w, h, mv = sample[i]
        par.add(serve_oracle_frame(lib, scenes[sc], w, h, mv), (colours[i], None, None, None), {"color": True},
                f"scene{sc}_{w}x{h}")

    order = sorted(range(len(sample)), key=lambda i: -W.scene_triangles(scenes[sample[i][1]]))
    with cf.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        list(ex.map(one, order))
    out = par.summary()
    out["oracle_wall_s"] = round(time.perf_counter() - t0, 2)
    out["sample"] = f"{len(sample)} requests of the timed trace (seeded choice), served again as one burst"
    return out


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
    """The oracle on all host cores (one context per frame and thread) over whole frames of the
    batch, plus the same on one thread (every 8th frame of the sample) and with the
    reference's shipped optimisation flags."""
    lib = _oracle_lib()
    sample, k, threads = cpu_batch_sample(seconds)
    wall = cpu_batch_frames(lib, sample, threads)
    one = sample[::8]
    wall1 = cpu_batch_frames(lib, one, 1)
    wall_s = cpu_batch_frames(_oracle_lib(shipped=True), sample, threads)
    return {"value": round(len(sample) / wall, 4), "unit": "frames/s", "cores": threads, "kind": "port",
            "cpu_model": cpu_model(), "build": STRICT_BUILD,
            "sample": (f"{'every frame' if k == 1 else f'every {k}th frame'} of the 256-frame batch "
                       f"({len(sample)} frames, whole frames), "
                       f"one oracle context per frame on {threads} threads"), "wall_s": round(wall, 2),
            "one_thread": {"value": round(len(one) / wall1, 4), "unit": "frames/s", "cores": 1,
                           "sample": f"{len(one)} whole frames (every 8th of the sample) on one thread"},
            "shipped_flags": {"value": round(len(sample) / wall_s, 4), "unit": "frames/s", "cores": threads,
                              "build": SHIPPED_BUILD, "sample": "the same frames and threads"},
            "vs_reference": PORT_VS_REFERENCE}


STRICT_BUILD = "oracle (restatement of MyTinyGL's renderer), -O2 -ffp-contract=off"
SHIPPED_BUILD = "oracle with MyTinyGL's shipped flags (Makefile:3) minus -march=native: -O3 -ffast-math"
PORT_VS_REFERENCE = ("oracle frame time / reference frame time, same frames, one thread, measured where the "
                     "reference's sources compile (oracle/speed_vs_reference.py): 1.09-1.26 strict, "
                     "1.05-1.52 with shipped flags")


def cpu_model():
    """The host CPU's model name (lscpu), for the baseline lines."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def _oracle_lib(shipped=False):
    """The CPU oracle (checker and CPU baseline); shipped=True: the build with the reference's
    shipped optimisation flags, for timing only."""
    target, name = ("shipped", "libmtgl_oracle_shipped.so") if shipped else ("all", "libmtgl_oracle.so")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), target], check=True, capture_output=True)
    return G.load(os.path.join(REPO, "oracle", "_build", name))


def cpu_frame_time(lib, scene, reps):
    """Seconds per whole frame (the frame part; the resident part is played once, untimed)."""
    fs = W.frame_start(scene)
    ctx = lib.context(scene.width, scene.height)
    scene.play(ctx, 0, fs)
    t0 = time.perf_counter()
    for _ in range(reps):
        scene.play(ctx, fs)
    ctx.glFinish()
    dt = time.perf_counter() - t0
    ctx.destroy()
    return dt / reps


def cpu_single_frames(lib, scene, reps, threads):
    """Frames/s of `threads` contexts each rendering the whole frame `reps` times at once."""
    with cf.ThreadPoolExecutor(threads) as ex:
        times = list(ex.map(lambda _: cpu_frame_time(lib, scene, reps), range(threads)))
    return threads / statistics.median(times)


def single_reps(lib, spec, scene, seconds):
    """Renders per context so that each thread works about `seconds` (at least one whole frame),
    from a 500-triangle cut's time scaled to the full count."""
    full = spec["full_tris"]
    cut = spec["builder"](use_vbo=False, ntri=min(full, 500)) if spec is not WORKLOADS["sphere"] else scene
    t = cpu_frame_time(lib, cut, 1) * (full / min(full, 500) if spec is not WORKLOADS["sphere"] else 1.0)
    return max(1, int(seconds / max(t, 1e-6)))


def cpu_baseline(spec, seconds):
    """The oracle on every host core, one context per thread (the reference keeps one current
    context per thread, gl_api.c:14-23), each rendering the whole frame; plus one thread, and
    the build with the reference's shipped flags."""
    lib = _oracle_lib()
    threads = os.cpu_count() or 1
    scene = spec["builder"](use_vbo=False)
    reps = single_reps(lib, spec, scene, seconds)
    t0 = time.perf_counter()
    fps = cpu_single_frames(lib, scene, reps, threads)
    wall = time.perf_counter() - t0
    fps1 = cpu_single_frames(lib, scene, reps, 1)
    fps_s = cpu_single_frames(_oracle_lib(shipped=True), scene, reps, threads)
    return {"value": round(fps, 5), "unit": "frames/s", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
            "build": STRICT_BUILD,
            "sample": (f"the whole frame, {reps} renders per context, {threads} contexts on {threads} threads"),
            "wall_s": round(wall, 2),
            "one_thread": {"value": round(fps1, 5), "unit": "frames/s", "cores": 1,
                           "sample": f"the whole frame, {reps} renders on one thread"},
            "shipped_flags": {"value": round(fps_s, 5), "unit": "frames/s", "cores": threads,
                              "build": SHIPPED_BUILD, "sample": "the same renders and threads"},
            "vs_reference": PORT_VS_REFERENCE}


def run_reference(args, spec):
    """The reference arm: the CPU implementation of the path (the oracle, built with MyTinyGL's
    shipped optimisation flags) on every host core, one context per thread, on the same
    workload and config as the GPU arm; rank 0 only."""
    world, rank, local = dist_init()
    if rank != 0:
        return None
    lib = _oracle_lib(shipped=True)
    threads = os.cpu_count() or 1
    common = {"impl": "reference", "metric": "frames/s", "unit": "frames/s", "n_gpus": world, "steps": args.steps,
              "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
              "dtype": "f32"}

    def line(fps, ms, config, data, desc, **extra):
        out = dict(common, value=round(fps, 5), ms_per_step=round(ms, 3), data=data, config=config)
        out.update(extra)
        out["cpu_baseline"] = {"value": round(fps, 5), "unit": "frames/s", "cores": threads, "kind": "port",
                               "build": SHIPPED_BUILD, "cpu_model": cpu_model(), "sample": desc,
                               "vs_reference": PORT_VS_REFERENCE}
        out["e2e"] = {"value": round(fps, 5), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
        return out

    if spec is WORKLOADS["serve"]:
        budget = 120.0 / max(1, args.steps + args.warmup)
        cpu_serve_sample(lib, min(2.0, budget), threads)  # warm-up
        times = cpu_serve_sample(lib, budget * (args.steps / max(1, args.steps)), threads)
        fps = threads / statistics.mean(times)
        desc = (f"{len(times)} requests of the trace in order, each frame rendered on its own oracle context "
                f"(scene set-up untimed), {threads} threads at once; frames/s = threads / mean frame time")
        return line(fps, statistics.mean(times) * 1e3,
                    serve_config(spec, args, len(W.serve_trace(args.serve_seconds, args.serve_rate, seed=6)), world),
                    "synthetic (seeded; mytinygl_gb300/workloads.py serve_scenes / serve_trace)", desc,
                    latency_ms={"p50": round(float(np.percentile(times, 50)) * 1e3, 3),
                                "p99": round(float(np.percentile(times, 99)) * 1e3, 3)})
    if spec is WORKLOADS["batch"]:
        sample, k, threads = cpu_batch_sample(120.0 / max(1, args.steps + args.warmup))
        for _ in range(args.warmup):
            cpu_batch_frames(lib, sample, threads)
        walls = [cpu_batch_frames(lib, sample, threads) for _ in range(args.steps)]
        fps = len(sample) / statistics.median(walls)
        desc = (f"{'every frame' if k == 1 else f'every {k}th frame'} of the 256-frame batch ({len(sample)} whole "
                f"frames) per step, one oracle "
                f"context per frame on {threads} threads")
        return line(fps, statistics.median(walls) * 1e3, batch_config(spec, W.uneven_batch(BATCH_FRAMES, use_vbo=False), world),
                    "synthetic (seeded; mytinygl_gb300/workloads.py uneven_batch)", desc)
    # single frames: a frame's first `sample` triangles per context and step, the frame time
    # scaled to the full triangle count, so the whole run stays within a couple of minutes
    full = spec["full_tris"]
    budget = 120.0 / max(1, args.steps + args.warmup)
    if spec is WORKLOADS["sphere"]:
        sample, scene = full, spec["builder"](use_vbo=False)
    else:
        t1 = cpu_frame_time(lib, spec["builder"](use_vbo=False, ntri=500), 1)
        sample = int(min(full, max(100, budget * 500 / max(t1, 1e-9))))
        scene = spec["builder"](use_vbo=False, ntri=sample)

    def step():
        with cf.ThreadPoolExecutor(threads) as ex:
            return list(ex.map(lambda _: cpu_frame_time(lib, scene, 1), range(threads)))

    for _ in range(args.warmup):
        step()
    per = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        per.append(statistics.median(step()))
    wall = time.perf_counter() - t0
    fps = threads / (statistics.median(per) * (full / sample))
    desc = (f"first {sample} of {full} triangles of the frame per context, {threads} contexts on {threads} "
            f"threads per step; frame time scaled by {full}/{sample}")
    return line(fps, wall * 1e3 / args.steps, single_config(spec, spec["builder"](use_vbo=False), world),
                "synthetic (seeded; mytinygl_gb300/workloads.py)", desc)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="batch")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline work per thread")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle comparison of the timed frames")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="serving trace length (workload serve)")
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="offered requests/s (workload serve)")
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
