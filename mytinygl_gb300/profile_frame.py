"""Renders one benchmark workload's frame a few times in a row, for profilers.

    python -m mytinygl_gb300.profile_frame --workload textured --frames 3
    python -m mytinygl_gb300.profile_frame --workload batch --frames 3 [--batch-frames 256]

Each frame is the workload's per-frame GL calls followed by glFinish, on one context, with
nothing else on the GPU in between (no cache flush, no timing events), so a profiler's
capture of the n-th frame's kernels sees what the previous frame left in L2 and nothing
else. `batch` renders the uneven batch of bench.py (256 contexts, one mtgl_batch_render per
repetition, the batch's defaults). Workloads are those of mytinygl_gb300/workloads.py.
"""
from __future__ import annotations

import argparse

from . import library
from . import workloads as W

SCENES = {
    "textured": W.textured_scene,
    "rop": W.rop_scene,
    "sphere": W.sphere_scene,
}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--workload", choices=sorted(SCENES) + ["batch"], default="textured")
    ap.add_argument("--frames", type=int, default=3, help="repetitions")
    ap.add_argument("--batch-frames", type=int, default=256)
    args = ap.parse_args()
    lib = library()
    if args.workload == "batch":
        scenes = W.uneven_batch(args.batch_frames)
        ctxs, streams = [], []
        for sc in scenes:
            c = lib.context(sc.width, sc.height)
            k = W.frame_start(sc)
            sc.play(c, 0, k)
            c.glFinish()
            ctxs.append(c)
            streams.append(sc.stream(k))
        b = lib.batch()
        for _ in range(args.frames):
            lib.play_many(ctxs, streams)
            b.render(ctxs)
            b.wait()
        print(f"batch of {len(scenes)}: {args.frames} runs, stats {b.stats()}")
        b.destroy()
        for c in ctxs:
            c.destroy()
        return
    scene = SCENES[args.workload]()
    fs = W.frame_start(scene)
    ctx = lib.context(scene.width, scene.height)
    scene.play(ctx, 0, fs)
    ctx.glFinish()
    for _ in range(args.frames):
        scene.play(ctx, fs)
        ctx.glFinish()
    print(f"{args.workload}: {args.frames} frames, stats {ctx.stats()}")
    ctx.destroy()


if __name__ == "__main__":
    main()
