"""Autotuner of the batched renderer: tile size, persistent CTAs per SM, work order (costliest
tiles first, or frame order) and the record / tile-pair capacity factors, measured on the
uneven-batch workload on this GPU.

    python -m mytinygl_gb300.autotune [--frames 256] [--steps 5]

Writes mytinygl_gb300/tuned.json (every configuration measured) and csrc/dev/tuned.h (the
defaults mtgl_dev_batch_defaults returns; rebuild the library afterwards). A configuration
is timed on the host clock around mtgl_batch_render + mtgl_dev_batch_wait with the frames'
GL calls already queued, so the figure includes the submission's host work and the whole
device pipeline (graph replay), which is what a caller waits for.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import time

from . import build, library
from . import workloads as W
from .gl import PreparedStreams

HERE = os.path.dirname(os.path.abspath(__file__))
TUNED_JSON = os.path.join(HERE, "tuned.json")
TUNED_H = os.path.join(HERE, "csrc", "dev", "tuned.h")


def setup(lib, scenes):
    ctxs, streams = [], []
    for sc in scenes:
        c = lib.context(sc.width, sc.height)
        k = W.frame_start(sc)
        sc.play(c, 0, k)
        ctxs.append(c)
        streams.append(sc.stream(k))
    for c in ctxs:
        c.glFinish()
    return ctxs, PreparedStreams(lib, ctxs, streams)


def time_config(lib, ctxs, streams, steps, **cfg):
    b = lib.batch(**cfg)
    for _ in range(2):  # capture, learn capacities
        streams.play()
        b.render(ctxs)
        b.wait()
    times = []
    for _ in range(steps):
        streams.play()
        t0 = time.perf_counter()
        b.render(ctxs)
        b.wait()
        times.append(time.perf_counter() - t0)
    st = b.stats()
    b.destroy()
    return statistics.median(times) * 1e3, st


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--frames", type=int, default=256)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--seed", type=int, default=3)
    args = ap.parse_args()
    build()
    lib = library()
    scenes = W.uneven_batch(args.frames, seed=args.seed)
    ctxs, streams = setup(lib, scenes)
    tris = sum(W.scene_triangles(s) for s in scenes)
    results = []
    for tile in (8, 16, 32):
        for ctas in (0, 1, 2, 4, 8):
            if tile == 32 and ctas > 1:
                continue  # a 32x32 CTA is 1024 threads: one fits an SM
            for order in (1, 0):
                ms, st = time_config(lib, ctxs, streams, args.steps, tile_size=tile, ctas_per_sm=ctas,
                                     order_by_cost=order)
                r = dict(tile_size=tile, ctas_per_sm=ctas, order_by_cost=order, ms=round(ms, 3),
                         frames_per_s=round(args.frames / (ms / 1e3), 1), persistent_ctas=st["ctas"],
                         records=st["setup_triangles"] // max(1, st["batches"]),
                         pairs=st["bin_entries"] // max(1, st["batches"]))
                results.append(r)
                print(json.dumps(r), flush=True)
    best = min(results, key=lambda r: r["ms"])
    # capacity factors: the measured totals of the best tile size with 1/8 headroom
    rec_factor = math.ceil(best["records"] / max(1, tris) * 1.125 * 100) / 100
    pair_factor = math.ceil(best["pairs"] / max(1, best["records"]) * 1.125 * 10) / 10
    out = {"workload": f"uneven_batch({args.frames}, seed={args.seed})", "input_triangles": tris,
           "best": best, "record_factor": rec_factor, "pair_factor": pair_factor, "results": results}
    with open(TUNED_JSON, "w") as f:
        json.dump(out, f, indent=1)
    with open(TUNED_H, "w") as f:
        f.write("// tuned.h — batch defaults chosen by mytinygl_gb300/autotune.py on a GB300 (the full sweep\n"
                "// is in mytinygl_gb300/tuned.json). Regenerate with that script; do not edit by hand.\n"
                "#pragma once\n"
                f"#define MTGL_TUNED_TILE_SIZE {best['tile_size']}\n"
                f"#define MTGL_TUNED_CTAS_PER_SM {best['ctas_per_sm']}\n"
                f"#define MTGL_TUNED_ORDER_BY_COST {best['order_by_cost']}\n"
                f"#define MTGL_TUNED_RECORD_FACTOR {rec_factor:.2f}f\n"
                f"#define MTGL_TUNED_PAIR_FACTOR {pair_factor:.1f}f\n")
    print(json.dumps({"best": best, "record_factor": rec_factor, "pair_factor": pair_factor}))
    for c in ctxs:
        c.destroy()


if __name__ == "__main__":
    main()
