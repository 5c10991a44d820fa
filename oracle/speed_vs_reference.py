#!/usr/bin/env python3
"""TEST INFRASTRUCTURE ONLY: how fast the CPU oracle renders compared with MyTinyGL itself.

The benchmark's CPU baseline and reference arm time the oracle (oracle_backend.c behind this
repository's C99 front end), because the reference's sources do not travel to the GPU host.
This script ties that figure to the reference: it renders the same seeded frames, one thread,
with the oracle and with the reference compiled from its own sources (oracle/Makefile `ref`),
each in the strict build (-O2 -ffp-contract=off) and in the reference's shipped flags
(-O3 -ffast-math), and prints per-workload frame times and the oracle/reference ratio as a
markdown table. Frames are checked to match between the two strict builds.

    python oracle/speed_vs_reference.py [--reps N]
"""
import argparse
import os
import platform
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

from mytinygl_gb300 import gl as G  # noqa: E402
from mytinygl_gb300 import workloads as W  # noqa: E402

LIBS = {
    "oracle": ("all", "_build/libmtgl_oracle.so"),
    "oracle, shipped flags": ("shipped", "_build/libmtgl_oracle_shipped.so"),
    "reference": ("ref", "_ref/libmtgl_ref.so"),
    "reference, shipped flags": ("ref-shipped", "_ref/libmtgl_ref_shipped.so"),
}


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def frame_seconds(lib, scene, reps):
    """Median time of the frame part (glClear .. last draw), the resident part played once."""
    k = W.frame_start(scene)
    c = lib.context(scene.width, scene.height)
    scene.play(c, 0, k)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        scene.play(c, k)
        c.glFinish()
        times.append(time.perf_counter() - t0)
    out = c.read()
    c.destroy()
    return float(np.median(times)), out


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    if subprocess.run(["make", "-s", "-C", HERE, "has-ref"], capture_output=True).returncode != 0:
        sys.exit("the reference's sources are not present (set MTGL_REF_SRC)")
    libs = {}
    for name, (target, path) in LIBS.items():
        subprocess.run(["make", "-s", "-C", HERE, target], check=True, capture_output=True)
        libs[name] = G.load(os.path.join(HERE, path))
    batch = W.uneven_batch(256, use_vbo=False)[::8]
    work = [
        ("sphere 800x600, 1,984 triangles", [W.sphere_scene(use_vbo=False)], 20),
        ("textured 1920x1080, 100k triangles", [W.textured_scene(use_vbo=False)], 1),
        ("rop 1920x1080, 1M triangles", [W.rop_scene(use_vbo=False)], 1),
        (f"uneven batch, every 8th frame ({len(batch)} frames)", batch, 1),
    ]
    print(f"CPU: {cpu_model()}, one thread; frame part only (resident uploads untimed); median of reps\n")
    print("| workload | " + " | ".join(f"{n} (ms/frame)" for n in LIBS) + " | oracle / reference | "
          "oracle / reference, shipped flags |")
    print("|---|" + "---:|" * (len(LIBS) + 2))
    for label, scenes, reps in work:
        reps = max(1, reps * args.reps // 3)
        tot = {}
        for name, lib in libs.items():
            t = 0.0
            for sc in scenes:
                dt, out = frame_seconds(lib, sc, reps)
                t += dt
                if name == "oracle":
                    sc._oracle_out = out
                elif name == "reference":
                    # buffers the frame clears (the reference leaves the others uninitialised)
                    bits = 0
                    for cname, a in sc.cmds[W.frame_start(sc):]:
                        if cname == "glClear":
                            bits |= int(a[0])
                    keep = [bits & G.GL_COLOR_BUFFER_BIT, bits & G.GL_DEPTH_BUFFER_BIT, bits & G.GL_STENCIL_BUFFER_BIT]
                    same = all(np.array_equal(a.view(np.uint8), b.view(np.uint8))
                               for a, b, k in zip(sc._oracle_out, out, keep) if k)
                    assert same, f"{sc.name}: oracle and reference frames differ"
            tot[name] = t / len(scenes)
        cells = " | ".join(f"{tot[n] * 1e3:.2f}" for n in LIBS)
        r1 = tot["oracle"] / tot["reference"]
        r2 = tot["oracle, shipped flags"] / tot["reference, shipped flags"]
        print(f"| {label} | {cells} | {r1:.3f} | {r2:.3f} |", flush=True)


if __name__ == "__main__":
    main()
