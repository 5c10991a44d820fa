"""Regenerate the golden fixtures from the reference itself.

Each fixture stores a scene script (every matrix and vertex as data, so it replays
bit-identically on any host) and the framebuffer MyTinyGL renders for it, compiled from
its own sources with the reference's strict numerics (oracle/Makefile, target `ref`).
Run here, where the reference sources exist:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import harness  # noqa: E402
import feature_scenes as F  # noqa: E402
from mytinygl_gb300 import workloads as W  # noqa: E402
from mytinygl_gb300.scene import render  # noqa: E402


def golden_scenes():
    for name, (builder, flags) in F.SCENES.items():
        yield name, builder()
    yield "headline_sphere_small", W.sphere_scene(200, 150, seed=0)
    yield "headline_textured_small", W.textured_scene(240, 136, ntri=3000, seed=1, tex_size=64)
    yield "headline_rop_small", W.rop_scene(240, 136, ntri=20000, seed=2)


def main():
    ref = harness.reference()
    if ref is None:
        sys.exit("reference sources not found; fixtures can only be generated where they exist")
    for name, scene in golden_scenes():
        c, d, s, err = render(ref, scene)
        bufs = harness.cleared_buffers(scene)
        # a buffer the scene never clears holds the reference's uninitialised memory: store zeros
        c, d, s = (x if bufs[k] else np.zeros_like(x) for x, k in ((c, "color"), (d, "depth"), (s, "stencil")))
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, scene=np.frombuffer(scene.to_bytes(), np.uint8), color=c, depth=d, stencil=s,
                            error=np.int64(err), defined_color=bufs["color"], defined_depth=bufs["depth"],
                            defined_stencil=bufs["stencil"])
        print(f"{name}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
