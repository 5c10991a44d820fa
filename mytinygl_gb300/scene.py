"""Scene scripts: recorded GL call sequences that replay through any GL library.

A Scene is an ordered list of (entry point, arguments). Arrays are numpy arrays (passed by
pointer, kept alive for the whole replay, as client vertex arrays must be). Scenes
serialise to a JSON call list plus an .npz of arrays, which is how golden fixtures store
their inputs: a fixture replays bit-identically on any host because every matrix and
vertex is stored, not recomputed.
"""
from __future__ import annotations

import io
import json
import zipfile

import numpy as np

from . import gl as G


class Scene:
    def __init__(self, name: str, width: int, height: int):
        self.name = name
        self.width = int(width)
        self.height = int(height)
        self.cmds: list = []

    def __getattr__(self, name):
        if name.startswith("gl") and name in G.PROTOS:
            def rec(*args):
                self.cmds.append((name, tuple(args)))
            return rec
        raise AttributeError(name)

    def add(self, name, *args):
        self.cmds.append((name, tuple(args)))

    def play(self, ctx, start=0, stop=None):
        """Replays the calls [start, stop) on ctx, made current on this thread first."""
        ctx.make_current()
        for name, args in self.cmds[start:stop]:
            ctx.call(name, *args)

    def stream(self, start=0, stop=None) -> bytes:
        """The calls [start, stop) as a native command stream (mtgl_play). Arrays are passed
        by address, so the scene must outlive every replay of the stream."""
        from .gen_play import encode
        return encode(self.cmds[start:stop])

    # ---- serialisation -------------------------------------------------------------
    def to_bytes(self) -> bytes:
        arrays = {}
        calls = []
        for name, args in self.cmds:
            enc = []
            for a in args:
                if isinstance(a, np.ndarray):
                    key = f"a{len(arrays)}"
                    arrays[key] = a
                    enc.append({"array": key})
                elif isinstance(a, (float, np.floating)):
                    enc.append({"f": float.hex(float(a))})
                elif a is None:
                    enc.append(None)
                else:
                    enc.append(int(a))
            calls.append([name, enc])
        meta = {"name": self.name, "width": self.width, "height": self.height, "calls": calls}
        buf = io.BytesIO()
        arr = io.BytesIO()
        np.savez(arr, **arrays)
        # fixed member dates keep the bytes a function of the script alone
        with zipfile.ZipFile(buf, "w", zipfile.ZIP_DEFLATED) as z:
            for member, data in (("scene.json", json.dumps(meta).encode()), ("arrays.npz", arr.getvalue())):
                info = zipfile.ZipInfo(member, date_time=(1980, 1, 1, 0, 0, 0))
                info.compress_type = zipfile.ZIP_DEFLATED
                z.writestr(info, data)
        return buf.getvalue()

    @staticmethod
    def from_bytes(data: bytes) -> "Scene":
        with zipfile.ZipFile(io.BytesIO(data)) as z:
            meta = json.loads(z.read("scene.json"))
            arrays = np.load(io.BytesIO(z.read("arrays.npz")))
            s = Scene(meta["name"], meta["width"], meta["height"])
            for name, enc in meta["calls"]:
                args = []
                for a in enc:
                    if isinstance(a, dict) and "array" in a:
                        args.append(np.ascontiguousarray(arrays[a["array"]]))
                    elif isinstance(a, dict) and "f" in a:
                        args.append(float.fromhex(a["f"]))
                    else:
                        args.append(a)
                s.cmds.append((name, tuple(args)))
        return s


def render(glib: "G.GLLibrary", scene: Scene):
    """Render a scene in a fresh context; return (color, depth, stencil) numpy arrays."""
    ctx = glib.context(scene.width, scene.height)
    try:
        scene.play(ctx)
        c, d, s = ctx.read()
        err = ctx.glGetError()
        return c, d, s, err
    finally:
        ctx.destroy()
