"""Test harness: locating/building the three GL implementations and comparing framebuffers.

  product   mytinygl_gb300/lib/libmytinygl_gb300.so  (the GB300 back end under test)
  oracle    oracle/_build/libmtgl_oracle.so          (CPU restatement of the reference: the checker)
  reference oracle/_ref/libmtgl_ref.so               (MyTinyGL itself; only where its sources exist)
"""
from __future__ import annotations

import os
import subprocess

import numpy as np

from mytinygl_gb300 import gl as G
from mytinygl_gb300.scene import Scene

TESTS = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(TESTS)
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libmtgl_oracle.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libmtgl_ref.so")
GOLDEN_DIR = os.path.join(TESTS, "golden")


def oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True, capture_output=True)
    return G.load(ORACLE_LIB)


def reference_root():
    """The reference checkout's root directory, or None where its sources are not present
    (oracle/Makefile knows where to look; MTGL_REF_SRC overrides it)."""
    r = subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref-dir"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 and r.stdout.strip() else None


def has_reference_sources():
    return reference_root() is not None


def reference():
    """The reference build, or None where its sources are not present."""
    if not has_reference_sources():
        return None
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref"], check=True, capture_output=True)
    return G.load(REF_LIB)


def product():
    import mytinygl_gb300 as M

    M.build()
    return M.library()


def cleared_buffers(scene: Scene):
    """Buffers the scene clears (the reference leaves uncleared buffers uninitialised)."""
    bits = 0
    for name, args in scene.cmds:
        if name == "glClear":
            bits |= int(args[0])
    return {
        "color": bool(bits & G.GL_COLOR_BUFFER_BIT),
        "depth": bool(bits & G.GL_DEPTH_BUFFER_BIT),
        "stencil": bool(bits & G.GL_STENCIL_BUFFER_BIT),
    }


def depth_equal(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Bitwise depth equality; any NaN equals any NaN (NaN payloads differ between CPUs and GPUs)."""
    same = a.view(np.uint32) == b.view(np.uint32)
    return same | (np.isnan(a) & np.isnan(b))


def compare(a, b, buffers=None):
    """a, b: (color u32, depth f32, stencil u8, gl_error). Returns parity statistics."""
    buffers = buffers or {"color": True, "depth": True, "stencil": True}
    out = {"error_equal": int(a[3]) == int(b[3])}
    if buffers["color"]:
        ca = a[0].view(np.uint8).reshape(*a[0].shape, 4).astype(np.int16)
        cb = b[0].view(np.uint8).reshape(*b[0].shape, 4).astype(np.int16)
        d = np.abs(ca - cb)
        out["color_max_err"] = int(d.max()) if d.size else 0
        out["color_mismatch_frac"] = float((d.max(axis=-1) > 0).mean()) if d.size else 0.0
    if buffers["depth"]:
        eq = depth_equal(a[1], b[1])
        out["depth_mismatches"] = int((~eq).sum())
    if buffers["stencil"]:
        out["stencil_mismatches"] = int((a[2] != b[2]).sum())
    return out


def assert_parity(stats, color_tol=1, name=""):
    assert stats["error_equal"], f"{name}: glGetError differs"
    if "depth_mismatches" in stats:
        assert stats["depth_mismatches"] == 0, f"{name}: depth differs at {stats['depth_mismatches']} pixels"
    if "stencil_mismatches" in stats:
        assert stats["stencil_mismatches"] == 0, f"{name}: stencil differs at {stats['stencil_mismatches']} pixels"
    if "color_max_err" in stats:
        assert stats["color_max_err"] <= color_tol, (
            f"{name}: colour error {stats['color_max_err']} LSB > {color_tol} "
            f"(mismatching fraction {stats['color_mismatch_frac']:.2e})")


def load_golden(path):
    z = np.load(path, allow_pickle=False)
    scene = Scene.from_bytes(z["scene"].tobytes())
    out = (z["color"], z["depth"], z["stencil"], int(z["error"]))
    buffers = {k: bool(z[f"defined_{k}"]) for k in ("color", "depth", "stencil")}
    return scene, out, buffers


def golden_files():
    return sorted(os.path.join(GOLDEN_DIR, f) for f in os.listdir(GOLDEN_DIR) if f.endswith(".npz"))
