"""The drop-in boundary: header parity with the reference and the exported C ABI (CPU only)."""
import ctypes
import os
import re

import pytest

import harness

INCLUDE = os.path.join(harness.REPO, "include")


def declared_functions(headers=("GL/gl.h", "mytinygl/mytinygl.h", "mytinygl/mtgl_dev.h")):
    """Every extern function declared by the given headers under include/ (default: the GL
    API, the context API and the back-end ABI, which the oracle exports too)."""
    names = set()
    for rel in headers:
        text = open(os.path.join(INCLUDE, rel)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b((?:gl|mtgl)\w*)\s*\(", text, re.M):
            if "static inline" in text[max(0, m.start() - 30):m.start() + 14]:
                continue
            names.add(m.group(1))
    return sorted(names)


def test_declares_the_reference_api():
    names = declared_functions()
    gl = [n for n in names if n.startswith("gl") and not n.startswith("gl_")]
    assert len(gl) == 111, len(gl)
    for n in ("gl_create_context", "gl_destroy_context", "gl_make_current", "gl_get_current_context"):
        assert n in names


def test_gl_header_matches_reference_enums_and_prototypes():
    root = harness.reference_root()
    ref_h = os.path.join(root, "include", "GL", "gl.h") if root else ""
    if not root or not os.path.exists(ref_h):
        pytest.skip("reference headers not present")
    def enums(path):
        return {n: int(v, 0) for n, v in re.findall(r"^#define\s+(GL_\w+)\s+(0x[0-9A-Fa-f]+|\d+)", open(path).read(), re.M)}
    mine, ref = enums(os.path.join(INCLUDE, "GL", "gl.h")), enums(ref_h)
    assert set(ref) <= set(mine)
    assert {n: mine[n] for n in ref} == ref

    def protos(path):
        text = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
        out = {}
        for ret, name, args in re.findall(r"^\s*(const GLubyte \*|\w+)\s+(gl\w+)\((.*?)\);", text, re.M | re.S):
            types = [re.sub(r"\s+\w+$", "", a.strip()).replace(" ", "") for a in args.split(",")]
            out[name] = (ret.replace(" ", ""), types)
        return out
    assert protos(os.path.join(INCLUDE, "GL", "gl.h")) == protos(ref_h)


def test_library_exports_every_declared_symbol():
    lib_path = harness.product().path
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_functions() + declared_functions(("mytinygl/mtgl_serve.h",))
               if not hasattr(lib, n)]
    assert not missing, missing


def test_oracle_exports_the_same_gl_api():
    lib = ctypes.CDLL(harness.oracle().path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_no_gpu_means_no_context():
    """Without a visible CUDA device the product refuses to create a context (no CPU fallback)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    lib = harness.product()
    assert lib.backend == "cuda-sm_103a"
    assert lib.lib.gl_create_context(64, 64) is None
