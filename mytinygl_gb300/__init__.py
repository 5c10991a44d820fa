"""mytinygl_gb300 — MyTinyGL's OpenGL 1.5 fixed-function pipeline on a GB300 (sm_103a).

The product is libmytinygl_gb300.so (C ABI: include/GL/gl.h, include/mytinygl/*.h). This
package builds it in-tree and offers a ctypes binding (`gl`), scene scripts (`scene`) and
the seeded synthetic workloads (`workloads`) used by the benchmark and the tests.
"""
import os

from . import build as _build

LIB_PATH = _build.LIB_PATH


def build(verbose=False, force=False, debug_bounds=False) -> str:
    return _build.build(verbose=verbose, force=force, debug_bounds=debug_bounds)


def library(debug_bounds=False):
    """Load libmytinygl_gb300.so (debug_bounds: libmytinygl_gb300_debug.so, the build whose
    kernels check their indices). There is no CPU fallback: a missing library is an error,
    and creating a context without a visible CUDA device fails."""
    from . import gl

    path = _build.DEBUG_LIB_PATH if debug_bounds else LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built; run mytinygl_gb300.build() (nvcc, sm_103a)")
    return gl.load(path)
