"""ctypes binding of the OpenGL 1.5 C ABI (include/GL/gl.h) for any library that exports it.

The same binding drives libmytinygl_gb300.so (the GB300 back end), the CPU oracle and
MyTinyGL itself, so one scene script renders through all three. Prototypes and enum values
are parsed from this repository's include/GL/gl.h; the context API is
include/mytinygl/mytinygl.h (src/mytinygl.h:228-233 in the reference).
"""
from __future__ import annotations

import ctypes
import os
import re
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(_HERE)
GL_HEADER = os.path.join(REPO, "include", "GL", "gl.h")

_CTYPE = {
    "GLenum": ctypes.c_uint,
    "GLboolean": ctypes.c_ubyte,
    "GLbitfield": ctypes.c_uint,
    "GLbyte": ctypes.c_byte,
    "GLshort": ctypes.c_short,
    "GLint": ctypes.c_int,
    "GLubyte": ctypes.c_ubyte,
    "GLushort": ctypes.c_ushort,
    "GLuint": ctypes.c_uint,
    "GLsizei": ctypes.c_int,
    "GLfloat": ctypes.c_float,
    "GLclampf": ctypes.c_float,
    "GLdouble": ctypes.c_double,
    "GLclampd": ctypes.c_double,
    "GLsizeiptr": ctypes.c_long,
    "GLintptr": ctypes.c_long,
    "void": None,
}


def _parse_header(path=GL_HEADER):
    text = open(path).read()
    enums = {}
    for name, val in re.findall(r"^#define\s+(GL_\w+)\s+(0x[0-9A-Fa-f]+|\d+)", text, re.M):
        enums[name] = int(val, 0)
    protos = {}
    for ret, name, args in re.findall(r"^\s*(const GLubyte \*|\w+)\s+(gl\w+)\(([^)]*)\);", text, re.M):
        if ret.startswith("const GLubyte"):
            restype = ctypes.c_char_p
        else:
            restype = _CTYPE[ret]
        argtypes = []
        args = args.strip()
        if args and args != "void":
            for a in args.split(","):
                a = a.strip()
                if "*" in a:
                    argtypes.append(ctypes.c_void_p)
                else:
                    argtypes.append(_CTYPE[a.split()[0]])
        protos[name] = (restype, argtypes)
    return enums, protos


ENUMS, PROTOS = _parse_header()
globals().update(ENUMS)


def _ptr(x):
    """Pointer argument: numpy arrays by address, ints as raw addresses (buffer offsets)."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays passed to GL must be C-contiguous")
        return x.ctypes.data
    if isinstance(x, (bytes, bytearray)):
        return ctypes.cast(ctypes.c_char_p(bytes(x)), ctypes.c_void_p).value
    return int(x)


class GLLibrary:
    """One loaded GL implementation (a shared library exporting include/GL/gl.h)."""

    def __init__(self, path: str):
        self.path = path
        self.lib = ctypes.CDLL(path, mode=os.RTLD_LOCAL | os.RTLD_NOW)
        for name, (res, args) in PROTOS.items():
            f = getattr(self.lib, name)
            f.restype = res
            f.argtypes = args
        L = self.lib
        L.gl_create_context.restype = ctypes.c_void_p
        L.gl_create_context.argtypes = [ctypes.c_int32, ctypes.c_int32]
        L.gl_destroy_context.restype = None
        L.gl_destroy_context.argtypes = [ctypes.c_void_p]
        L.gl_make_current.restype = None
        L.gl_make_current.argtypes = [ctypes.c_void_p]
        L.gl_get_current_context.restype = ctypes.c_void_p
        L.gl_get_current_context.argtypes = []
        L.mtgl_read_framebuffer.restype = ctypes.c_int
        L.mtgl_read_framebuffer.argtypes = [ctypes.c_void_p] * 4
        L.mtgl_finish.restype = ctypes.c_int
        L.mtgl_finish.argtypes = [ctypes.c_void_p]
        L.mtgl_backend_name.restype = ctypes.c_char_p
        L.mtgl_backend_name.argtypes = []

    @property
    def backend(self) -> str:
        return self.lib.mtgl_backend_name().decode()

    def context(self, width: int, height: int) -> "GLContext":
        return GLContext(self, width, height)


class GLContext:
    """A context of one library plus a call interface: ctx.glClear(...), ctx.call(name, *args)."""

    def __init__(self, glib: GLLibrary, width: int, height: int):
        self.glib = glib
        self.width, self.height = int(width), int(height)
        h = glib.lib.gl_create_context(self.width, self.height)
        if not h:
            raise RuntimeError(f"gl_create_context({width}, {height}) failed in {glib.path}")
        self.handle = h
        self._keep = []  # arrays referenced by stored vertex-array pointers
        self.make_current()

    def make_current(self):
        self.glib.lib.gl_make_current(self.handle)

    def destroy(self):
        if self.handle:
            if self.glib.lib.gl_get_current_context() == self.handle:
                self.glib.lib.gl_make_current(None)
            self.glib.lib.gl_destroy_context(self.handle)
            self.handle = None
            self._keep = []

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def call(self, name, *args):
        fn = getattr(self.glib.lib, name)
        _, argtypes = PROTOS[name]
        conv = []
        for a, t in zip(args, argtypes):
            if t is ctypes.c_void_p:
                if isinstance(a, np.ndarray):
                    self._keep.append(a)
                conv.append(_ptr(a))
            else:
                conv.append(a)
        return fn(*conv)

    def __getattr__(self, name):
        if name.startswith("gl") and name in PROTOS:
            return lambda *a: self.call(name, *a)
        raise AttributeError(name)

    def finish(self):
        return self.glib.lib.mtgl_finish(self.handle)

    def read(self, color=True, depth=True, stencil=True):
        """Synchronise and return (color u32 [h,w], depth f32 [h,w], stencil u8 [h,w]); row 0 = top."""
        n = (self.height, self.width)
        c = np.empty(n, np.uint32) if color else None
        d = np.empty(n, np.float32) if depth else None
        s = np.empty(n, np.uint8) if stencil else None
        st = self.glib.lib.mtgl_read_framebuffer(self.handle, _ptr(c), _ptr(d), _ptr(s))
        if st != 0:
            raise RuntimeError(f"mtgl_read_framebuffer failed with status {st}")
        return c, d, s

    def forget_arrays(self):
        self._keep = []


_lib_cache: dict = {}
_lib_lock = threading.Lock()


def load(path: str) -> GLLibrary:
    with _lib_lock:
        if path not in _lib_cache:
            _lib_cache[path] = GLLibrary(path)
        return _lib_cache[path]
