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
    for ret, name, args in re.findall(r"^\s*(const GLubyte \*\s*|\w+\s+)(gl\w+)\(([^)]*)\);", text, re.M):
        ret = ret.strip()
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


def _nbytes(x):
    """Size of a destination array (raw addresses are taken on trust)."""
    return x.nbytes if isinstance(x, np.ndarray) else 1 << 62


class Stats(ctypes.Structure):
    """mtgl_stats (include/mytinygl/mtgl_dev.h)"""
    _fields_ = [(n, ctypes.c_uint64) for n in ("draws", "input_triangles", "setup_triangles", "bin_entries",
                                               "fragments", "passes", "kernel_launches", "staged_bytes",
                                               "allocations", "vertices", "vertex_bytes", "debug_status")]


class BatchConfig(ctypes.Structure):
    """mtgl_batch_config (include/mytinygl/mtgl_dev.h); zero fields take the tuned defaults."""
    _fields_ = [("tile_size", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("record_factor", ctypes.c_float),
                ("pair_factor", ctypes.c_float), ("use_graph", ctypes.c_int32), ("order_by_cost", ctypes.c_int32),
                ("readback_kernel", ctypes.c_int32)]


class BatchStats(ctypes.Structure):
    """mtgl_batch_stats (include/mytinygl/mtgl_dev.h)"""
    _fields_ = [(n, ctypes.c_uint64) for n in ("batches", "frames", "input_triangles", "setup_triangles",
                                               "bin_entries", "fragments", "graph_captures", "graph_replays",
                                               "overflow_reruns", "kernel_launches")] + \
               [("record_capacity", ctypes.c_uint32), ("pair_capacity", ctypes.c_uint32),
                ("tile_size", ctypes.c_int32), ("ctas", ctypes.c_int32),
                ("vertices", ctypes.c_uint64), ("vertex_bytes", ctypes.c_uint64),
                ("debug_status", ctypes.c_uint64)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Timings(ctypes.Structure):
    """mtgl_timings (include/mytinygl/mtgl_dev.h)"""
    _fields_ = [("vertex_ms", ctypes.c_double), ("setup_ms", ctypes.c_double), ("bin_ms", ctypes.c_double),
                ("tile_ms", ctypes.c_double), ("passes", ctypes.c_uint64)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class ServerConfig(ctypes.Structure):
    """mtgl_server_config (include/mytinygl/mtgl_serve.h)"""
    _fields_ = [("memory_budget", ctypes.c_uint64), ("max_batch", ctypes.c_int32), ("executors", ctypes.c_int32),
                ("batch", BatchConfig)]


class Request(ctypes.Structure):
    """mtgl_request (include/mytinygl/mtgl_serve.h)"""
    _fields_ = [("scene", ctypes.c_int32), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("modelview", ctypes.c_float * 16), ("color", ctypes.c_void_p), ("arrival", ctypes.c_double),
                ("admitted", ctypes.c_double), ("finished", ctypes.c_double), ("status", ctypes.c_int32),
                ("batch_size", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    """mtgl_server_stats (include/mytinygl/mtgl_serve.h)"""
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "failed", "batches",
                                               "deferred_for_budget", "peak_bytes_admitted",
                                               "framebuffers_allocated")] + [("busy_seconds", ctypes.c_double),
                                                                             ("kernel_launches", ctypes.c_uint64)]


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
        L.mtgl_get_stats.restype = ctypes.c_int
        L.mtgl_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(Stats)]
        L.mtgl_reset_stats.restype = ctypes.c_int
        L.mtgl_reset_stats.argtypes = [ctypes.c_void_p]
        self.has_player = hasattr(L, "mtgl_play")  # the reference build has none
        if self.has_player:
            L.mtgl_play.restype = ctypes.c_int
            L.mtgl_play.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
            L.mtgl_play_many.restype = ctypes.c_int
            L.mtgl_play_many.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                         ctypes.POINTER(ctypes.c_size_t), ctypes.c_int32]
        self.has_batches = hasattr(L, "mtgl_dev_batch_create")  # the reference build has none
        if self.has_batches:
            self._bind_batches(L)
        self.has_server = hasattr(L, "mtgl_server_create")  # the GB300 library only
        if self.has_server:
            L.mtgl_server_create.restype = ctypes.c_int
            L.mtgl_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]
            L.mtgl_server_destroy.restype = ctypes.c_int
            L.mtgl_server_destroy.argtypes = [ctypes.c_void_p]
            L.mtgl_server_add_scene.restype = ctypes.c_int
            L.mtgl_server_add_scene.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                ctypes.c_uint64]
            L.mtgl_server_now.restype = ctypes.c_double
            L.mtgl_server_now.argtypes = [ctypes.c_void_p]
            L.mtgl_server_submit.restype = ctypes.c_int
            L.mtgl_server_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(Request)]
            L.mtgl_server_drain.restype = ctypes.c_int
            L.mtgl_server_drain.argtypes = [ctypes.c_void_p]
            L.mtgl_server_run_trace.restype = ctypes.c_int
            L.mtgl_server_run_trace.argtypes = [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_int32]
            L.mtgl_server_get_stats.restype = ctypes.c_int
            L.mtgl_server_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ServerStats)]

    @staticmethod
    def _bind_batches(L):
        L.mtgl_dev_batch_defaults.restype = None
        L.mtgl_dev_batch_defaults.argtypes = [ctypes.POINTER(BatchConfig)]
        L.mtgl_dev_batch_create.restype = ctypes.c_int
        L.mtgl_dev_batch_create.argtypes = [ctypes.POINTER(BatchConfig), ctypes.POINTER(ctypes.c_void_p)]
        for n in ("mtgl_dev_batch_destroy", "mtgl_dev_batch_wait", "mtgl_dev_batch_reset_stats"):
            getattr(L, n).restype = ctypes.c_int
            getattr(L, n).argtypes = [ctypes.c_void_p]
        L.mtgl_dev_batch_stats.restype = ctypes.c_int
        L.mtgl_dev_batch_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(BatchStats)]
        L.mtgl_dev_batch_profile.restype = ctypes.c_int
        L.mtgl_dev_batch_profile.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.mtgl_dev_batch_timings.restype = ctypes.c_int
        L.mtgl_dev_batch_timings.argtypes = [ctypes.c_void_p, ctypes.POINTER(Timings)]
        L.mtgl_dev_batch_stream.restype = ctypes.c_void_p
        L.mtgl_dev_batch_stream.argtypes = [ctypes.c_void_p]
        L.mtgl_batch_render.restype = ctypes.c_int
        L.mtgl_batch_render.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32]
        L.mtgl_batch_render_read.restype = ctypes.c_int
        L.mtgl_batch_render_read.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                             ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32]

    @property
    def backend(self) -> str:
        return self.lib.mtgl_backend_name().decode()

    def context(self, width: int, height: int) -> "GLContext":
        return GLContext(self, width, height)

    def play(self, ctx: "GLContext", stream: bytes):
        """Replay an encoded command stream (mytinygl_gb300.gen_play.encode) onto ctx."""
        st = self.lib.mtgl_play(ctx.handle, stream, len(stream))
        if st != 0:
            raise RuntimeError(f"mtgl_play failed with status {st}")

    def play_many(self, contexts, streams):
        """Replay streams[i] onto contexts[i] for every i with one native call."""
        PreparedStreams(self, contexts, streams).play()


    def batch(self, **config) -> "Batch":
        """A batch executor; keyword arguments override fields of mtgl_batch_config."""
        return Batch(self, **config)

    def server(self, memory_budget=0, max_batch=0, executors=0, **batch) -> "Server":
        """A serving loop (mtgl_serve.h); batch keywords override fields of mtgl_batch_config."""
        return Server(self, memory_budget, max_batch, executors, **batch)


class Server:
    """mtgl_server: resident scenes, requests admitted against a memory budget, batched."""

    def __init__(self, glib: GLLibrary, memory_budget=0, max_batch=0, executors=0, **batch):
        self.glib = glib
        cfg = ServerConfig()
        cfg.memory_budget, cfg.max_batch, cfg.executors = memory_budget, max_batch, executors
        glib.lib.mtgl_dev_batch_defaults(ctypes.byref(cfg.batch))
        for k, v in batch.items():
            setattr(cfg.batch, k, v)
        h = ctypes.c_void_p()
        st = glib.lib.mtgl_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            raise RuntimeError(f"mtgl_server_create failed with status {st}")
        self.handle = h.value
        self._keep = []

    def add_scene(self, ctx: "GLContext", stream: bytes, triangles: int) -> int:
        buf = ctypes.create_string_buffer(stream, len(stream))
        self._keep.append((ctx, buf))
        sid = self.glib.lib.mtgl_server_add_scene(self.handle, ctx.handle, buf, len(stream), int(triangles))
        if sid < 0:
            raise RuntimeError(f"mtgl_server_add_scene failed with status {-sid}")
        return sid

    def now(self) -> float:
        return self.glib.lib.mtgl_server_now(self.handle)

    def run_trace(self, reqs):
        """reqs: a ctypes array of Request; returns when all have finished."""
        st = self.glib.lib.mtgl_server_run_trace(self.handle, reqs, len(reqs))
        if st != 0:
            raise RuntimeError(f"mtgl_server_run_trace failed with status {st}")

    def stats(self) -> dict:
        s = ServerStats()
        self.glib.lib.mtgl_server_get_stats(self.handle, ctypes.byref(s))
        return {n: getattr(s, n) for n, _ in ServerStats._fields_}

    def destroy(self):
        if self.handle:
            self.glib.lib.mtgl_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class PreparedStreams:
    """Command streams bound to their contexts once, for replaying with one native call."""

    def __init__(self, glib: GLLibrary, contexts, streams):
        n = len(contexts)
        if len(streams) != n:
            raise ValueError("one stream per context")
        self.glib = glib
        self.contexts = list(contexts)
        self._bufs = [ctypes.create_string_buffer(bytes(s), len(s)) for s in streams]
        self._ctxs = (ctypes.c_void_p * n)(*[c.handle for c in contexts])
        self._ptrs = (ctypes.c_void_p * n)(*[ctypes.addressof(b) for b in self._bufs])
        self._sizes = (ctypes.c_size_t * n)(*[len(s) for s in streams])
        self.n = n

    def play(self):
        st = self.glib.lib.mtgl_play_many(self._ctxs, self._ptrs, self._sizes, self.n)
        if st != 0:
            raise RuntimeError(f"mtgl_play_many failed with status {st}")


class Batch:
    """mtgl_batch: renders many contexts' pending frames in one pipeline run."""

    def __init__(self, glib: GLLibrary, **config):
        self.glib = glib
        cfg = BatchConfig()
        glib.lib.mtgl_dev_batch_defaults(ctypes.byref(cfg))
        for k, v in config.items():
            setattr(cfg, k, v)
        self.config = cfg
        h = ctypes.c_void_p()
        st = glib.lib.mtgl_dev_batch_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            raise RuntimeError(f"mtgl_dev_batch_create failed with status {st}")
        self.handle = h.value

    def render(self, contexts, colors=None):
        """mtgl_batch_render; with `colors` (one host array or None per context, uint32
        [height, width], page-locked for asynchronous copies: mtgl_batch_render_read), each
        listed colour buffer is copied out after the run (landed when wait() returns)."""
        n = len(contexts)
        arr = (ctypes.c_void_p * n)(*[c.handle for c in contexts])
        if colors is None:
            st = self.glib.lib.mtgl_batch_render(self.handle, arr, n)
        else:
            if len(colors) != n:
                raise ValueError("one colour destination (or None) per context")
            for c, h in zip(contexts, colors):
                if h is not None and _nbytes(h) < 4 * c.width * c.height:
                    raise ValueError("colour destination smaller than the framebuffer")
            dst = (ctypes.c_void_p * n)(*[_ptr(h) if h is not None else None for h in colors])
            st = self.glib.lib.mtgl_batch_render_read(self.handle, arr, dst, n)
        if st != 0:
            raise RuntimeError(f"mtgl_batch_render failed with status {st}")

    def wait(self):
        st = self.glib.lib.mtgl_dev_batch_wait(self.handle)
        if st != 0:
            raise RuntimeError(f"mtgl_dev_batch_wait failed with status {st}")

    def stats(self) -> dict:
        s = BatchStats()
        st = self.glib.lib.mtgl_dev_batch_stats(self.handle, ctypes.byref(s))
        if st != 0:
            raise RuntimeError(f"mtgl_dev_batch_stats failed with status {st}")
        return s.as_dict()

    def reset_stats(self):
        self.glib.lib.mtgl_dev_batch_reset_stats(self.handle)

    def profile(self, enable: bool):
        self.glib.lib.mtgl_dev_batch_profile(self.handle, 1 if enable else 0)

    def timings(self) -> dict:
        t = Timings()
        st = self.glib.lib.mtgl_dev_batch_timings(self.handle, ctypes.byref(t))
        if st != 0:
            raise RuntimeError(f"mtgl_dev_batch_timings failed with status {st}")
        return t.as_dict()

    @property
    def stream(self) -> int:
        return self.glib.lib.mtgl_dev_batch_stream(self.handle) or 0

    def destroy(self):
        if self.handle:
            self.glib.lib.mtgl_dev_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


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

    def stats(self) -> dict:
        """mtgl_get_stats (synchronises)"""
        s = Stats()
        st = self.glib.lib.mtgl_get_stats(self.handle, ctypes.byref(s))
        if st != 0:
            raise RuntimeError(f"mtgl_get_stats failed with status {st}")
        return {n: getattr(s, n) for n, _ in Stats._fields_}

    def reset_stats(self):
        self.glib.lib.mtgl_reset_stats(self.handle)


_lib_cache: dict = {}
_lib_lock = threading.Lock()


def load(path: str) -> GLLibrary:
    with _lib_lock:
        if path not in _lib_cache:
            _lib_cache[path] = GLLibrary(path)
        return _lib_cache[path]
