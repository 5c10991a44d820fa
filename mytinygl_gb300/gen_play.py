"""Generates csrc/front/fe_play.c: the native player of GL command streams.

A command stream is a byte string of records, each `u32 function id, u32 argument count`
followed by one 8-byte slot per argument (int64 for integer, enum and pointer arguments,
IEEE double for float and double arguments). Function ids index the GL entry points of
include/GL/gl.h in sorted name order (`FUNCTIONS`). mtgl_play replays a stream onto a
context in native code, so a frame's GL calls cost no Python round trips per call.

Run `python -m mytinygl_gb300.gen_play` after changing include/GL/gl.h; the test suite
checks that the committed file is current.
"""
from __future__ import annotations

import os
import re
import struct

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
GL_HEADER = os.path.join(os.path.dirname(_HERE), "include", "GL", "gl.h")
OUT = os.path.join(_HERE, "csrc", "front", "fe_play.c")

_FLOAT = {"GLfloat", "GLclampf", "GLdouble", "GLclampd"}


def prototypes(path=GL_HEADER):
    """name -> list of (declared type text, is_float, is_pointer), in header order."""
    text = open(path).read()
    out = {}
    for _ret, name, args in re.findall(r"^\s*(const GLubyte \*\s*|\w+\s+)(gl\w+)\(([^)]*)\);", text, re.M):
        params = []
        args = args.strip()
        if args and args != "void":
            for a in args.split(","):
                a = a.strip()
                if "*" in a:
                    ctype = a[:a.rindex("*") + 1].strip()
                    params.append((ctype, False, True))
                else:
                    ctype = a.split()[0]
                    params.append((ctype, ctype in _FLOAT, False))
        out[name] = params
    return out


PROTOS = prototypes()
FUNCTIONS = sorted(PROTOS)
FUNCTION_ID = {n: i for i, n in enumerate(FUNCTIONS)}


def encode(calls) -> bytes:
    """Encode (name, args) pairs. Arrays are passed by address: the caller keeps them alive
    for as long as the stream is played."""
    out = bytearray()
    for name, args in calls:
        params = PROTOS[name]
        if len(args) != len(params):
            raise ValueError(f"{name}: {len(args)} arguments, expected {len(params)}")
        out += struct.pack("<II", FUNCTION_ID[name], len(args))
        for a, (_, is_float, is_ptr) in zip(args, params):
            if is_ptr:
                if a is None:
                    v = 0
                elif isinstance(a, np.ndarray):
                    if not a.flags["C_CONTIGUOUS"]:
                        raise ValueError("arrays passed to GL must be C-contiguous")
                    v = a.ctypes.data
                else:
                    v = int(a)
                out += struct.pack("<Q", v)
            elif is_float:
                out += struct.pack("<d", float(a))
            else:
                out += struct.pack("<q", int(a))
    return bytes(out)


def _arg(i, ctype, is_float, is_ptr):
    if is_ptr:
        return f"({ctype})(uintptr_t)a[{i}].i"
    if is_float:
        return f"({ctype})a[{i}].f"
    return f"({ctype})a[{i}].i"


def generate() -> str:
    lines = [
        "/* fe_play.c — GENERATED by mytinygl_gb300/gen_play.py from include/GL/gl.h; do not edit.",
        " *",
        " * Native player of GL command streams (no counterpart in the reference). A stream is a",
        " * sequence of records: u32 function id (index of the entry point in sorted name order),",
        " * u32 argument count, then one 8-byte slot per argument: int64 for integers, enums and",
        " * pointers, IEEE double for GLfloat/GLdouble arguments. Playing a stream calls the same",
        " * public entry points an application would, in order, on the given context. */",
        "#include <stdint.h>",
        "#include <stddef.h>",
        "#include <string.h>",
        "",
        '#include "GL/gl.h"',
        '#include "mytinygl/mytinygl.h"',
        "",
        "typedef union {",
        "    int64_t i;",
        "    double f;",
        "} play_arg;",
        "",
        f"#define PLAY_FUNCTIONS {len(FUNCTIONS)}",
        "",
        "static const uint8_t k_play_nargs[PLAY_FUNCTIONS] = {",
    ]
    row = [str(len(PROTOS[n])) for n in FUNCTIONS]
    for i in range(0, len(row), 24):
        lines.append("    " + ", ".join(row[i:i + 24]) + ",")
    lines += ["};", "", "static void play_call(uint32_t fid, const play_arg *a)", "{", "    switch (fid) {"]
    for i, n in enumerate(FUNCTIONS):
        args = ", ".join(_arg(k, *p) for k, p in enumerate(PROTOS[n]))
        lines.append(f"    case {i}: (void){n}({args}); break;")
    lines += [
        "    default: break;",
        "    }",
        "}",
        "",
        "int mtgl_play_function_count(void) { return PLAY_FUNCTIONS; }",
        "",
        "int mtgl_play(GLState *ctx, const void *stream, size_t bytes)",
        "{",
        "    const uint8_t *p = (const uint8_t *)stream;",
        "    size_t at = 0;",
        "    if (!ctx || (bytes && !stream)) return MTGL_ERR_INVALID;",
        "    gl_make_current(ctx);",
        "    while (at < bytes) {",
        "        uint32_t hdr[2];",
        "        play_arg a[16];",
        "        if (bytes - at < sizeof(hdr)) return MTGL_ERR_INVALID;",
        "        memcpy(hdr, p + at, sizeof(hdr));",
        "        at += sizeof(hdr);",
        "        if (hdr[0] >= PLAY_FUNCTIONS || hdr[1] != k_play_nargs[hdr[0]] || hdr[1] > 16) return MTGL_ERR_INVALID;",
        "        if (bytes - at < (size_t)hdr[1] * 8u) return MTGL_ERR_INVALID;",
        "        memcpy(a, p + at, (size_t)hdr[1] * 8u);",
        "        at += (size_t)hdr[1] * 8u;",
        "        play_call(hdr[0], a);",
        "    }",
        "    return MTGL_OK;",
        "}",
        "",
    ]
    return "\n".join(lines)


def main():
    with open(OUT, "w") as f:
        f.write(generate())
    print(OUT)


if __name__ == "__main__":
    main()
