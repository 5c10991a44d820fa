"""mtgl_flush_noalloc: rendering a context's queued pass without any device allocation.

The entry point exists for callers that cannot let the renderer allocate while they render
(real-time threads that cannot take cudaMalloc's device-wide synchronisation, processes that
keep device memory under their own budget, hosts whose CUDA allocator belongs to another
runtime). Its scratch is one static 64 MiB device array shared by every call. These tests
call it through the C ABI and compare its frames with the ones the normal path
(glFinish -> per-context scratch from the stream-ordered allocator) renders for the same
calls, with the parity tolerance of the other GPU tests (depth and stencil exact, colour
within 1 LSB). This file is collected last.
"""
import ctypes

import pytest

import harness
from mytinygl_gb300 import gl as G
from mytinygl_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MTGL_ERR_OVERFLOW = 7


@pytest.fixture(scope="module")
def gpu():
    lib = harness.product()
    L = lib.lib
    L.mtgl_flush_noalloc.argtypes = [ctypes.c_void_p]
    L.mtgl_flush_noalloc.restype = ctypes.c_int
    return lib


def passes(ctx):
    """Passes rendered so far. Reading the counters waits for the context, so it also
    renders anything still queued: call it only when nothing should be."""
    s = G.Stats()
    assert ctx.glib.lib.mtgl_get_stats(ctx.handle, ctypes.byref(s)) == 0
    return int(s.passes)


def frame(ctx, scene):
    scene.play(ctx, W.frame_start(scene))


def test_noalloc_flush_matches_default_flush_twice(gpu):
    scenes = [W.sphere_scene(seed=0), W.sphere_scene(seed=1), W.sphere_scene(seed=2)]
    setup = scenes[0]
    fs = W.frame_start(setup)

    ref = gpu.context(setup.width, setup.height)
    setup.play(ref, 0, fs)
    expected = []
    for s in scenes[1:]:
        frame(ref, s)
        ref.glFinish()
        expected.append(ref.read() + (ref.glGetError(),))
    ref.destroy()

    ctx = gpu.context(setup.width, setup.height)
    setup.play(ctx, 0, fs)
    frame(ctx, scenes[0])  # one ordinary frame sizes the context's staging areas
    ctx.glFinish()
    for s, exp in zip(scenes[1:], expected):
        before = passes(ctx)
        frame(ctx, s)
        st = ctx.glib.lib.mtgl_flush_noalloc(ctx.handle)
        assert st == 0, f"mtgl_flush_noalloc failed with status {st}"
        assert passes(ctx) == before + 1, "the queued pass must run inside mtgl_flush_noalloc"
        got = ctx.read() + (ctx.glGetError(),)
        assert passes(ctx) == before + 1, "nothing may be left queued for the read-back"
        harness.assert_parity(harness.compare(exp, got), color_tol=1, name="noalloc")
    ctx.destroy()


def test_noalloc_refuses_a_pass_beyond_its_scratch(gpu):
    """400k triangle records need ~77 MB of scratch: refused before drawing, still queued,
    and the next glFinish renders it on the normal path."""
    big = W.rop_scene(1920, 1080, ntri=400_000, seed=4)
    fs = W.frame_start(big)
    ref = gpu.context(big.width, big.height)
    big.play(ref)
    ref.glFinish()
    expected = ref.read() + (ref.glGetError(),)
    ref.destroy()

    ctx = gpu.context(big.width, big.height)
    big.play(ctx, 0, fs)
    frame(ctx, big)
    ctx.glFinish()  # sizes staging, so the refusal below comes from the scratch limit
    before = passes(ctx)
    frame(ctx, big)
    st = ctx.glib.lib.mtgl_flush_noalloc(ctx.handle)
    assert st == MTGL_ERR_OVERFLOW
    got = ctx.read() + (ctx.glGetError(),)  # the refused pass renders here, on the normal path
    assert passes(ctx) == before + 1
    harness.assert_parity(harness.compare(expected, got), color_tol=1, name="noalloc-overflow")
    ctx.destroy()
