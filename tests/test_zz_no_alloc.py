"""mtgl_flush_noalloc: rendering a context's queued pass without any device allocation.

The entry point exists for callers that cannot let the renderer allocate while they render
(real-time threads that cannot take cudaMalloc's device-wide synchronisation, processes that
keep device memory under their own budget, hosts whose CUDA allocator belongs to another
runtime). Its scratch is one static 64 MiB device array shared by every call. These tests
call it through the C ABI and compare its frames with the ones the normal path
(glFinish -> per-context scratch from the stream-ordered allocator) renders for the same
calls, with the parity tolerance of the other GPU tests (depth and stencil exact, colour
within 1 LSB). They also check that nothing is allocated: the context's own count of scratch
and staging allocations (mtgl_stats.allocations), and the high-water mark of the device's
stream-ordered memory pool, read through the CUDA driver, stay where they were. This file
is collected last.
"""
import ctypes

import pytest

import harness
from mytinygl_gb300 import gl as G
from mytinygl_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MTGL_ERR_OVERFLOW = 7
CU_MEMPOOL_ATTR_USED_MEM_CURRENT = 7
CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8


@pytest.fixture(scope="module")
def gpu():
    lib = harness.product()
    L = lib.lib
    L.mtgl_flush_noalloc.argtypes = [ctypes.c_void_p]
    L.mtgl_flush_noalloc.restype = ctypes.c_int
    return lib


class DevicePool:
    """The current device's default stream-ordered memory pool (the one cudaMallocAsync draws
    from), read through the CUDA driver API."""

    def __init__(self):
        cu = ctypes.CDLL("libcuda.so.1")
        assert cu.cuInit(0) == 0
        dev = ctypes.c_int(0)
        assert cu.cuCtxGetDevice(ctypes.byref(dev)) == 0, "no current CUDA context"
        self.pool = ctypes.c_void_p()
        assert cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0
        self.cu = cu

    def get(self, attr):
        v = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def reset_high(self):
        """Sets the used-memory high-water mark to the memory in use now; returns that."""
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, ctypes.byref(zero)) == 0
        return self.get(CU_MEMPOOL_ATTR_USED_MEM_CURRENT)

    def high(self):
        return self.get(CU_MEMPOOL_ATTR_USED_MEM_HIGH)


def stats(ctx):
    """Counters of ctx. Reading them waits for the context, so it also renders anything still
    queued: call it only when nothing should be."""
    s = G.Stats()
    assert ctx.glib.lib.mtgl_get_stats(ctx.handle, ctypes.byref(s)) == 0
    return {k: int(getattr(s, k)) for k, _ in G.Stats._fields_}


def frame(ctx, scene):
    scene.play(ctx, W.frame_start(scene))


def expected_frames(gpu, setup, scenes):
    """The frames the normal path (glFinish) renders for `scenes`, one after another on one
    context set up by `setup`."""
    ref = gpu.context(setup.width, setup.height)
    setup.play(ref, 0, W.frame_start(setup))
    out = []
    for s in scenes:
        frame(ref, s)
        ref.glFinish()
        out.append(ref.read() + (ref.glGetError(),))
    ref.destroy()
    return out


def sized_context(gpu, setup):
    """A context with the set-up part of `setup` played and one ordinary frame rendered, which
    sizes its staging areas for frames like it."""
    ctx = gpu.context(setup.width, setup.height)
    setup.play(ctx, 0, W.frame_start(setup))
    frame(ctx, setup)
    ctx.glFinish()
    return ctx


def test_noalloc_flush_matches_default_flush_twice(gpu):
    scenes = [W.sphere_scene(seed=0), W.sphere_scene(seed=1), W.sphere_scene(seed=2)]
    setup = scenes[0]
    expected = expected_frames(gpu, setup, scenes[1:])

    ctx = sized_context(gpu, setup)
    pool = DevicePool()
    for s, exp in zip(scenes[1:], expected):
        before = stats(ctx)
        frame(ctx, s)
        used = pool.reset_high()
        st = ctx.glib.lib.mtgl_flush_noalloc(ctx.handle)
        assert st == 0, f"mtgl_flush_noalloc failed with status {st}"
        after = stats(ctx)  # waits for the pass
        assert pool.high() == used, "the stream-ordered pool grew during mtgl_flush_noalloc"
        assert after["allocations"] == before["allocations"], "scratch or staging was allocated"
        assert after["passes"] == before["passes"] + 1, "the queued pass must run inside mtgl_flush_noalloc"
        got = ctx.read() + (ctx.glGetError(),)
        assert stats(ctx)["passes"] == before["passes"] + 1, "nothing may be left queued for the read-back"
        harness.assert_parity(harness.compare(exp, got), color_tol=1, name="noalloc")
    ctx.destroy()


def test_noalloc_two_contexts_in_turn(gpu):
    """Two contexts flushed one right after the other, with no wait between: each renders on
    its own stream, and both passes use the one static array. The second call's GPU work
    must wait for the first's, so both frames come out as the normal path renders them."""
    sa, sb = W.sphere_scene(seed=3), W.rop_scene(320, 240, ntri=20_000, seed=9)
    exp_a = expected_frames(gpu, sa, [W.sphere_scene(seed=4)])[0]
    exp_b = expected_frames(gpu, sb, [sb])[0]
    a, b = sized_context(gpu, sa), sized_context(gpu, sb)
    pool = DevicePool()
    for _ in range(2):
        before = (stats(a)["allocations"], stats(b)["allocations"])
        frame(a, W.sphere_scene(seed=4))
        frame(b, sb)
        used = pool.reset_high()
        assert a.glib.lib.mtgl_flush_noalloc(a.handle) == 0
        assert b.glib.lib.mtgl_flush_noalloc(b.handle) == 0
        got_b = b.read() + (b.glGetError(),)
        got_a = a.read() + (a.glGetError(),)
        assert pool.high() == used, "the stream-ordered pool grew during mtgl_flush_noalloc"
        assert (stats(a)["allocations"], stats(b)["allocations"]) == before
        harness.assert_parity(harness.compare(exp_a, got_a), color_tol=1, name="noalloc-a")
        harness.assert_parity(harness.compare(exp_b, got_b), color_tol=1, name="noalloc-b")
    a.destroy()
    b.destroy()


def test_noalloc_refuses_a_pass_beyond_its_scratch(gpu):
    """400k triangle records need ~77 MB of scratch: refused before drawing, still queued,
    and the next glFinish renders it on the normal path."""
    big = W.rop_scene(1920, 1080, ntri=400_000, seed=4)
    expected = expected_frames(gpu, big, [big])[0]
    ctx = sized_context(gpu, big)  # sizes staging, so the refusal below comes from the scratch limit
    before = stats(ctx)["passes"]
    frame(ctx, big)
    st = ctx.glib.lib.mtgl_flush_noalloc(ctx.handle)
    assert st == MTGL_ERR_OVERFLOW
    got = ctx.read() + (ctx.glGetError(),)  # the refused pass renders here, on the normal path
    assert stats(ctx)["passes"] == before + 1
    harness.assert_parity(harness.compare(expected, got), color_tol=1, name="noalloc-overflow")
    ctx.destroy()
