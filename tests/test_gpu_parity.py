"""GPU parity: libmytinygl_gb300.so against the CPU oracle and the golden fixtures.

Tolerance (BASELINE the benchmark spec): depth and stencil bit-exact (NaN payloads aside), RGBA8
colour within 1 LSB per channel, identical glGetError. The colour slack covers CUDA's
expf/log2f/powf against glibc's in fog factors, texture LOD and specular terms.
"""
import numpy as np
import pytest

import feature_scenes as F
import harness
from mytinygl_gb300 import gl as G
from mytinygl_gb300 import workloads as W
from mytinygl_gb300.scene import Scene, render

pytestmark = pytest.mark.gpu

ALL_SCENES = sorted(F.SCENES)


@pytest.fixture(scope="module")
def gpu():
    return harness.product()


@pytest.fixture(scope="module")
def oracle():
    return harness.oracle()


def check(gpu, oracle, scene, tol=1):
    a = render(oracle, scene)
    b = render(gpu, scene)
    stats = harness.compare(a, b)
    harness.assert_parity(stats, color_tol=tol, name=scene.name)
    return stats


@pytest.mark.parametrize("name", ALL_SCENES)
def test_feature_scene(gpu, oracle, name):
    check(gpu, oracle, F.SCENES[name][0]())


@pytest.mark.parametrize("path", harness.golden_files(), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_golden(gpu, path):
    scene, expected, buffers = harness.load_golden(path)
    stats = harness.compare(expected, render(gpu, scene), buffers)
    harness.assert_parity(stats, color_tol=1, name=scene.name)


def test_sphere_full_size(gpu, oracle):
    check(gpu, oracle, W.sphere_scene())
    check(gpu, oracle, W.sphere_scene(use_vbo=False, seed=7))


def test_textured_reduced(gpu, oracle):
    check(gpu, oracle, W.textured_scene(480, 270, ntri=6000))


def test_rop_reduced(gpu, oracle):
    check(gpu, oracle, W.rop_scene(480, 270, ntri=60000))


@pytest.mark.slow
def test_textured_full_size(gpu, oracle):
    """The benchmark's textured frame at its real size: 1920x1080, 100k clip-straddling
    triangles, 512^2 trilinear texture, 8 point lights, EXP fog (seed 1)."""
    check(gpu, oracle, W.textured_scene())


@pytest.mark.slow
def test_rop_full_size(gpu, oracle):
    """The benchmark's ROP frame at its real size: 1920x1080, 1M small triangles blended in
    submission order, alpha test, stencil INCR, depth LEQUAL without writes (seed 2)."""
    check(gpu, oracle, W.rop_scene())


def test_immediate_equals_arrays(gpu):
    """The same triangles through glBegin/glEnd and through glDrawArrays give the same image."""
    rng = np.random.default_rng(9)
    pos = rng.uniform(-1.2, 1.2, (300, 3)).astype(np.float32)
    col = rng.uniform(0, 1, (300, 4)).astype(np.float32)
    a = F.base("imm", 128, 96, persp=False)
    a.glEnable(G.GL_DEPTH_TEST)
    a.glBegin(G.GL_TRIANGLES)
    for p, c in zip(pos, col):
        a.glColor4f(*map(float, c))
        a.glVertex3f(*map(float, p))
    a.glEnd()
    b = F.base("arr", 128, 96, persp=False)
    b.glEnable(G.GL_DEPTH_TEST)
    b.glEnableClientState(G.GL_VERTEX_ARRAY)
    b.glEnableClientState(G.GL_COLOR_ARRAY)
    b.glVertexPointer(3, G.GL_FLOAT, 0, pos)
    b.glColorPointer(4, G.GL_FLOAT, 0, col)
    b.glDrawArrays(G.GL_TRIANGLES, 0, 300)
    ra, rb = render(gpu, a), render(gpu, b)
    harness.assert_parity(harness.compare(ra, rb), color_tol=0, name="immediate-vs-arrays")


def test_many_draws_and_passes(gpu, oracle):
    """Hundreds of small draws, interleaved clears (new passes) and buffer updates between draws."""
    rng = np.random.default_rng(10)
    s = F.base("many", 96, 64)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glEnable(G.GL_BLEND)
    s.glBlendFunc(G.GL_SRC_ALPHA, G.GL_ONE_MINUS_SRC_ALPHA)
    vb = rng.uniform(-2, 2, (30, 3)).astype(np.float32)
    vb[:, 2] = rng.uniform(-6, -2, 30)
    s.glGenBuffers(1, np.zeros(1, np.uint32))
    s.glBindBuffer(G.GL_ARRAY_BUFFER, 1)
    s.glBufferData(G.GL_ARRAY_BUFFER, vb.nbytes, vb, G.GL_DYNAMIC_DRAW)
    s.glEnableClientState(G.GL_VERTEX_ARRAY)
    s.glVertexPointer(3, G.GL_FLOAT, 0, 0)
    for i in range(120):
        s.glColor4f(*map(float, rng.uniform(0, 1, 4)))
        s.glDrawArrays(G.GL_TRIANGLES, 3 * (i % 10), 3)
        if i % 17 == 5:
            upd = np.ascontiguousarray(rng.uniform(-2, 2, 3).astype(np.float32))
            s.glBufferSubData(G.GL_ARRAY_BUFFER, 12 * int(rng.integers(0, 30)), 12, upd)
        if i % 40 == 39:
            s.glEnable(G.GL_SCISSOR_TEST)
            s.glScissor(int(rng.integers(0, 40)), int(rng.integers(0, 30)), 40, 30)
            s.glClear(G.GL_DEPTH_BUFFER_BIT | G.GL_COLOR_BUFFER_BIT)
            s.glDisable(G.GL_SCISSOR_TEST)
    check(gpu, oracle, s)


def test_readpixels(gpu, oracle):
    scene = F.SCENES["blend"][0]()
    outs = []
    for lib in (oracle, gpu):
        ctx = lib.context(scene.width, scene.height)
        scene.play(ctx)
        buf = np.zeros((50, 70, 4), np.uint8)
        ctx.glReadPixels(-5, 30, 70, 50, G.GL_RGBA, G.GL_UNSIGNED_BYTE, buf)
        outs.append(buf.copy())
        ctx.destroy()
    d = np.abs(outs[0].astype(int) - outs[1].astype(int))
    assert d.max() <= 1


def test_random_points_and_lines(gpu, oracle):
    """Seeded mixes of points and lines of every mode and width with triangles, through
    random depth, blend, fog, texture and scissor states."""
    for seed in range(6):
        rng = np.random.default_rng(500 + seed)
        s = Scene(f"points_lines_{seed}", 80, 60)
        s.glViewport(0, 0, 80, 60)
        s.glClearColor(0.1, 0.1, 0.1, 1.0)
        s.glClear(G.GL_COLOR_BUFFER_BIT | G.GL_DEPTH_BUFFER_BIT | G.GL_STENCIL_BUFFER_BIT)
        s.glMatrixMode(G.GL_PROJECTION)
        s.glFrustum(*W.frustum_params(60.0, 80 / 60, 0.5, 20.0))
        s.glMatrixMode(G.GL_MODELVIEW)
        s.glTranslatef(0.0, 0.0, -4.0)
        F.checker_texture(s, 8)
        for _ in range(8):
            s.glDepthFunc([G.GL_LESS, G.GL_LEQUAL, G.GL_GREATER, G.GL_ALWAYS][int(rng.integers(0, 4))])
            for cap in (G.GL_DEPTH_TEST, G.GL_BLEND, G.GL_FOG, G.GL_TEXTURE_2D, G.GL_SCISSOR_TEST):
                (s.glEnable if rng.uniform() < 0.5 else s.glDisable)(cap)
            s.glBlendFunc(G.GL_SRC_ALPHA, G.GL_ONE_MINUS_SRC_ALPHA)
            s.glScissor(int(rng.integers(0, 30)), int(rng.integers(0, 20)), 50, 40)
            s.glLineWidth(float(rng.uniform(0.5, 5.0)))
            s.glPointSize(float(rng.uniform(0.5, 5.0)))
            mode = [G.GL_POINTS, G.GL_LINES, G.GL_LINE_STRIP, G.GL_LINE_LOOP, G.GL_TRIANGLES][int(rng.integers(0, 5))]
            F._line_batch(s, rng, mode, 12, spread=3.0, z=(-5.0, 3.0), uv=True)
        check(gpu, oracle, s)


@pytest.mark.parametrize("which", ["textured", "zbuffer", "depth_range", "clip_big", "stencil", "mipmap_floor",
                                   "depth_mix"])
def test_depth_rejection_changes_nothing(gpu, which):
    """Hierarchical-z rejection in the tile kernel only skips fragments that cannot pass the
    depth test and have no other effect: images are identical with it on and off, and with
    it off every covered fragment is counted."""
    import ctypes

    scene = W.textured_scene(480, 270, ntri=6000) if which == "textured" else F.SCENES[which][0]()
    gpu.lib.mtgl_set_option.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    gpu.lib.mtgl_set_option.restype = ctypes.c_int
    outs = []
    for enabled in (1, 0):
        ctx = gpu.context(scene.width, scene.height)
        assert gpu.lib.mtgl_set_option(ctx.handle, 1, enabled) == 0
        scene.play(ctx)
        outs.append(ctx.read() + (ctx.glGetError(),))
        ctx.destroy()
    harness.assert_parity(harness.compare(outs[0], outs[1]), color_tol=0, name=f"{which} rejection on/off")


def _list_calls(ctx, rng_seed=5, late=False):
    """A list of one 3,000-triangle block (colour and normal per vertex), called three times
    under different modelviews and lighting."""
    rng = np.random.default_rng(rng_seed)
    n = 9000
    pos = rng.uniform(-2.5, 2.5, (n, 3)).astype(np.float32)
    pos[:, 2] = rng.uniform(-7.0, -2.0, n)
    col = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    nrm = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    ctx.glViewport(0, 0, 160, 120)
    ctx.glMatrixMode(G.GL_PROJECTION)
    ctx.glLoadIdentity()
    ctx.glFrustum(-0.4, 0.4, -0.3, 0.3, 0.5, 20.0)
    ctx.glMatrixMode(G.GL_MODELVIEW)
    ctx.glLoadIdentity()
    ctx.glEnable(G.GL_DEPTH_TEST)
    ctx.glClear(G.GL_COLOR_BUFFER_BIT | G.GL_DEPTH_BUFFER_BIT | G.GL_STENCIL_BUFFER_BIT)
    ctx.glGenLists(1)
    ctx.glNewList(1, G.GL_COMPILE)
    ctx.glBegin(G.GL_TRIANGLES)
    for i in range(n):
        if not late or i > 0:
            ctx.glColor4f(*map(float, col[i]))
        ctx.glNormal3f(*map(float, nrm[i]))
        ctx.glVertex3f(*map(float, pos[i]))
    ctx.glEnd()
    ctx.glEndList()
    yield
    ctx.glCallList(1)
    ctx.glRotatef(25.0, 0.2, 0.3, 1.0)
    ctx.glEnable(G.GL_LIGHTING)
    ctx.glEnable(G.GL_LIGHT0)
    ctx.glEnable(G.GL_COLOR_MATERIAL)
    ctx.glCallList(1)
    ctx.glTranslatef(0.5, -0.3, -1.0)
    ctx.glDisable(G.GL_COLOR_MATERIAL)
    ctx.glCallList(1)


@pytest.mark.parametrize("late", [False, True], ids=["resident", "replayed"])
def test_list_block_device_resident(gpu, oracle, late):
    """glCallList draws a qualifying block from the list's device buffer: no client bytes
    are staged for it, and the frame matches the oracle. A block that sets its colour after
    a vertex has taken the caller's replays through immediate mode and stages its vertices."""
    out = []
    for lib in (oracle, gpu):
        ctx = lib.context(160, 120)
        ctx.make_current()
        steps = _list_calls(ctx, late=late)
        next(steps)
        ctx.finish()
        if lib is gpu:
            ctx.reset_stats()
        for _ in steps:
            pass
        out.append(ctx.read())
        if lib is gpu:
            st = ctx.stats()
            if late:
                assert st["staged_bytes"] >= 3 * 9000 * 48
            else:
                assert st["staged_bytes"] == 0
            assert st["input_triangles"] == 3 * 3000
        ctx.destroy()
    stats = harness.compare(out[0] + (0,), out[1] + (0,))
    harness.assert_parity(stats, color_tol=1, name="list_block")


def test_context_size_limits(gpu):
    """The same framebuffer size limits as the reference (framebuffer.h:30-35)."""
    import test_oracle

    for (w, h), ok in test_oracle.SIZE_CASES:
        assert test_oracle.context_created(gpu, w, h) == ok, (w, h)
