"""The debug-bounds build (MTGL_DEBUG_BOUNDS): device index checks that never trap.

The GPU pool offers no memory checker, so the library has a build whose kernels check the
indices of their data-dependent accesses (framebuffer pixels, records taken from tile lists,
tile-list positions, tile ids of sorted pairs, vertex slots) and, when one fails, record the
site in the context's status word (mtgl_stats.debug_status) and skip the access. These tests
render small, awkward cases through that build, tiny framebuffers whose sides are not tile
multiples, triangles across every tile and 8x4 block boundary, clipped ones, points and lines,
in single passes and in batches at every tile size, and require the status word to stay 0 and
every framebuffer to equal the ordinary build's.
"""
import numpy as np
import pytest

import feature_scenes as F
import harness
from mytinygl_gb300 import gl as G
from mytinygl_gb300 import workloads as W
from mytinygl_gb300.scene import Scene, render

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

SIZES = [(1, 1), (3, 5), (8, 4), (9, 17), (16, 16), (17, 15), (31, 33), (40, 7), (65, 33)]


@pytest.fixture(scope="module")
def libs():
    import mytinygl_gb300 as M

    M.build()
    M.build(debug_bounds=True)
    dbg = M.library(debug_bounds=True)
    assert dbg.lib.mtgl_dev_debug_bounds() == 1
    return M.library(), dbg


def edge_scene(w, h, seed):
    """Random triangles with vertices on and around tile (16) and block (8x4) boundaries,
    some far outside the view (clipped), then points and lines, depth and blend on."""
    rng = np.random.default_rng(seed)
    s = Scene(f"edges_{w}x{h}_{seed}", w, h)
    s.glViewport(0, 0, w, h)
    s.glClearColor(0.2, 0.1, 0.0, 1.0)
    s.glClear(G.GL_COLOR_BUFFER_BIT | G.GL_DEPTH_BUFFER_BIT | G.GL_STENCIL_BUFFER_BIT)
    s.glMatrixMode(G.GL_PROJECTION)
    s.glLoadIdentity()
    s.glOrtho(0.0, float(w), float(h), 0.0, -1.0, 1.0)
    s.glMatrixMode(G.GL_MODELVIEW)
    s.glLoadIdentity()
    s.glEnable(G.GL_DEPTH_TEST)
    s.glEnable(G.GL_BLEND)
    s.glBlendFunc(G.GL_SRC_ALPHA, G.GL_ONE_MINUS_SRC_ALPHA)
    marks = sorted({0, 1, 3, 4, 7, 8, 15, 16, 17, 31, 32, 33, w - 1, w, h - 1, h})
    s.glBegin(G.GL_TRIANGLES)
    for _ in range(60):
        for _ in range(3):
            x = float(rng.choice(marks)) + float(rng.choice([0.0, 0.5, -3.0, 2.0 * w]))
            y = float(rng.choice(marks)) + float(rng.choice([0.0, 0.5, -3.0, 2.0 * h]))
            s.glColor4f(*map(float, rng.uniform(0, 1, 4)))
            s.glVertex3f(x, y, float(rng.uniform(-1.5, 1.5)))
    s.glEnd()
    s.glPointSize(3.0)
    s.glBegin(G.GL_POINTS)
    for _ in range(20):
        s.glColor4f(*map(float, rng.uniform(0, 1, 4)))
        s.glVertex3f(float(rng.uniform(-2, w + 2)), float(rng.uniform(-2, h + 2)), 0.0)
    s.glEnd()
    s.glLineWidth(2.0)
    s.glBegin(G.GL_LINES)
    for _ in range(20):
        s.glColor4f(*map(float, rng.uniform(0, 1, 4)))
        s.glVertex3f(float(rng.uniform(-5, w + 5)), float(rng.uniform(-5, h + 5)), 0.0)
    s.glEnd()
    return s


def debug_status(ctx):
    return ctx.stats()["debug_status"]


def test_single_passes_stay_in_bounds(libs):
    plain, dbg = libs
    scenes = [edge_scene(w, h, i) for i, (w, h) in enumerate(SIZES)]
    scenes += [F.SCENES[n][0]() for n in ("clip_big", "prims_tri", "stencil", "texture_wrap_hint", "max_width")]
    scenes.append(W.rop_scene(97, 61, ntri=3000, seed=12))
    for s in scenes:
        want = render(plain, s)
        ctx = dbg.context(s.width, s.height)
        s.play(ctx)
        c, d, st = ctx.read()
        got = (c, d, st, ctx.glGetError())
        assert debug_status(ctx) == 0, s.name
        ctx.destroy()
        harness.assert_parity(harness.compare(want, got), color_tol=0, name=s.name)


@pytest.mark.parametrize("tile", [8, 16, 32])
def test_batches_stay_in_bounds(libs, tile):
    plain, dbg = libs
    scenes = [edge_scene(w, h, 100 + i) for i, (w, h) in enumerate(SIZES)]
    scenes += W.uneven_batch(6, seed=9, min_side=1, max_side=70, min_tri=5, max_tri=800, tex_size=16)
    want = [render(plain, s) for s in scenes]
    ctxs = [dbg.context(s.width, s.height) for s in scenes]
    b = dbg.batch(tile_size=tile)
    dbg.play_many(ctxs, [s.stream() for s in scenes])
    b.render(ctxs)
    b.wait()
    assert b.stats()["debug_status"] == 0
    for s, c, w in zip(scenes, ctxs, want):
        col, dep, st = c.read()
        harness.assert_parity(harness.compare(w, (col, dep, st, c.glGetError())), color_tol=0, name=s.name)
        assert debug_status(c) == 0, s.name
        c.destroy()
    b.destroy()
