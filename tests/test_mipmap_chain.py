"""MTGL_OPT_MIPMAP_CHAIN: the opt-in full mipmap chain, an extension of this library.

MyTinyGL's glTexImage2D accepts level 0 only and its sampler knows level 0 plus one derived
level (gl_api.c:803-806, textures.c:311-354, 457-557); that stays the default and is what the
parity tests compare. With the option on, a texture image also gets every further level (each
the 2x2 box filter of the one before), levels above 0 can be replaced through glTexImage2D,
and the mipmap filters use the whole chain. The CPU oracle implements the same extension, so
the GPU is checked against it with the usual tolerance; the oracle itself is checked here on
the CPU: the level rules, and a far-minified triangle that must show the chain's last level,
computed independently below.
"""
import ctypes

import numpy as np
import pytest

import feature_scenes as F
import harness
from mytinygl_gb300 import gl as G
from mytinygl_gb300.scene import Scene

MTGL_OPT_MIPMAP_CHAIN = 2


def bind(lib):
    lib.lib.mtgl_set_option.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.lib.mtgl_set_option.restype = ctypes.c_int
    return lib


def render_chain(lib, scene, on=True):
    """The scene on a fresh context with the extension switched on (or left off) first."""
    ctx = lib.context(scene.width, scene.height)
    try:
        if on:
            assert lib.lib.mtgl_set_option(ctx.handle, MTGL_OPT_MIPMAP_CHAIN, 1) == 0
        scene.play(ctx)
        c, d, s = ctx.read()
        return c, d, s, ctx.glGetError()
    finally:
        ctx.destroy()


def box_chain(tex):
    """The chain of an RGBA8 texture [h, w, 4] as the box filter builds it: channels as
    byte / 255 in float32, the four texels summed in order, times 0.25, clamped, * 255 and
    truncated (textures.c:311-354 for level 1, the same rule for every further level)."""
    f = np.float32
    levels = [tex]
    cur = tex
    while cur.shape[0] >= 2 and cur.shape[1] >= 2:
        h, w = cur.shape[0] // 2, cur.shape[1] // 2
        c = cur[:2 * h, :2 * w].astype(np.float32) / f(255.0)
        s = ((c[0::2, 0::2] + c[0::2, 1::2]) + c[1::2, 0::2]) + c[1::2, 1::2]
        s = np.clip(s * f(0.25), f(0), f(1))
        cur = (s * f(255.0)).astype(np.int32).astype(np.uint8)
        levels.append(cur)
    return levels


def far_triangle_scene(tex, min_filter):
    """One small triangle over a huge texture-coordinate range (LOD far above the top level)."""
    h, w = tex.shape[:2]
    s = Scene("chain_far", 48, 40)
    s.glViewport(0, 0, 48, 40)
    s.glClearColor(0.0, 0.0, 0.0, 1.0)
    s.glClear(G.GL_COLOR_BUFFER_BIT | G.GL_DEPTH_BUFFER_BIT)
    s.glGenTextures(1, np.zeros(1, np.uint32))
    s.glBindTexture(G.GL_TEXTURE_2D, 1)
    s.glTexImage2D(G.GL_TEXTURE_2D, 0, G.GL_RGBA, w, h, 0, G.GL_RGBA, G.GL_UNSIGNED_BYTE, np.ascontiguousarray(tex))
    s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MIN_FILTER, min_filter)
    s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MAG_FILTER, G.GL_LINEAR)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glBegin(G.GL_TRIANGLES)
    for (x, y, u, v) in ((-0.8, -0.8, 0.0, 0.0), (0.8, -0.8, 600.0, 0.0), (-0.8, 0.8, 0.0, 600.0)):
        s.glTexCoord2f(u, v)
        s.glVertex3f(x, y, 0.0)
    s.glEnd()
    return s


@pytest.fixture(scope="module")
def oracle():
    return bind(harness.oracle())


def test_level_rules(oracle):
    rng = np.random.default_rng(3)
    tex = rng.integers(0, 256, (16, 16, 4), dtype=np.uint8)
    lvl2 = np.ascontiguousarray(rng.integers(0, 256, (4, 4, 4), dtype=np.uint8))

    def errors(on, calls):
        ctx = oracle.context(8, 8)
        if on:
            assert oracle.lib.mtgl_set_option(ctx.handle, MTGL_OPT_MIPMAP_CHAIN, 1) == 0
        ctx.glGenTextures(1, np.zeros(1, np.uint32))
        ctx.glBindTexture(G.GL_TEXTURE_2D, 1)
        out = []
        for level, w, h, data in calls:
            ctx.glTexImage2D(G.GL_TEXTURE_2D, level, G.GL_RGBA, w, h, 0, G.GL_RGBA, G.GL_UNSIGNED_BYTE, data)
            out.append(ctx.glGetError())
        ctx.destroy()
        return out

    base = (0, 16, 16, np.ascontiguousarray(tex))
    # without the option: level 0 only, as the reference (gl_api.c:803-806)
    assert errors(False, [base, (2, 4, 4, lvl2)]) == [G.GL_NO_ERROR, G.GL_INVALID_VALUE]
    # with it: a level of the right size, a wrong size, a level beyond the chain, no base yet
    assert errors(True, [base, (2, 4, 4, lvl2), (2, 8, 8, np.zeros((8, 8, 4), np.uint8)),
                         (9, 1, 1, np.zeros((1, 1, 4), np.uint8)), (-1, 4, 4, lvl2)]) == \
        [G.GL_NO_ERROR, G.GL_NO_ERROR, G.GL_INVALID_VALUE, G.GL_INVALID_VALUE, G.GL_INVALID_VALUE]
    assert errors(True, [(1, 8, 8, np.zeros((8, 8, 4), np.uint8))]) == [G.GL_INVALID_OPERATION]


@pytest.mark.parametrize("min_filter", [G.GL_NEAREST_MIPMAP_NEAREST, G.GL_LINEAR_MIPMAP_LINEAR])
def test_far_triangle_shows_the_last_level(oracle, min_filter):
    """Far beyond the top level every covered pixel is the chain's 1x1 level (the texture's
    box-filtered mean; bilinear filtering of that one texel may move a channel by 1 in the
    repacking); without the option the reference's level 1 shows instead."""
    rng = np.random.default_rng(4)
    tex = rng.integers(0, 256, (32, 32, 4), dtype=np.uint8)
    top = box_chain(tex)[-1]
    assert top.shape[:2] == (1, 1)
    c, _, _, err = render_chain(oracle, far_triangle_scene(tex, min_filter))
    assert err == 0
    covered = c != 0xFF000000
    assert covered.sum() > 200
    got = c[covered].view(np.uint8).reshape(-1, 4).astype(int)
    tol = 0 if min_filter == G.GL_NEAREST_MIPMAP_NEAREST else 1
    assert np.abs(got - top[0, 0].astype(int)).max() <= tol
    c_off, _, _, _ = render_chain(oracle, far_triangle_scene(tex, min_filter), on=False)
    off = c_off[covered].view(np.uint8).reshape(-1, 4).astype(int)
    assert np.abs(off - top[0, 0].astype(int)).max() > 8


def test_explicit_level_replaces_the_built_one(oracle):
    """A level given through glTexImage2D replaces the built one: a uniform colour given as
    the last level shows on the far triangle."""
    rng = np.random.default_rng(5)
    tex = rng.integers(0, 256, (8, 8, 4), dtype=np.uint8)
    s = far_triangle_scene(tex, G.GL_NEAREST_MIPMAP_NEAREST)
    i = next(k for k, (n, _) in enumerate(s.cmds) if n == "glTexParameteri")
    s.cmds.insert(i, ("glTexImage2D", (G.GL_TEXTURE_2D, 3, G.GL_RGBA, 1, 1, 0, G.GL_RGBA, G.GL_UNSIGNED_BYTE,
                                       np.array([[[10, 200, 30, 255]]], np.uint8))))
    c, _, _, err = render_chain(oracle, s)
    assert err == 0
    covered = c != 0xFF000000
    assert covered.sum() > 200 and (c[covered] == np.array([10, 200, 30, 255], np.uint8).view(np.uint32)[0]).all()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mipmap_floor", "texture_modes", "texture_wrap_hint", "phong_textured_fog"])
def test_gpu_matches_oracle_with_the_chain(oracle, name):
    gpu = bind(harness.product())
    scene = F.SCENES[name][0]()
    stats = harness.compare(render_chain(oracle, scene), render_chain(gpu, scene))
    harness.assert_parity(stats, color_tol=1, name=f"{name} (mipmap chain)")


@pytest.mark.gpu
@pytest.mark.parametrize("min_filter", [G.GL_NEAREST_MIPMAP_NEAREST, G.GL_LINEAR_MIPMAP_NEAREST,
                                        G.GL_NEAREST_MIPMAP_LINEAR, G.GL_LINEAR_MIPMAP_LINEAR])
def test_gpu_far_and_explicit_levels(oracle, min_filter):
    gpu = bind(harness.product())
    rng = np.random.default_rng(6)
    tex = rng.integers(0, 256, (64, 32, 4), dtype=np.uint8)
    s = far_triangle_scene(tex, min_filter)
    stats = harness.compare(render_chain(oracle, s), render_chain(gpu, s))
    harness.assert_parity(stats, color_tol=1, name="far triangle (mipmap chain)")
    # the same with levels 1 and 4 given explicitly
    i = next(k for k, (n, _) in enumerate(s.cmds) if n == "glTexParameteri")
    s.cmds.insert(i, ("glTexImage2D", (G.GL_TEXTURE_2D, 4, G.GL_RGBA, 2, 4, 0, G.GL_RGBA, G.GL_UNSIGNED_BYTE,
                                       np.ascontiguousarray(rng.integers(0, 256, (4, 2, 4), dtype=np.uint8)))))
    s.cmds.insert(i, ("glTexImage2D", (G.GL_TEXTURE_2D, 1, G.GL_RGBA, 16, 32, 0, G.GL_RGBA, G.GL_UNSIGNED_BYTE,
                                       np.ascontiguousarray(rng.integers(0, 256, (32, 16, 4), dtype=np.uint8)))))
    a, b = render_chain(oracle, s), render_chain(gpu, s)
    assert a[3] == 0
    harness.assert_parity(harness.compare(a, b), color_tol=1, name="explicit levels (mipmap chain)")
