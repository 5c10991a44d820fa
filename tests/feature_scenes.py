"""Feature scenes: small seeded GL call scripts covering the fixed-function path.

They restate the recipes of MyTinyGL's interactive testbed headlessly (clipping 1.0-3,
primitives 1.0-4/1.0-8, culling 1.0-5, z-buffer 1.0-6, textured cube 1.0-7, fog 1.0-9,
lighting 1.0-10, blend 1.0-11, filters 1.0-12, display lists 1.0-13, mipmaps 1.0-14, texenv
1.0-15, extreme inputs 1.0-16, stencil 1.0-17, VBOs 1.5-0) as scripts with fixed inputs, plus
quirk cases of the reference (alpha test only on textured fragments, stencil zpass before
the alpha test, flat shading from the clipped fan's last vertex, ...).

Every scene clears every buffer it is compared on. `SCENES` maps a name to
(builder, flags); flags: "lines" marks scenes that draw points or lines, "slow" marks
scenes too large for the golden set.
"""
from __future__ import annotations

import math

import numpy as np

from mytinygl_gb300 import gl as G
from mytinygl_gb300.scene import Scene
from mytinygl_gb300.workloads import euler_matrix, frustum_params

W, H = 96, 72
ALL = G.GL_COLOR_BUFFER_BIT | G.GL_DEPTH_BUFFER_BIT | G.GL_STENCIL_BUFFER_BIT


def f32(*v):
    return np.array(v, np.float32)


def base(name, w=W, h=H, persp=True, clear=(0.05, 0.05, 0.1, 1.0)):
    s = Scene(name, w, h)
    s.glViewport(0, 0, w, h)
    s.glClearColor(*clear)
    s.glClearDepth(1.0)
    s.glClearStencil(0)
    s.glMatrixMode(G.GL_PROJECTION)
    s.glLoadIdentity()
    if persp:
        s.glFrustum(*frustum_params(60.0, w / h, 0.5, 20.0))
    s.glMatrixMode(G.GL_MODELVIEW)
    s.glLoadIdentity()
    s.glClear(ALL)
    return s


def rand_tris(s, rng, n, spread=2.0, z=(-6.0, -2.0), color=True, uv=False, normal=False, alpha=(1.0, 1.0), mode=G.GL_TRIANGLES):
    s.glBegin(mode)
    for _ in range(n * 3):
        if color:
            c = rng.uniform(0, 1, 4)
            c[3] = rng.uniform(*alpha)
            s.glColor4f(*map(float, c))
        if uv:
            s.glTexCoord2f(*map(float, rng.uniform(-1.0, 2.0, 2)))
        if normal:
            n3 = rng.uniform(-1, 1, 3)
            s.glNormal3f(*map(float, n3))
        p = rng.uniform(-spread, spread, 3)
        p[2] = rng.uniform(*z)
        s.glVertex3f(*map(float, p))
    s.glEnd()


def checker_texture(s, size=8, seed=5, fmt=G.GL_RGBA, alpha_ramp=False, tex_id=1):
    rng = np.random.default_rng(seed)
    comps = {G.GL_RGBA: 4, G.GL_RGB: 3, G.GL_LUMINANCE: 1, G.GL_LUMINANCE_ALPHA: 2}[fmt]
    w = size[0] if isinstance(size, tuple) else size
    h = size[1] if isinstance(size, tuple) else size
    data = rng.integers(0, 256, (h, w, comps), dtype=np.uint8)
    if alpha_ramp and comps in (2, 4):
        data[..., -1] = np.linspace(0, 255, w * h).astype(np.uint8).reshape(h, w)
    s.glGenTextures(1, np.zeros(1, np.uint32))
    s.glBindTexture(G.GL_TEXTURE_2D, tex_id)
    s.glTexImage2D(G.GL_TEXTURE_2D, 0, fmt, w, h, 0, fmt, G.GL_UNSIGNED_BYTE, np.ascontiguousarray(data))


# ----------------------------------------------------------------------------- scenes

def sc_clip_big():
    s = base("clip_big")
    rng = np.random.default_rng(11)
    s.glTranslatef(0.0, 0.0, -3.0)
    s.glMultMatrixf(euler_matrix(0.3, 0.7, 0.2))
    rand_tris(s, rng, 24, spread=6.0, z=(-8.0, 6.0))
    return s


def sc_clip_near_far():
    s = base("clip_near_far")
    rng = np.random.default_rng(12)
    rand_tris(s, rng, 30, spread=3.0, z=(-25.0, 1.0))
    return s


def sc_primitives_tri():
    s = base("prims_tri")
    rng = np.random.default_rng(13)
    s.glTranslatef(0.0, 0.0, -4.0)
    for mode in (G.GL_TRIANGLES, G.GL_TRIANGLE_STRIP, G.GL_TRIANGLE_FAN, G.GL_QUADS, G.GL_QUAD_STRIP, G.GL_POLYGON):
        s.glBegin(mode)
        for _ in range(int(rng.integers(5, 13))):
            s.glColor3f(*map(float, rng.uniform(0, 1, 3)))
            s.glVertex2f(*map(float, rng.uniform(-2, 2, 2)))
        s.glEnd()
    return s


def sc_primitives_lines():
    s = base("prims_lines")
    rng = np.random.default_rng(14)
    s.glTranslatef(0.0, 0.0, -4.0)
    s.glEnable(G.GL_DEPTH_TEST)
    for mode in (G.GL_POINTS, G.GL_LINES, G.GL_LINE_STRIP, G.GL_LINE_LOOP):
        for width in (1.0, 3.0):
            s.glPointSize(width + 1.0)
            s.glLineWidth(width)
            s.glBegin(mode)
            for _ in range(int(rng.integers(4, 9))):
                s.glColor3f(*map(float, rng.uniform(0, 1, 3)))
                s.glVertex3f(*map(float, rng.uniform(-3, 3, 3)))
            s.glEnd()
    return s


def sc_polygon_modes():
    s = base("polygon_modes")
    rng = np.random.default_rng(15)
    s.glTranslatef(0.0, 0.0, -4.0)
    s.glPolygonMode(G.GL_FRONT, G.GL_LINE)
    s.glPolygonMode(G.GL_BACK, G.GL_POINT)
    s.glPointSize(2.0)
    rand_tris(s, rng, 10, spread=2.0, z=(-2.0, 1.0))
    s.glPolygonMode(G.GL_FRONT_AND_BACK, G.GL_FILL)
    rand_tris(s, rng, 4, spread=2.0, z=(-2.0, 1.0))
    return s


def sc_culling():
    s = base("culling")
    rng = np.random.default_rng(16)
    s.glTranslatef(0.0, 0.0, -4.0)
    s.glEnable(G.GL_CULL_FACE)
    for ff, cm in ((G.GL_CCW, G.GL_BACK), (G.GL_CW, G.GL_BACK), (G.GL_CCW, G.GL_FRONT), (G.GL_CW, G.GL_FRONT_AND_BACK)):
        s.glFrontFace(ff)
        s.glCullFace(cm)
        rand_tris(s, rng, 8, spread=2.5, z=(-2.0, 1.0))
    return s


def sc_zbuffer():
    s = base("zbuffer")
    rng = np.random.default_rng(17)
    s.glEnable(G.GL_DEPTH_TEST)
    for func in (G.GL_LESS, G.GL_LEQUAL, G.GL_GREATER, G.GL_GEQUAL, G.GL_EQUAL, G.GL_NOTEQUAL, G.GL_ALWAYS, G.GL_NEVER):
        s.glDepthFunc(func)
        rand_tris(s, rng, 6, spread=2.5, z=(-6.0, -1.0))
    s.glDepthMask(0)
    s.glDepthFunc(G.GL_LESS)
    rand_tris(s, rng, 6, spread=2.5, z=(-6.0, -1.0))
    return s


def sc_depth_range():
    s = base("depth_range")
    rng = np.random.default_rng(18)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glDepthRange(0.2, 0.7)
    rand_tris(s, rng, 12, spread=2.5, z=(-6.0, -1.0))
    s.glDepthRange(0.9, 0.1)
    rand_tris(s, rng, 12, spread=2.5, z=(-6.0, -1.0))
    return s


def sc_texture_modes():
    s = base("texture_modes")
    rng = np.random.default_rng(19)
    checker_texture(s, 16, alpha_ramp=True)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glTexEnvfv(G.GL_TEXTURE_ENV, G.GL_TEXTURE_ENV_COLOR, f32(0.2, 0.7, 0.4, 0.5))
    s.glTranslatef(0.0, 0.0, -3.0)
    for env in (G.GL_MODULATE, G.GL_DECAL, G.GL_REPLACE, G.GL_BLEND, G.GL_ADD):
        for filt in (G.GL_NEAREST, G.GL_LINEAR):
            s.glTexEnvi(G.GL_TEXTURE_ENV, G.GL_TEXTURE_ENV_MODE, env)
            s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MAG_FILTER, filt)
            s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MIN_FILTER, filt)
            rand_tris(s, rng, 2, spread=2.0, z=(-2.0, 1.0), uv=True)
    return s


def sc_texture_wrap_hint():
    s = base("texture_wrap_hint")
    rng = np.random.default_rng(20)
    checker_texture(s, (8, 4))
    s.glEnable(G.GL_TEXTURE_2D)
    s.glTranslatef(0.0, 0.0, -3.0)
    for ws, wt in ((G.GL_REPEAT, G.GL_CLAMP), (G.GL_CLAMP_TO_EDGE, G.GL_REPEAT)):
        for hint in (G.GL_FASTEST, G.GL_NICEST):
            s.glHint(G.GL_PERSPECTIVE_CORRECTION_HINT, hint)
            s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_WRAP_S, ws)
            s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_WRAP_T, wt)
            s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MAG_FILTER, G.GL_LINEAR)
            rand_tris(s, rng, 3, spread=2.0, z=(-3.0, 1.0), uv=True)
    return s


def sc_texture_formats():
    s = base("texture_formats")
    rng = np.random.default_rng(21)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glTranslatef(0.0, 0.0, -3.0)
    for i, (fmt, size) in enumerate(((G.GL_RGB, 8), (G.GL_LUMINANCE, (4, 16)), (G.GL_LUMINANCE_ALPHA, 8), (G.GL_RGBA, (1, 8)))):
        checker_texture(s, size, seed=30 + i, fmt=fmt, tex_id=i + 1)
        s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MIN_FILTER, G.GL_LINEAR_MIPMAP_LINEAR)
        s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MAG_FILTER, G.GL_LINEAR)
        rand_tris(s, rng, 3, spread=2.0, z=(-3.0, 1.0), uv=True)
    return s


def sc_mipmap_floor():
    s = base("mipmap_floor", 128, 96)
    checker_texture(s, 32, seed=7)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MAG_FILTER, G.GL_LINEAR)
    filters = (G.GL_NEAREST, G.GL_LINEAR, G.GL_NEAREST_MIPMAP_NEAREST, G.GL_LINEAR_MIPMAP_NEAREST,
               G.GL_NEAREST_MIPMAP_LINEAR, G.GL_LINEAR_MIPMAP_LINEAR)
    for i, f in enumerate(filters):
        s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MIN_FILTER, f)
        x0 = -3.0 + i * 1.0
        s.glBegin(G.GL_QUADS)
        for (x, z, u, v) in ((x0, -1.0, 0.0, 0.0), (x0 + 1.0, -1.0, 4.0, 0.0), (x0 + 1.0, -15.0, 4.0, 30.0), (x0, -15.0, 0.0, 30.0)):
            s.glTexCoord2f(u, v)
            s.glVertex3f(x, -1.0, z)
        s.glEnd()
    return s


def sc_fog():
    s = base("fog")
    rng = np.random.default_rng(22)
    s.glEnable(G.GL_FOG)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glFogfv(G.GL_FOG_COLOR, f32(0.6, 0.6, 0.7, 1.0))
    for mode, dens, start, end in ((G.GL_LINEAR, 1.0, 1.0, 8.0), (G.GL_EXP, 0.3, 0.0, 1.0), (G.GL_EXP2, 0.2, 0.0, 1.0),
                                   (G.GL_LINEAR, 1.0, 3.0, 3.0)):
        s.glFogi(G.GL_FOG_MODE, mode)
        s.glFogf(G.GL_FOG_DENSITY, dens)
        s.glFogf(G.GL_FOG_START, start)
        s.glFogf(G.GL_FOG_END, end)
        rand_tris(s, rng, 6, spread=3.0, z=(-10.0, -1.0))
    return s


def _sphere_immediate(s, stacks=8, slices=12, r=1.0):
    for i in range(stacks):
        t0, t1 = math.pi * i / stacks, math.pi * (i + 1) / stacks
        s.glBegin(G.GL_QUAD_STRIP)
        for j in range(slices + 1):
            p = 2 * math.pi * j / slices
            for t in (t0, t1):
                n = (math.sin(t) * math.cos(p), math.cos(t), math.sin(t) * math.sin(p))
                s.glNormal3f(*n)
                s.glVertex3f(*(r * c for c in n))
        s.glEnd()


def sc_lighting(shade):
    def build():
        s = base(f"lighting_{shade}", 112, 84)
        s.glEnable(G.GL_DEPTH_TEST)
        s.glEnable(G.GL_LIGHTING)
        s.glShadeModel(shade)
        s.glLightModelfv(G.GL_LIGHT_MODEL_AMBIENT, f32(0.1, 0.1, 0.15, 1.0))
        s.glLightfv(G.GL_LIGHT0, G.GL_POSITION, f32(2.0, 2.0, 1.0, 1.0))
        s.glLightf(G.GL_LIGHT0, G.GL_LINEAR_ATTENUATION, 0.2)
        s.glEnable(G.GL_LIGHT0)
        s.glLightfv(G.GL_LIGHT1, G.GL_POSITION, f32(-1.0, 0.5, 2.0, 0.0))
        s.glLightfv(G.GL_LIGHT1, G.GL_DIFFUSE, f32(0.3, 0.4, 0.9, 1.0))
        s.glLightfv(G.GL_LIGHT1, G.GL_SPECULAR, f32(1.0, 1.0, 1.0, 1.0))
        s.glEnable(G.GL_LIGHT1)
        s.glLightfv(G.GL_LIGHT2, G.GL_POSITION, f32(0.0, 3.0, -2.0, 1.0))
        s.glLightfv(G.GL_LIGHT2, G.GL_SPOT_DIRECTION, f32(0.0, -1.0, -1.0))
        s.glLightf(G.GL_LIGHT2, G.GL_SPOT_CUTOFF, 40.0)
        s.glLightf(G.GL_LIGHT2, G.GL_SPOT_EXPONENT, 4.0)
        s.glLightfv(G.GL_LIGHT2, G.GL_DIFFUSE, f32(0.9, 0.7, 0.2, 1.0))
        s.glEnable(G.GL_LIGHT2)
        s.glMaterialfv(G.GL_FRONT, G.GL_SPECULAR, f32(0.8, 0.8, 0.8, 1.0))
        s.glMaterialf(G.GL_FRONT, G.GL_SHININESS, 24.0)
        s.glMaterialfv(G.GL_BACK, G.GL_DIFFUSE, f32(0.9, 0.2, 0.2, 1.0))
        s.glTranslatef(-1.2, 0.0, -4.0)
        _sphere_immediate(s)
        s.glLightModeli(G.GL_LIGHT_MODEL_LOCAL_VIEWER, 1)
        s.glLightModeli(G.GL_LIGHT_MODEL_TWO_SIDE, 1)
        s.glEnable(G.GL_NORMALIZE)
        s.glTranslatef(2.4, 0.0, 0.0)
        s.glScalef(1.0, 0.7, 1.3)
        _sphere_immediate(s)
        return s
    return build


def sc_color_material():
    s = base("color_material")
    rng = np.random.default_rng(23)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glEnable(G.GL_LIGHTING)
    s.glEnable(G.GL_LIGHT0)
    s.glEnable(G.GL_COLOR_MATERIAL)
    for face, mode in ((G.GL_FRONT_AND_BACK, G.GL_AMBIENT_AND_DIFFUSE), (G.GL_FRONT, G.GL_DIFFUSE),
                       (G.GL_BACK, G.GL_AMBIENT), (G.GL_FRONT, G.GL_EMISSION), (G.GL_FRONT, G.GL_SPECULAR)):
        s.glColorMaterial(face, mode)
        rand_tris(s, rng, 4, spread=2.5, z=(-6.0, -2.0), normal=True)
    s.glDisable(G.GL_COLOR_MATERIAL)
    rand_tris(s, rng, 4, spread=2.5, z=(-6.0, -2.0), normal=True)
    return s


def sc_blend():
    s = base("blend")
    rng = np.random.default_rng(24)
    s.glEnable(G.GL_BLEND)
    factors = (G.GL_ZERO, G.GL_ONE, G.GL_SRC_COLOR, G.GL_ONE_MINUS_SRC_COLOR, G.GL_DST_COLOR, G.GL_ONE_MINUS_DST_COLOR,
               G.GL_SRC_ALPHA, G.GL_ONE_MINUS_SRC_ALPHA, G.GL_DST_ALPHA, G.GL_ONE_MINUS_DST_ALPHA,
               G.GL_CONSTANT_COLOR)
    for i, sf in enumerate(factors + (G.GL_SRC_ALPHA_SATURATE,)):
        df = factors[(i * 5 + 3) % len(factors)]
        s.glBlendFunc(sf, df)
        rand_tris(s, rng, 2, spread=2.5, z=(-6.0, -2.0), alpha=(0.0, 1.0))
    return s


def sc_stencil():
    s = base("stencil")
    rng = np.random.default_rng(25)
    s.glEnable(G.GL_STENCIL_TEST)
    s.glEnable(G.GL_DEPTH_TEST)
    ops = (G.GL_KEEP, G.GL_ZERO, G.GL_REPLACE, G.GL_INCR, G.GL_INCR_WRAP, G.GL_DECR, G.GL_DECR_WRAP, G.GL_INVERT)
    funcs = (G.GL_ALWAYS, G.GL_LESS, G.GL_EQUAL, G.GL_LEQUAL, G.GL_GREATER, G.GL_NOTEQUAL, G.GL_GEQUAL, G.GL_NEVER)
    for i in range(16):
        s.glStencilFunc(funcs[i % 8], int(rng.integers(0, 4)), 0xFF if i % 3 else 0x0F)
        s.glStencilOp(ops[i % 8], ops[(i + 3) % 8], ops[(i + 5) % 8])
        s.glStencilMask(0xFF if i % 4 else 0xF3)
        rand_tris(s, rng, 3, spread=2.5, z=(-6.0, -2.0))
    return s


def sc_alpha_test():
    s = base("alpha_test")
    rng = np.random.default_rng(26)
    checker_texture(s, 8, alpha_ramp=True)
    s.glEnable(G.GL_ALPHA_TEST)
    s.glEnable(G.GL_STENCIL_TEST)
    s.glStencilOp(G.GL_KEEP, G.GL_KEEP, G.GL_INCR)
    s.glEnable(G.GL_DEPTH_TEST)
    for i, func in enumerate((G.GL_GREATER, G.GL_LESS, G.GL_EQUAL, G.GL_NOTEQUAL, G.GL_GEQUAL, G.GL_LEQUAL)):
        s.glAlphaFunc(func, 0.4)
        if i % 2:
            s.glEnable(G.GL_TEXTURE_2D)
        else:
            s.glDisable(G.GL_TEXTURE_2D)
        rand_tris(s, rng, 3, spread=2.5, z=(-6.0, -2.0), uv=True, alpha=(0.0, 1.0))
    return s


def sc_scissor_mask():
    s = base("scissor_mask")
    rng = np.random.default_rng(27)
    s.glEnable(G.GL_SCISSOR_TEST)
    s.glScissor(10, 5, 50, 40)
    s.glClearColor(0.9, 0.2, 0.2, 1.0)
    s.glClear(G.GL_COLOR_BUFFER_BIT)
    s.glScissor(-5, 20, 60, 200)
    s.glColorMask(1, 0, 1, 1)
    rand_tris(s, rng, 6, spread=2.5, z=(-6.0, -2.0))
    s.glColorMask(0, 1, 0, 0)
    s.glDisable(G.GL_SCISSOR_TEST)
    rand_tris(s, rng, 6, spread=2.5, z=(-6.0, -2.0))
    s.glColorMask(0, 0, 0, 0)
    rand_tris(s, rng, 3, spread=2.5, z=(-6.0, -2.0))
    return s


def sc_viewport():
    s = base("viewport")
    rng = np.random.default_rng(28)
    s.glViewport(20, 10, 200, 40)
    rand_tris(s, rng, 8, spread=2.5, z=(-6.0, -2.0))
    s.glViewport(-30, -15, 80, 60)
    rand_tris(s, rng, 8, spread=2.5, z=(-6.0, -2.0))
    return s


def sc_display_lists():
    s = base("display_lists")
    rng = np.random.default_rng(29)
    s.glGenLists(3)
    s.glNewList(1, G.GL_COMPILE)
    s.glPushMatrix()
    s.glRotatef(30.0, 0.0, 0.0, 1.0)
    s.glTranslatef(0.5, 0.0, 0.0)
    rand_tris(s, rng, 4, spread=1.5, z=(-6.0, -3.0))
    s.glPopMatrix()
    s.glEndList()
    s.glNewList(2, G.GL_COMPILE_AND_EXECUTE)
    s.glCallList(1)
    s.glTranslatef(-0.7, 0.3, 0.0)
    s.glCallList(1)
    s.glEndList()
    s.glListBase(1)
    s.glCallLists(2, G.GL_UNSIGNED_BYTE, np.array([0, 1], np.uint8))
    return s


def _block(s, rng, mode, n, color="each", uv=False, normal="each", z=(-6.0, -3.0), spread=1.6, two_d=False):
    """One glBegin/glEnd block. color / normal: "each" (set before every vertex), "once"
    (set before the first vertex only), "late" (set after the first vertex: the block takes
    the caller's value first, so it must replay), None (never set: the caller's value)."""
    s.glBegin(mode)
    for k in range(n):
        if color == "each" or (color == "once" and k == 0) or (color == "late" and k == 1):
            s.glColor4f(*map(float, rng.uniform(0, 1, 4)))
        if uv:
            s.glTexCoord2f(*map(float, rng.uniform(-0.5, 1.5, 2)))
        if normal == "each" or (normal == "once" and k == 0) or (normal == "late" and k == 1):
            s.glNormal3f(*map(float, rng.uniform(-1, 1, 3)))
        p = rng.uniform(-spread, spread, 3)
        if two_d:
            s.glVertex2f(float(p[0]), float(p[1]))
        else:
            s.glVertex3f(float(p[0]), float(p[1]), float(rng.uniform(*z)))
    if color == "once" and n > 2:
        s.glColor3f(0.2, 0.9, 0.4)  # after the last vertex: current afterwards, drawn by no vertex
    s.glEnd()


def sc_list_blocks():
    """Display lists whose begin/end blocks are drawn from device-resident vertices, called
    under changing matrices, current attributes and lighting; immediate draws after each call
    take the current colour / texcoord / normal and the colour-material writes the calls left."""
    s = base("list_blocks")
    rng = np.random.default_rng(41)
    checker_texture(s, size=8, seed=12)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glGenLists(4)
    s.glNewList(1, G.GL_COMPILE)
    _block(s, rng, G.GL_TRIANGLES, 18, uv=True)
    _block(s, rng, G.GL_TRIANGLE_FAN, 7, color=None, normal=None)
    s.glPushMatrix()
    s.glTranslatef(0.3, -0.2, -4.5)
    _block(s, rng, G.GL_TRIANGLE_STRIP, 9, color="once", normal=None, two_d=True)
    s.glPopMatrix()
    _block(s, rng, G.GL_QUADS, 8, color="late")
    _block(s, rng, G.GL_TRIANGLES, 0)
    s.glEndList()
    s.glNewList(2, G.GL_COMPILE)
    _block(s, rng, G.GL_TRIANGLES, 15, color="once", normal="each")
    _block(s, rng, G.GL_POLYGON, 6, color=None, normal="once")
    _block(s, rng, G.GL_TRIANGLE_STRIP, 8, color="each", normal="late")
    s.glEndList()
    s.glNewList(3, G.GL_COMPILE)
    s.glRotatef(20.0, 0.0, 0.0, 1.0)
    s.glCallList(1)
    _block(s, rng, G.GL_TRIANGLES, 9, color="each", uv=True, normal=None)
    s.glEndList()

    def immediate(n=3):
        _block(s, rng, G.GL_TRIANGLES, n, color=None, normal=None, spread=2.0, z=(-7.0, -2.5))

    s.glColor4f(0.9, 0.3, 0.2, 1.0)
    s.glCallList(1)
    immediate()
    s.glTranslatef(0.4, 0.3, 0.0)
    s.glColor4f(0.1, 0.5, 0.9, 0.5)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glCallList(1)
    immediate()
    s.glDisable(G.GL_TEXTURE_2D)
    s.glEnable(G.GL_LIGHTING)
    s.glEnable(G.GL_LIGHT0)
    s.glEnable(G.GL_COLOR_MATERIAL)
    s.glNormal3f(0.0, 0.0, 1.0)
    s.glCallList(2)
    immediate()
    s.glColorMaterial(G.GL_FRONT, G.GL_DIFFUSE)
    s.glColor4f(0.8, 0.8, 0.1, 1.0)
    s.glNormal3f(0.3, -0.5, 0.8)
    s.glCallList(2)
    s.glDisable(G.GL_COLOR_MATERIAL)
    immediate()
    s.glDisable(G.GL_LIGHTING)
    # executed while another list is compiled: every block replays and is recorded
    s.glNewList(4, G.GL_COMPILE_AND_EXECUTE)
    s.glCallList(3)
    s.glEndList()
    s.glScalef(0.7, 0.7, 1.0)
    s.glCallList(4)
    immediate()
    # a vertex emitted outside glBegin/glEnd is pending: the next block replays and takes it
    s.glVertex3f(0.1, 0.2, -3.0)
    s.glCallList(1)
    immediate()
    s.glDeleteLists(1, 1)
    s.glCallList(3)
    s.glNewList(2, G.GL_COMPILE)
    _block(s, rng, G.GL_TRIANGLES, 6, color="each", normal=None)
    s.glEndList()
    s.glCallList(2)
    immediate()
    return s


def _limit_frame(name, w, h, tex_w, tex_h):
    """A framebuffer at the reference's largest side (16384, framebuffer.h:30) with a texture
    at its largest side (2048, textures.h:17): long thin triangles, lines and points across
    the whole frame, flat and textured, depth tested."""
    s = base(name, w, h, persp=False)
    rng = np.random.default_rng(w * 7 + h)
    checker_texture(s, size=(tex_w, tex_h), seed=13)
    s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MIN_FILTER, G.GL_LINEAR_MIPMAP_LINEAR)
    s.glEnable(G.GL_DEPTH_TEST)
    for textured in (False, True):
        (s.glEnable if textured else s.glDisable)(G.GL_TEXTURE_2D)
        s.glBegin(G.GL_TRIANGLES)
        for _ in range(12):
            c = rng.uniform(0, 1, 4)
            s.glColor4f(*map(float, c))
            s.glTexCoord2f(*map(float, rng.uniform(-0.5, 1.5, 2)))
            s.glVertex3f(*map(float, rng.uniform(-1.1, 1.1, 3)))
        s.glEnd()
    s.glDisable(G.GL_TEXTURE_2D)
    s.glLineWidth(2.0)
    _block(s, rng, G.GL_LINE_STRIP, 6, normal=None, spread=1.0, z=(-0.9, 0.9))
    s.glPointSize(3.0)
    _block(s, rng, G.GL_POINTS, 10, normal=None, spread=1.0, z=(-0.9, 0.9))
    return s


def sc_max_width():
    return _limit_frame("max_width", 16384, 8, 2048, 4)


def sc_max_height():
    return _limit_frame("max_height", 8, 16384, 4, 2048)


def sc_ragged():
    """Empty and ragged inputs: every mode with 0-5 vertices (incomplete primitives dropped),
    empty glBegin/glEnd, zero-count and negative-first array draws, a zero-size viewport,
    degenerate triangles, and a texture one texel over the size limit (refused)."""
    s = base("ragged")
    rng = np.random.default_rng(47)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glTranslatef(0.0, 0.0, -4.0)
    for mode in (G.GL_POINTS, G.GL_LINES, G.GL_LINE_LOOP, G.GL_LINE_STRIP, G.GL_TRIANGLES, G.GL_TRIANGLE_STRIP,
                 G.GL_TRIANGLE_FAN, G.GL_QUADS, G.GL_QUAD_STRIP, G.GL_POLYGON):
        for n in range(6):
            _block(s, rng, mode, n, normal=None, spread=2.0, z=(-1.0, 1.0))
    s.glBegin(G.GL_TRIANGLES)  # degenerate: a repeated vertex, then three collinear ones
    for p in ((0.1, 0.1, 0.0), (0.1, 0.1, 0.0), (0.9, 0.5, 0.0), (-1.0, -1.0, 0.0), (0.0, 0.0, 0.0),
              (1.0, 1.0, 0.0)):
        s.glVertex3f(*p)
    s.glEnd()
    pos = rng.uniform(-2, 2, (12, 3)).astype(np.float32)
    s.glEnableClientState(G.GL_VERTEX_ARRAY)
    s.glVertexPointer(3, G.GL_FLOAT, 0, pos)
    s.glDrawArrays(G.GL_TRIANGLES, 0, 0)
    s.glDrawArrays(G.GL_TRIANGLES, -2, 8)  # elements before the array read the defaults
    s.glDrawElements(G.GL_TRIANGLES, 0, G.GL_UNSIGNED_SHORT, np.zeros(3, np.uint16))
    s.glDisableClientState(G.GL_VERTEX_ARRAY)
    s.glViewport(10, 10, 0, 0)
    _block(s, rng, G.GL_TRIANGLES, 6, normal=None, spread=2.0, z=(-1.0, 1.0))
    s.glViewport(0, 0, W, H)
    big = np.zeros((2, 2049, 4), np.uint8)
    s.glGenTextures(1, np.zeros(1, np.uint32))
    s.glBindTexture(G.GL_TEXTURE_2D, 1)
    s.glTexImage2D(G.GL_TEXTURE_2D, 0, G.GL_RGBA, 2049, 2, 0, G.GL_RGBA, G.GL_UNSIGNED_BYTE, big)
    s.glEnable(G.GL_TEXTURE_2D)
    _block(s, rng, G.GL_TRIANGLES, 6, uv=True, normal=None, spread=2.0, z=(-1.0, 1.0))
    return s


def sc_deferred_colour():
    """One pass of opaque triangles whose colour the tile kernel defers to the tile's end:
    heavy overdraw under every depth function, a colour-masked depth pre-pass, depth writes
    off, stencil updates, and raster states that change between draws (flat / smooth,
    texture on / off with every env mode and filter, fog, perspective hint)."""
    s = base("deferred_colour")
    rng = np.random.default_rng(53)
    checker_texture(s, 16, seed=21)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glEnable(G.GL_STENCIL_TEST)
    s.glStencilFunc(G.GL_ALWAYS, 3, 0xFF)
    s.glStencilOp(G.GL_KEEP, G.GL_INCR, G.GL_REPLACE)
    s.glColorMask(0, 0, 0, 0)  # depth pre-pass: no colour written
    rand_tris(s, rng, 6, spread=2.0, z=(-5.0, -3.0))
    s.glColorMask(1, 1, 1, 1)
    s.glDepthFunc(G.GL_LEQUAL)
    for k, env in enumerate((G.GL_MODULATE, G.GL_DECAL, G.GL_REPLACE, G.GL_BLEND, G.GL_ADD)):
        (s.glEnable if k % 2 == 0 else s.glDisable)(G.GL_TEXTURE_2D)
        s.glTexEnvi(G.GL_TEXTURE_ENV, G.GL_TEXTURE_ENV_MODE, env)
        s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MIN_FILTER,
                          (G.GL_LINEAR_MIPMAP_LINEAR, G.GL_NEAREST, G.GL_LINEAR_MIPMAP_NEAREST)[k % 3])
        s.glShadeModel(G.GL_FLAT if k % 3 == 1 else G.GL_SMOOTH)
        s.glHint(G.GL_PERSPECTIVE_CORRECTION_HINT, G.GL_FASTEST if k == 3 else G.GL_NICEST)
        (s.glEnable if k >= 2 else s.glDisable)(G.GL_FOG)
        rand_tris(s, rng, 8, spread=2.2, z=(-6.0, -2.0), uv=True)
    for func in (G.GL_GREATER, G.GL_ALWAYS, G.GL_NEVER, G.GL_NOTEQUAL, G.GL_LESS):
        s.glDepthFunc(func)
        rand_tris(s, rng, 4, spread=2.2, z=(-6.0, -2.0), uv=True)
    s.glDepthMask(0)
    rand_tris(s, rng, 4, spread=2.2, z=(-6.0, -2.0), uv=True)
    return s


def sc_vertex_arrays():
    s = base("vertex_arrays")
    rng = np.random.default_rng(30)
    n = 18
    pos = rng.uniform(-2, 2, (n, 3)).astype(np.float32)
    pos[:, 2] = rng.uniform(-6, -2, n)
    col_ub = rng.integers(0, 256, (n, 4), dtype=np.uint8)
    col_f = rng.uniform(-0.5, 1.5, (n, 3)).astype(np.float32)
    idx16 = rng.integers(0, n, 24).astype(np.uint16)
    s.glEnableClientState(G.GL_VERTEX_ARRAY)
    s.glEnableClientState(G.GL_COLOR_ARRAY)
    s.glVertexPointer(3, G.GL_FLOAT, 0, pos)
    s.glColorPointer(4, G.GL_UNSIGNED_BYTE, 0, col_ub)
    s.glDrawArrays(G.GL_TRIANGLES, 0, n)
    s.glColorPointer(3, G.GL_FLOAT, 0, col_f)
    s.glDrawElements(G.GL_TRIANGLE_STRIP, 12, G.GL_UNSIGNED_SHORT, idx16)
    pos2 = np.ascontiguousarray(pos[:, :2] * 0.5)
    s.glVertexPointer(2, G.GL_FLOAT, 0, pos2)
    s.glDisableClientState(G.GL_COLOR_ARRAY)
    s.glDrawArrays(G.GL_TRIANGLE_FAN, 2, 7)
    # after the draws the current colour is the last element's: this triangle shows it
    s.glBegin(G.GL_TRIANGLES)
    s.glVertex3f(-1.0, -1.0, -3.0)
    s.glVertex3f(1.0, -1.0, -3.0)
    s.glVertex3f(0.0, 1.0, -3.0)
    s.glEnd()
    s.glDisableClientState(G.GL_VERTEX_ARRAY)
    return s


def sc_vbo():
    s = base("vbo")
    rng = np.random.default_rng(31)
    n = 30
    rec = np.zeros(n, dtype=[("p", "<f4", 3), ("c", "<f4", 4), ("t", "<f4", 2), ("n", "<f4", 3)])
    rec["p"] = rng.uniform(-2, 2, (n, 3))
    rec["p"][:, 2] = rng.uniform(-6, -2, n)
    rec["c"] = rng.uniform(0, 1, (n, 4))
    rec["t"] = rng.uniform(0, 2, (n, 2))
    rec["n"] = rng.uniform(-1, 1, (n, 3))
    raw = np.frombuffer(rec.tobytes(), np.uint8)
    idx8 = rng.integers(0, n, 21).astype(np.uint8)
    idx32 = rng.integers(0, n, 24).astype(np.uint32)
    checker_texture(s, 8)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glEnable(G.GL_LIGHTING)
    s.glEnable(G.GL_LIGHT0)
    s.glEnable(G.GL_COLOR_MATERIAL)
    s.glGenBuffers(3, np.zeros(3, np.uint32))
    s.glBindBuffer(G.GL_ARRAY_BUFFER, 1)
    s.glBufferData(G.GL_ARRAY_BUFFER, raw.nbytes, raw, G.GL_STATIC_DRAW)
    s.glBindBuffer(G.GL_ELEMENT_ARRAY_BUFFER, 2)
    s.glBufferData(G.GL_ELEMENT_ARRAY_BUFFER, idx8.nbytes, idx8, G.GL_STATIC_DRAW)
    for a in (G.GL_VERTEX_ARRAY, G.GL_COLOR_ARRAY, G.GL_TEXTURE_COORD_ARRAY, G.GL_NORMAL_ARRAY):
        s.glEnableClientState(a)
    s.glVertexPointer(3, G.GL_FLOAT, 48, 0)
    s.glColorPointer(4, G.GL_FLOAT, 48, 12)
    s.glTexCoordPointer(2, G.GL_FLOAT, 48, 28)
    s.glNormalPointer(G.GL_FLOAT, 48, 36)
    s.glDrawElements(G.GL_TRIANGLES, 21, G.GL_UNSIGNED_BYTE, 0)
    s.glBindBuffer(G.GL_ELEMENT_ARRAY_BUFFER, 3)
    s.glBufferData(G.GL_ELEMENT_ARRAY_BUFFER, idx32.nbytes, idx32, G.GL_STATIC_DRAW)
    s.glDrawElements(G.GL_QUADS, 20, G.GL_UNSIGNED_INT, 16)
    s.glBindBuffer(G.GL_ARRAY_BUFFER, 1)
    upd = np.ascontiguousarray(rng.uniform(-2, 2, 3).astype(np.float32))
    s.glBufferSubData(G.GL_ARRAY_BUFFER, 48 * 3, upd.nbytes, upd)
    s.glTexCoordPointer(1, G.GL_FLOAT, 48, 28)
    s.glDrawArrays(G.GL_TRIANGLES, 0, 27)
    return s


def sc_state_in_begin_end():
    s = base("state_in_begin_end")
    rng = np.random.default_rng(32)
    s.glEnable(G.GL_LIGHTING)
    s.glEnable(G.GL_LIGHT0)
    s.glEnable(G.GL_COLOR_MATERIAL)
    s.glTranslatef(0.0, 0.0, -4.0)
    s.glBegin(G.GL_TRIANGLES)
    for i in range(12):
        if i % 4 == 0:
            s.glRotatef(25.0, 0.0, 0.0, 1.0)
        if i == 7:
            s.glMaterialfv(G.GL_FRONT, G.GL_AMBIENT, f32(0.9, 0.1, 0.1, 1.0))
            s.glColorMaterial(G.GL_FRONT, G.GL_DIFFUSE)
        s.glColor3f(*map(float, rng.uniform(0, 1, 3)))
        s.glNormal3f(*map(float, rng.uniform(-1, 1, 3)))
        s.glVertex2f(*map(float, rng.uniform(-2, 2, 2)))
    s.glEnd()
    # vertices emitted outside glBegin/glEnd stay queued for the next glEnd (gl_api.c:664-686)
    s.glColor3f(0.2, 0.9, 0.3)
    s.glVertex2f(-1.5, -1.5)
    s.glBegin(G.GL_TRIANGLES)
    s.glVertex2f(1.5, -1.5)
    s.glVertex2f(0.0, 1.5)
    s.glEnd()
    return s


def sc_flat_clip():
    s = base("flat_clip")
    rng = np.random.default_rng(33)
    s.glShadeModel(G.GL_FLAT)
    rand_tris(s, rng, 16, spread=5.0, z=(-10.0, 2.0))
    return s


def sc_extreme_values():
    s = base("extreme_values")
    s.glEnable(G.GL_DEPTH_TEST)
    s.glTranslatef(0.0, 0.0, -3.0)
    vals = [(1e10, 0.0, 0.0), (-1e10, 1e10, -5.0), (0.0, 0.0, 1e10), (float("inf"), 0.0, 0.0), (float("nan"), 1.0, 0.0),
            (0.5, 0.5, -1.0), (-0.5, 0.5, -1.0), (0.0, -0.5, float("-inf")), (1e-30, 1e-30, 1e-30)]
    s.glBegin(G.GL_TRIANGLES)
    for i in range(len(vals) * 2):
        a = vals[i % len(vals)]
        s.glColor4f(float("nan") if i == 3 else 0.5, 2.0, -1.0, float("inf") if i == 5 else 0.8)
        s.glVertex3f(*a)
    s.glEnd()
    s.glBegin(G.GL_TRIANGLES)
    s.glColor3f(0.8, 0.3, 0.1)
    s.glVertex3f(-1.0, -1.0, 0.0)
    s.glVertex3f(1e10, -1.0, 0.0)
    s.glVertex3f(0.0, 1e10, 0.0)
    s.glEnd()
    return s


def sc_draw_pixels():
    s = base("draw_pixels", persp=False)
    rng = np.random.default_rng(34)
    s.glMatrixMode(G.GL_PROJECTION)
    s.glLoadIdentity()
    s.glOrtho(0.0, float(W), 0.0, float(H), -1.0, 1.0)
    s.glMatrixMode(G.GL_MODELVIEW)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glBegin(G.GL_TRIANGLES)
    s.glColor3f(0.2, 0.3, 0.9)
    s.glVertex3f(5.0, 5.0, 0.5)
    s.glVertex3f(80.0, 10.0, 0.5)
    s.glVertex3f(30.0, 60.0, 0.5)
    s.glEnd()
    for i, (fmt, comps) in enumerate(((G.GL_RGBA, 4), (G.GL_RGB, 3), (G.GL_LUMINANCE, 1), (G.GL_LUMINANCE_ALPHA, 2))):
        img = rng.integers(0, 256, (12, 20, comps), dtype=np.uint8)
        s.glRasterPos2i(5 + 20 * i, 8 + 12 * i)
        if i == 2:
            s.glEnable(G.GL_BLEND)
            s.glBlendFunc(G.GL_SRC_ALPHA, G.GL_ONE_MINUS_SRC_ALPHA)
        if i == 3:
            s.glEnable(G.GL_ALPHA_TEST)
            s.glAlphaFunc(G.GL_GREATER, 0.5)
        s.glDrawPixels(20, 12, fmt, G.GL_UNSIGNED_BYTE, np.ascontiguousarray(img))
    s.glRasterPos2f(90.0, 70.0)
    s.glDrawPixels(20, 12, G.GL_RGB, G.GL_UNSIGNED_BYTE, np.ascontiguousarray(rng.integers(0, 256, (12, 20, 3), dtype=np.uint8)))
    return s


def sc_phong_textured_fog():
    s = base("phong_textured_fog", 112, 84)
    checker_texture(s, 16)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MIN_FILTER, G.GL_LINEAR_MIPMAP_NEAREST)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glEnable(G.GL_LIGHTING)
    s.glEnable(G.GL_LIGHT0)
    s.glLightfv(G.GL_LIGHT0, G.GL_POSITION, f32(1.0, 1.0, 1.0, 0.0))
    s.glShadeModel(G.GL_PHONG)
    s.glEnable(G.GL_FOG)
    s.glFogi(G.GL_FOG_MODE, G.GL_EXP2)
    s.glFogf(G.GL_FOG_DENSITY, 0.15)
    s.glTranslatef(0.0, 0.0, -4.0)
    s.glBegin(G.GL_QUADS)
    for (x, y, u, v) in ((-2, -2, 0, 0), (2, -2, 3, 0), (2, 2, 3, 3), (-2, 2, 0, 3)):
        s.glNormal3f(x * 0.3, y * 0.3, 1.0)
        s.glTexCoord2f(float(u), float(v))
        s.glVertex3f(float(x), float(y), -1.0 - 0.5 * x)
    s.glEnd()
    return s


def sc_texture_matrix():
    s = base("texture_matrix")
    rng = np.random.default_rng(35)
    checker_texture(s, 8)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glMatrixMode(G.GL_TEXTURE)
    s.glLoadIdentity()
    m = np.eye(4, dtype=np.float32)
    m[3, 0] = 0.3  # projective texture: w depends on s
    m[0, 1] = 0.5
    s.glMultMatrixf(np.ascontiguousarray(m.reshape(16)))
    s.glMatrixMode(G.GL_MODELVIEW)
    rand_tris(s, rng, 6, spread=2.5, z=(-6.0, -2.0), uv=True)
    return s


def sc_depth_mix():
    """Depth writes that raise stored depth (GL_ALWAYS, GL_GREATER, GL_NOTEQUAL) interleaved,
    triangle by triangle, with GL_LESS / GL_LEQUAL draws over the same pixels."""
    s = base("depth_mix", 64, 48)
    rng = np.random.default_rng(36)
    s.glEnable(G.GL_DEPTH_TEST)
    funcs = (G.GL_LESS, G.GL_LEQUAL, G.GL_ALWAYS, G.GL_GREATER, G.GL_LESS, G.GL_NOTEQUAL, G.GL_GEQUAL)
    for i in range(160):
        s.glDepthFunc(funcs[int(rng.integers(0, len(funcs)))])
        rand_tris(s, rng, 1, spread=1.5, z=(-8.0, -1.5))
    return s


def _line_batch(s, rng, mode, n, spread=3.0, z=(-6.0, 0.5), uv=False):
    s.glBegin(mode)
    for _ in range(n):
        c = rng.uniform(0, 1, 4)
        c[3] = rng.uniform(0.3, 1.0)
        s.glColor4f(*map(float, c))
        if uv:
            s.glTexCoord2f(*map(float, rng.uniform(-1.0, 2.0, 2)))
        p = rng.uniform(-spread, spread, 3)
        p[2] = rng.uniform(*z)
        s.glVertex3f(*map(float, p))
    s.glEnd()


def sc_lines_states():
    """Lines of widths 1-6 in all three line modes through depth test and writes, blending,
    linear fog and a scissor box; endpoints beyond every clip plane (near included), so
    clip_line cuts most segments."""
    s = base("lines_states", 96, 72)
    rng = np.random.default_rng(37)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glEnable(G.GL_FOG)
    s.glFogi(G.GL_FOG_MODE, G.GL_LINEAR)
    s.glFogf(G.GL_FOG_START, 1.0)
    s.glFogf(G.GL_FOG_END, 9.0)
    s.glFogfv(G.GL_FOG_COLOR, f32(0.6, 0.2, 0.1, 1.0))
    rand_tris(s, rng, 6, spread=2.0, z=(-5.0, -2.0))
    for i, (mode, width) in enumerate(((G.GL_LINES, 1.0), (G.GL_LINE_STRIP, 2.0), (G.GL_LINE_LOOP, 3.0),
                                       (G.GL_LINES, 6.0), (G.GL_LINE_STRIP, 1.4), (G.GL_LINE_LOOP, 4.6))):
        s.glLineWidth(width)
        if i == 3:
            s.glEnable(G.GL_BLEND)
            s.glBlendFunc(G.GL_SRC_ALPHA, G.GL_ONE_MINUS_SRC_ALPHA)
        if i == 4:
            s.glEnable(G.GL_SCISSOR_TEST)
            s.glScissor(10, 8, 60, 40)
            s.glDepthFunc(G.GL_LEQUAL)
            s.glDepthMask(0)
        _line_batch(s, rng, mode, 10, spread=4.0, z=(-9.0, 1.0))
    return s


def sc_points_states():
    """Points of sizes 1-6 (odd and even squares) through a texture sampled at lod 0 with
    the alpha test on its alpha, EXP fog, blending and the depth test, near every edge."""
    s = base("points_states", 96, 72)
    rng = np.random.default_rng(38)
    checker_texture(s, 8, alpha_ramp=True)
    s.glTexEnvi(G.GL_TEXTURE_ENV, G.GL_TEXTURE_ENV_MODE, G.GL_MODULATE)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glEnable(G.GL_FOG)
    s.glFogi(G.GL_FOG_MODE, G.GL_EXP)
    s.glFogf(G.GL_FOG_DENSITY, 0.2)
    rand_tris(s, rng, 4, spread=2.0, z=(-5.0, -2.0))
    for i, size in enumerate((1.0, 2.0, 3.0, 4.4, 6.0)):
        s.glPointSize(size)
        if i == 1:
            s.glEnable(G.GL_TEXTURE_2D)
            s.glEnable(G.GL_ALPHA_TEST)
            s.glAlphaFunc(G.GL_GREATER, 0.3)
        if i == 3:
            s.glEnable(G.GL_BLEND)
            s.glBlendFunc(G.GL_ONE, G.GL_ONE)
        _line_batch(s, rng, G.GL_POINTS, 40, spread=3.2, z=(-8.0, 0.5), uv=True)
    s.glDisable(G.GL_TEXTURE_2D)
    s.glPointSize(2.0)
    _line_batch(s, rng, G.GL_POINTS, 30, spread=3.2, z=(-8.0, 0.5))  # alpha test on the colour
    return s


def sc_polygon_modes_lit():
    """glPolygonMode LINE on front faces and POINT on back faces under GL_PHONG lighting
    (vertex colours lit per vertex), a bound texture (lines sample it, points do not), fog and
    wide lines, on triangles that the near and side planes clip."""
    s = base("polygon_modes_lit", 96, 72)
    rng = np.random.default_rng(39)
    checker_texture(s, 8)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glEnable(G.GL_LIGHTING)
    s.glEnable(G.GL_LIGHT0)
    s.glLightfv(G.GL_LIGHT0, G.GL_POSITION, f32(1.0, 2.0, 2.0, 0.0))
    s.glShadeModel(G.GL_PHONG)
    s.glEnable(G.GL_FOG)
    s.glFogi(G.GL_FOG_MODE, G.GL_EXP2)
    s.glFogf(G.GL_FOG_DENSITY, 0.12)
    s.glPolygonMode(G.GL_FRONT, G.GL_LINE)
    s.glPolygonMode(G.GL_BACK, G.GL_POINT)
    s.glLineWidth(2.0)
    s.glTranslatef(0.0, 0.0, -3.0)
    rand_tris(s, rng, 12, spread=2.5, z=(-3.0, 3.5), uv=True, normal=True)
    s.glShadeModel(G.GL_SMOOTH)
    s.glPolygonMode(G.GL_FRONT_AND_BACK, G.GL_LINE)
    s.glLineWidth(1.0)
    rand_tris(s, rng, 8, spread=2.5, z=(-3.0, 3.5), uv=True, normal=True)
    return s


SCENES = {
    "clip_big": (sc_clip_big, ()),
    "clip_near_far": (sc_clip_near_far, ()),
    "prims_tri": (sc_primitives_tri, ()),
    "prims_lines": (sc_primitives_lines, ("lines",)),
    "polygon_modes": (sc_polygon_modes, ("lines",)),
    "culling": (sc_culling, ()),
    "zbuffer": (sc_zbuffer, ()),
    "depth_range": (sc_depth_range, ()),
    "texture_modes": (sc_texture_modes, ()),
    "texture_wrap_hint": (sc_texture_wrap_hint, ()),
    "texture_formats": (sc_texture_formats, ()),
    "mipmap_floor": (sc_mipmap_floor, ()),
    "fog": (sc_fog, ()),
    "lighting_smooth": (sc_lighting(G.GL_SMOOTH), ()),
    "lighting_flat": (sc_lighting(G.GL_FLAT), ()),
    "lighting_phong": (sc_lighting(G.GL_PHONG), ()),
    "color_material": (sc_color_material, ()),
    "blend": (sc_blend, ()),
    "stencil": (sc_stencil, ()),
    "alpha_test": (sc_alpha_test, ()),
    "scissor_mask": (sc_scissor_mask, ()),
    "viewport": (sc_viewport, ()),
    "display_lists": (sc_display_lists, ()),
    "list_blocks": (sc_list_blocks, ()),
    "max_width": (sc_max_width, ("lines",)),
    "max_height": (sc_max_height, ("lines",)),
    "ragged": (sc_ragged, ("lines",)),
    "deferred_colour": (sc_deferred_colour, ()),
    "vertex_arrays": (sc_vertex_arrays, ()),
    "vbo": (sc_vbo, ()),
    "state_in_begin_end": (sc_state_in_begin_end, ()),
    "flat_clip": (sc_flat_clip, ()),
    "extreme_values": (sc_extreme_values, ()),
    "draw_pixels": (sc_draw_pixels, ()),
    "phong_textured_fog": (sc_phong_textured_fog, ()),
    "texture_matrix": (sc_texture_matrix, ()),
    "depth_mix": (sc_depth_mix, ()),
    "lines_states": (sc_lines_states, ("lines",)),
    "points_states": (sc_points_states, ("lines",)),
    "polygon_modes_lit": (sc_polygon_modes_lit, ("lines",)),
}
