"""Seeded synthetic workloads: the headline scenes and the feature scenes used by tests.

Every matrix is computed here in double precision and handed to GL as float32 through
glLoadMatrixf / glMultMatrixf (or as doubles to glFrustum/glOrtho), so a scene is the same
bits on every host and the renderers differ only in how they render it.

Headline configurations (identity of each recipe is in its docstring):
  sphere_scene   — 800x600, UV sphere 32x32 (1,984 triangles), one directional light.
  textured_scene — 1920x1080, 100k triangles straddling the frustum, trilinear texture,
                   8 point lights, EXP fog.
  rop_scene      — 1920x1080, 1M small blended triangles with alpha, stencil and depth tests.
"""
from __future__ import annotations

import math

import numpy as np

from . import gl as G
from .scene import Scene


def frustum_params(fovy_deg, aspect, near, far):
    """gluPerspective's glFrustum arguments (glu.h:114-119), evaluated in double precision."""
    h = near * math.tan(fovy_deg * math.pi / 360.0)
    w = h * aspect
    return (-w, w, -h, h, near, far)


def euler_matrix(ax, ay, az):
    """Column-major float32 rotation Rx(ax) * Ry(ay) * Rz(az), built in double precision."""
    cx, sx, cy, sy, cz, sz = math.cos(ax), math.sin(ax), math.cos(ay), math.sin(ay), math.cos(az), math.sin(az)
    rx = np.array([[1, 0, 0, 0], [0, cx, -sx, 0], [0, sx, cx, 0], [0, 0, 0, 1]], np.float64)
    ry = np.array([[cy, 0, sy, 0], [0, 1, 0, 0], [-sy, 0, cy, 0], [0, 0, 0, 1]], np.float64)
    rz = np.array([[cz, -sz, 0, 0], [sz, cz, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], np.float64)
    m = rx @ ry @ rz
    return np.ascontiguousarray(m.T.reshape(16).astype(np.float32))


def uv_sphere(stacks=32, slices=32, radius=1.0):
    """Positions, normals (float32 [n,3]) and triangle indices (uint32) of a UV sphere.
    Quads are split in two; the degenerate halves at the poles are dropped, so 32x32 gives
    2*32*32 - 2*32 = 1,984 triangles over 33*33 = 1,089 vertices."""
    pos = []
    for i in range(stacks + 1):
        th = math.pi * i / stacks
        for j in range(slices + 1):
            ph = 2 * math.pi * j / slices
            pos.append((math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph)))
    p = np.array(pos, np.float64)
    nrm = p / np.linalg.norm(p, axis=1, keepdims=True)
    idx = []
    w = slices + 1
    for i in range(stacks):
        for j in range(slices):
            a, b, c, d = i * w + j, (i + 1) * w + j, (i + 1) * w + j + 1, i * w + j + 1
            if i != 0:
                idx += [a, b, d]
            if i != stacks - 1:
                idx += [b, c, d]
    return (p * radius).astype(np.float32), nrm.astype(np.float32), np.array(idx, np.uint32)


def frame_start(scene: Scene) -> int:
    """Index of the first call of the per-frame part (the first glClear): everything before
    it uploads resident inputs (buffers, textures) once."""
    for i, (name, _) in enumerate(scene.cmds):
        if name == "glClear":
            return i
    return 0


def _vbo(s: Scene, target, data: np.ndarray, buf_id: int):
    s.glBindBuffer(target, buf_id)
    s.glBufferData(target, int(data.nbytes), data, G.GL_STATIC_DRAW)


def sphere_uv(stacks, slices):
    """Texture coordinates (slice / slices, stack / stacks) per vertex of uv_sphere."""
    i, j = np.meshgrid(np.arange(stacks + 1), np.arange(slices + 1), indexing="ij")
    return np.stack([j / slices, i / stacks], axis=-1).reshape(-1, 2).astype(np.float32)


def sphere_scene(width=800, height=600, seed=0, use_vbo=True, near=0.1, far=100.0, stacks=32, slices=32,
                 light=(0.0, 0.0, 1.0), tex_size=0):
    """Plain single frame: 800x600 RGBA8 + float depth cleared to black, UV sphere r=1 of
    32 stacks x 32 slices (1,984 triangles), gluPerspective(60, w/h, 0.1, 100) at z=-3,
    Euler angles U[0, 2pi) from `seed`, GL_LIGHT0 directional white at (0,0,1,0) set before
    the model rotation, Gouraud shading, GL_LESS, back-face culling, no texture. With
    tex_size > 0 the sphere also carries a tex_size^2 noise texture (seeded by `seed`,
    GL_LINEAR_MIPMAP_LINEAR, GL_MODULATE) mapped by (slice, stack)."""
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0.0, 2 * math.pi, 3)
    pos, nrm, idx = uv_sphere(stacks, slices)
    s = Scene("sphere", width, height)
    if tex_size:
        s.glGenTextures(1, np.zeros(1, np.uint32))
        s.glBindTexture(G.GL_TEXTURE_2D, 1)
        s.glTexImage2D(G.GL_TEXTURE_2D, 0, G.GL_RGBA, tex_size, tex_size, 0, G.GL_RGBA, G.GL_UNSIGNED_BYTE,
                       np.ascontiguousarray(noise_texture(tex_size, seed)))
    uv = sphere_uv(stacks, slices)
    if use_vbo:
        # resident inputs, uploaded before the frame: one interleaved position+normal(+uv)
        # buffer (the array-buffer binding is read at draw time, so one buffer serves every
        # pointer) and an element buffer
        s.glGenBuffers(2, np.zeros(2, np.uint32))
        cols = [pos, nrm] + ([uv] if tex_size else [])
        inter = np.ascontiguousarray(np.concatenate(cols, axis=1).astype(np.float32))
        _vbo(s, G.GL_ARRAY_BUFFER, inter, 1)
        _vbo(s, G.GL_ELEMENT_ARRAY_BUFFER, idx, 2)
    stride = 32 if tex_size else 24
    s.glViewport(0, 0, width, height)
    s.glClearColor(0.0, 0.0, 0.0, 1.0)
    # ---- frame
    s.glClear(G.GL_COLOR_BUFFER_BIT | G.GL_DEPTH_BUFFER_BIT)
    s.glMatrixMode(G.GL_PROJECTION)
    s.glLoadIdentity()
    s.glFrustum(*frustum_params(60.0, width / height, near, far))
    s.glMatrixMode(G.GL_MODELVIEW)
    s.glLoadIdentity()
    s.glLightfv(G.GL_LIGHT0, G.GL_POSITION, np.array([*light, 0], np.float32))
    s.glLightfv(G.GL_LIGHT0, G.GL_DIFFUSE, np.array([1, 1, 1, 1], np.float32))
    s.glEnable(G.GL_LIGHTING)
    s.glEnable(G.GL_LIGHT0)
    s.glShadeModel(G.GL_SMOOTH)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glDepthFunc(G.GL_LESS)
    s.glEnable(G.GL_CULL_FACE)
    s.glCullFace(G.GL_BACK)
    s.glTranslatef(0.0, 0.0, -3.0)
    s.glMultMatrixf(euler_matrix(*ang))
    if tex_size:
        s.glBindTexture(G.GL_TEXTURE_2D, 1)
        s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MIN_FILTER, G.GL_LINEAR_MIPMAP_LINEAR)
        s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MAG_FILTER, G.GL_LINEAR)
        s.glTexEnvi(G.GL_TEXTURE_ENV, G.GL_TEXTURE_ENV_MODE, G.GL_MODULATE)
        s.glEnable(G.GL_TEXTURE_2D)
        s.glEnableClientState(G.GL_TEXTURE_COORD_ARRAY)
    s.glEnableClientState(G.GL_VERTEX_ARRAY)
    s.glEnableClientState(G.GL_NORMAL_ARRAY)
    if use_vbo:
        s.glBindBuffer(G.GL_ARRAY_BUFFER, 1)
        s.glBindBuffer(G.GL_ELEMENT_ARRAY_BUFFER, 2)
        s.glVertexPointer(3, G.GL_FLOAT, stride, 0)
        s.glNormalPointer(G.GL_FLOAT, stride, 12)
        if tex_size:
            s.glTexCoordPointer(2, G.GL_FLOAT, stride, 24)
        s.glDrawElements(G.GL_TRIANGLES, int(idx.size), G.GL_UNSIGNED_INT, 0)
    else:
        s.glVertexPointer(3, G.GL_FLOAT, 0, pos)
        s.glNormalPointer(G.GL_FLOAT, 0, nrm)
        if tex_size:
            s.glTexCoordPointer(2, G.GL_FLOAT, 0, uv)
        s.glDrawElements(G.GL_TRIANGLES, int(idx.size), G.GL_UNSIGNED_INT, idx)
    s.glDisableClientState(G.GL_VERTEX_ARRAY)
    s.glDisableClientState(G.GL_NORMAL_ARRAY)
    if tex_size:
        s.glDisableClientState(G.GL_TEXTURE_COORD_ARRAY)
    return s


def noise_texture(size, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 256, (size, size, 4), dtype=np.uint8)


TEXTURED_SPREAD = 0.33  # per-vertex offset U[-s, s]: ~30 % of the triangles straddle a clip plane


def textured_scene(width=1920, height=1080, ntri=100_000, seed=1, tex_size=512, use_vbo=True,
                   spread=TEXTURED_SPREAD, fog=True, lights=8, min_filter=G.GL_LINEAR_MIPMAP_LINEAR,
                   rotate_z=0.0, modelview_from_caller=False):
    """Textured with clipping and fog: identity modelview/projection; triangle centres
    U[-1.5, 1.5]^3 in clip space with per-vertex offsets U[-s, s]^3; per-vertex RGBA8 colour
    U[0,255], uv U[0,4) with GL_REPEAT, normals U[-1,1]^3; a tex_size^2 RGBA8 noise texture
    with GL_LINEAR_MIPMAP_LINEAR (the reference keeps level 0 plus its own level 1) and
    GL_MODULATE; 8 point lights at seeded positions with GL_COLOR_MATERIAL on so the vertex
    colours reach the lighting; GL_EXP fog, density 0.5; depth test GL_LESS."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-1.5, 1.5, (ntri, 1, 3))
    offs = rng.uniform(-spread, spread, (ntri, 3, 3))
    pos = (centres + offs).reshape(-1, 3).astype(np.float32)
    col = rng.integers(0, 256, (ntri * 3, 4), dtype=np.uint8)
    uv = rng.uniform(0.0, 4.0, (ntri * 3, 2)).astype(np.float32)
    nrm = rng.uniform(-1.0, 1.0, (ntri * 3, 3)).astype(np.float32)
    tex = noise_texture(tex_size, seed)
    lpos = rng.uniform(-2.0, 2.0, (lights, 3)).astype(np.float32)
    lcol = rng.uniform(0.2, 1.0, (lights, 3)).astype(np.float32)

    s = Scene("textured", width, height)
    s.glGenTextures(1, np.zeros(1, np.uint32))
    s.glBindTexture(G.GL_TEXTURE_2D, 1)
    s.glTexImage2D(G.GL_TEXTURE_2D, 0, G.GL_RGBA, tex_size, tex_size, 0, G.GL_RGBA, G.GL_UNSIGNED_BYTE,
                   np.ascontiguousarray(tex))
    if use_vbo:
        # resident inputs: one interleaved buffer pos f32x3 | colour u8x4 | uv f32x2 | normal f32x3 (36 B)
        rec = np.zeros(ntri * 3, dtype=[("p", "<f4", 3), ("c", "u1", 4), ("t", "<f4", 2), ("n", "<f4", 3)])
        rec["p"], rec["c"], rec["t"], rec["n"] = pos, col, uv, nrm
        raw = np.frombuffer(rec.tobytes(), np.uint8)
        s.glGenBuffers(1, np.zeros(1, np.uint32))
        _vbo(s, G.GL_ARRAY_BUFFER, raw, 1)
    s.glViewport(0, 0, width, height)
    s.glClearColor(0.1, 0.1, 0.2, 1.0)
    # ---- frame
    s.glClear(G.GL_COLOR_BUFFER_BIT | G.GL_DEPTH_BUFFER_BIT)
    s.glMatrixMode(G.GL_PROJECTION)
    s.glLoadIdentity()
    s.glMatrixMode(G.GL_MODELVIEW)
    if not modelview_from_caller:  # else the modelview loaded before the frame stays
        s.glLoadIdentity()
        if rotate_z:
            s.glMultMatrixf(euler_matrix(0.0, 0.0, rotate_z))
    s.glBindTexture(G.GL_TEXTURE_2D, 1)
    s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MIN_FILTER, min_filter)
    s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_MAG_FILTER, G.GL_LINEAR)
    s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_WRAP_S, G.GL_REPEAT)
    s.glTexParameteri(G.GL_TEXTURE_2D, G.GL_TEXTURE_WRAP_T, G.GL_REPEAT)
    s.glTexEnvi(G.GL_TEXTURE_ENV, G.GL_TEXTURE_ENV_MODE, G.GL_MODULATE)
    s.glEnable(G.GL_TEXTURE_2D)
    s.glEnable(G.GL_LIGHTING)
    s.glEnable(G.GL_COLOR_MATERIAL)
    s.glColorMaterial(G.GL_FRONT_AND_BACK, G.GL_AMBIENT_AND_DIFFUSE)
    for i in range(lights):
        L = G.GL_LIGHT0 + i
        s.glLightfv(L, G.GL_POSITION, np.array([*lpos[i], 1.0], np.float32))
        s.glLightfv(L, G.GL_DIFFUSE, np.array([*lcol[i], 1.0], np.float32))
        s.glLightf(L, G.GL_CONSTANT_ATTENUATION, 1.0)
        s.glLightf(L, G.GL_LINEAR_ATTENUATION, 0.25)
        s.glLightf(L, G.GL_QUADRATIC_ATTENUATION, 0.1)
        s.glEnable(L)
    if fog:
        s.glEnable(G.GL_FOG)
        s.glFogi(G.GL_FOG_MODE, G.GL_EXP)
        s.glFogf(G.GL_FOG_DENSITY, 0.5)
        s.glFogfv(G.GL_FOG_COLOR, np.array([0.5, 0.5, 0.6, 1.0], np.float32))
    s.glEnable(G.GL_DEPTH_TEST)
    s.glDepthFunc(G.GL_LESS)
    for a in (G.GL_VERTEX_ARRAY, G.GL_COLOR_ARRAY, G.GL_TEXTURE_COORD_ARRAY, G.GL_NORMAL_ARRAY):
        s.glEnableClientState(a)
    if use_vbo:
        s.glBindBuffer(G.GL_ARRAY_BUFFER, 1)
        s.glVertexPointer(3, G.GL_FLOAT, 36, 0)
        s.glColorPointer(4, G.GL_UNSIGNED_BYTE, 36, 12)
        s.glTexCoordPointer(2, G.GL_FLOAT, 36, 16)
        s.glNormalPointer(G.GL_FLOAT, 36, 24)
    else:
        s.glVertexPointer(3, G.GL_FLOAT, 0, pos)
        s.glColorPointer(4, G.GL_UNSIGNED_BYTE, 0, col)
        s.glTexCoordPointer(2, G.GL_FLOAT, 0, uv)
        s.glNormalPointer(G.GL_FLOAT, 0, nrm)
    s.glDrawArrays(G.GL_TRIANGLES, 0, ntri * 3)
    for a in (G.GL_VERTEX_ARRAY, G.GL_COLOR_ARRAY, G.GL_TEXTURE_COORD_ARRAY, G.GL_NORMAL_ARRAY):
        s.glDisableClientState(a)
    return s


def rop_scene(width=1920, height=1080, ntri=1_000_000, seed=2, median_area=20.0, sigma=1.0, use_vbo=True):
    """Order-sensitive ROP stress: identity transforms, ntri triangles with screen area
    LogNormal(ln median, sigma) px, centres uniform over the screen, random orientation,
    depth U[0,1] per triangle (NDC z = 2d-1); RGBA8 colour with alpha U[0,1]; blending
    GL_SRC_ALPHA / GL_ONE_MINUS_SRC_ALPHA in submission order; alpha test GL_GREATER 0.1
    (the reference applies it to textured fragments only, so here it passes everything);
    stencil GL_ALWAYS with GL_INCR on depth pass; depth GL_LEQUAL with depth writes off."""
    rng = np.random.default_rng(seed)
    area = rng.lognormal(math.log(median_area), sigma, ntri)
    r = np.sqrt(4.0 * area / (3.0 * math.sqrt(3.0)))  # circumradius of an equilateral triangle
    cx = rng.uniform(0, width, ntri)
    cy = rng.uniform(0, height, ntri)
    th = rng.uniform(0, 2 * math.pi, ntri)
    depth = rng.uniform(0.0, 1.0, ntri)
    k = np.arange(3)[None, :]
    ang = th[:, None] + k * (2 * math.pi / 3)
    px = cx[:, None] + r[:, None] * np.cos(ang)
    py = cy[:, None] + r[:, None] * np.sin(ang)
    x = px / width * 2.0 - 1.0
    y = py / height * 2.0 - 1.0
    z = np.repeat(depth[:, None] * 2.0 - 1.0, 3, axis=1)
    pos = np.stack([x, y, z], axis=-1).reshape(-1, 3).astype(np.float32)
    col = rng.integers(0, 256, (ntri, 4), dtype=np.uint8)
    col = np.repeat(col, 3, axis=0)

    s = Scene("rop", width, height)
    if use_vbo:
        rec = np.zeros(ntri * 3, dtype=[("p", "<f4", 3), ("c", "u1", 4)])
        rec["p"], rec["c"] = pos, col
        raw = np.frombuffer(rec.tobytes(), np.uint8)
        s.glGenBuffers(1, np.zeros(1, np.uint32))
        _vbo(s, G.GL_ARRAY_BUFFER, raw, 1)
    s.glViewport(0, 0, width, height)
    s.glClearColor(0.0, 0.0, 0.0, 1.0)
    s.glClearStencil(0)
    # ---- frame
    s.glClear(G.GL_COLOR_BUFFER_BIT | G.GL_DEPTH_BUFFER_BIT | G.GL_STENCIL_BUFFER_BIT)
    s.glMatrixMode(G.GL_PROJECTION)
    s.glLoadIdentity()
    s.glMatrixMode(G.GL_MODELVIEW)
    s.glLoadIdentity()
    s.glEnable(G.GL_BLEND)
    s.glBlendFunc(G.GL_SRC_ALPHA, G.GL_ONE_MINUS_SRC_ALPHA)
    s.glEnable(G.GL_ALPHA_TEST)
    s.glAlphaFunc(G.GL_GREATER, 0.1)
    s.glEnable(G.GL_STENCIL_TEST)
    s.glStencilFunc(G.GL_ALWAYS, 0, 0xFF)
    s.glStencilOp(G.GL_KEEP, G.GL_KEEP, G.GL_INCR)
    s.glEnable(G.GL_DEPTH_TEST)
    s.glDepthFunc(G.GL_LEQUAL)
    s.glDepthMask(0)
    s.glEnableClientState(G.GL_VERTEX_ARRAY)
    s.glEnableClientState(G.GL_COLOR_ARRAY)
    if use_vbo:
        s.glBindBuffer(G.GL_ARRAY_BUFFER, 1)
        s.glVertexPointer(3, G.GL_FLOAT, 16, 0)
        s.glColorPointer(4, G.GL_UNSIGNED_BYTE, 16, 12)
    else:
        s.glVertexPointer(3, G.GL_FLOAT, 0, pos)
        s.glColorPointer(4, G.GL_UNSIGNED_BYTE, 0, col)
    s.glDrawArrays(G.GL_TRIANGLES, 0, ntri * 3)
    s.glDisableClientState(G.GL_VERTEX_ARRAY)
    s.glDisableClientState(G.GL_COLOR_ARRAY)
    return s


def _log_uniform(rng, lo, hi):
    return math.exp(rng.uniform(math.log(lo), math.log(hi)))


def uneven_frame(index, seed=3, min_side=64, max_side=1024, min_tri=100, max_tri=200_000, tex_size=256,
                 use_vbo=True):
    """Frame `index` of the uneven batch: width and height log-uniform in [min_side, max_side],
    a triangle count log-uniform in [min_tri, max_tri], drawn with probability 1/2 like the
    sphere frame (a UV sphere tessellated to about that many triangles, its own rotation and
    directional light) or like the textured frame (that many clip-straddling triangles, its
    own rotation about z and 8 point lights); each frame has its own tex_size^2 mipmapped
    noise texture. Geometry sits in buffer objects uploaded before the frame (use_vbo) or
    in client arrays read at every draw."""
    rng = np.random.default_rng([seed, index])
    w = int(round(_log_uniform(rng, min_side, max_side)))
    h = int(round(_log_uniform(rng, min_side, max_side)))
    ntri = int(round(_log_uniform(rng, min_tri, max_tri)))
    fseed = int(rng.integers(0, 2**31 - 1))
    if rng.uniform() < 0.5:
        n = max(3, int(round(0.5 + math.sqrt(0.25 + ntri / 2.0))))  # 2 n (n - 1) triangles
        light = rng.normal(size=3)
        light = tuple(float(v) for v in (light / np.linalg.norm(light)).astype(np.float32))
        s = sphere_scene(w, h, seed=fseed, stacks=n, slices=n, light=light, tex_size=tex_size, use_vbo=use_vbo)
        s.name = f"uneven{index}_sphere"
    else:
        s = textured_scene(w, h, ntri=ntri, seed=fseed, tex_size=tex_size,
                           rotate_z=float(rng.uniform(0.0, 2 * math.pi)), use_vbo=use_vbo)
        s.name = f"uneven{index}_textured"
    return s


def uneven_batch(nframes=256, seed=3, **kw):
    """The batched uneven-frames workload: `nframes` independent frames (uneven_frame)."""
    return [uneven_frame(i, seed=seed, **kw) for i in range(nframes)]


SERVE_RESOLUTIONS = ((256, 256), (512, 512), (1280, 720), (1920, 1080))


def serve_scenes(nscenes=32, seed=5, min_tri=1000, max_tri=500_000, tex_sizes=(256, 512, 1024, 2048),
                 width=1920, height=1080):
    """Resident scenes of the serving workload, built like the textured frame (clip-straddling
    triangles, 8 point lights, EXP fog, trilinear texture): triangle counts log-uniform in
    [min_tri, max_tri], power-of-two textures log-uniform over tex_sizes. The frame part
    (from the first glClear) takes its modelview from the caller."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nscenes):
        ntri = int(round(_log_uniform(rng, min_tri, max_tri)))
        tex = int(tex_sizes[int(rng.integers(0, len(tex_sizes)))])
        s = textured_scene(width, height, ntri=ntri, seed=int(rng.integers(0, 2**31 - 1)), tex_size=tex,
                           modelview_from_caller=True)
        s.name = f"serve_scene{i}"
        out.append(s)
    return out


def serve_trace(duration_s=60.0, rate=2000.0, nscenes=32, seed=6, resolutions=SERVE_RESOLUTIONS):
    """Poisson arrivals at `rate` per second for `duration_s`: (arrival s, scene, width,
    height, modelview) with the scene uniform, the resolution uniform over `resolutions`
    and the modelview a rotation drawn from the request's own seed."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration_s:
            break
        w, h = resolutions[int(rng.integers(0, len(resolutions)))]
        r = np.random.default_rng([seed, len(out)])
        mv = euler_matrix(r.uniform(-0.3, 0.3), r.uniform(-0.3, 0.3), r.uniform(0.0, 2 * math.pi))
        out.append((t, int(rng.integers(0, nscenes)), w, h, mv))
    return out


def scene_triangles(scene: Scene) -> int:
    """Input triangles of a scene's draw calls (GL_TRIANGLES arrays and elements)."""
    n = 0
    for name, args in scene.cmds:
        if name == "glDrawArrays" and args[0] == G.GL_TRIANGLES:
            n += int(args[2]) // 3
        elif name == "glDrawElements" and args[0] == G.GL_TRIANGLES:
            n += int(args[1]) // 3
    return n


HEADLINE = {
    "sphere": sphere_scene,
    "textured": textured_scene,
    "rop": rop_scene,
}
