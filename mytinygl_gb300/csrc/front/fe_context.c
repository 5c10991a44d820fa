/*
 * fe_context.c — context lifecycle, error state, capability and fixed-function state
 * setters, fog, texture environment and the lighting/material API.
 *
 * Semantics follow MyTinyGL's src/gl_api.c line for line where the reference defines them
 * (citations per function); storage follows the GPU design (fe_internal.h).
 */
#include "fe_internal.h"

__thread GLState *fe_ctx = NULL;

void fe_set_error(GLState *c, GLenum e)
{
    /* gl_set_error (gl_api.c:30-35): only the first error sticks */
    if (c && c->error == GL_NO_ERROR) c->error = e;
}

void fe_dev_error(GLState *c, int status)
{
    if (!c || status == MTGL_OK) return;
    c->dev_status = status;
    fe_set_error(c, status == MTGL_ERR_OOM ? GL_OUT_OF_MEMORY : GL_INVALID_OPERATION);
}

void fe_state_changed(GLState *c)
{
    c->vs_dirty = 1;
}

/* light_init (lighting.h:18-32) */
void fe_light_init(mtgl_light *l, int index)
{
    memset(l, 0, sizeof(*l));
    l->ambient[3] = 1.0f;
    float d = index == 0 ? 1.0f : 0.0f;
    for (int i = 0; i < 3; i++) { l->diffuse[i] = d; l->specular[i] = d; }
    l->diffuse[3] = 1.0f;
    l->specular[3] = 1.0f;
    l->position[2] = 1.0f;
    l->spot_direction[2] = -1.0f;
    l->spot_exponent = 0.0f;
    l->spot_cutoff = 180.0f;
    l->constant_attenuation = 1.0f;
    l->enabled = 0;
}

/* material_init (lighting.h:35-41) */
void fe_material_init(mtgl_material *m)
{
    memset(m, 0, sizeof(*m));
    for (int i = 0; i < 3; i++) { m->ambient[i] = 0.2f; m->diffuse[i] = 0.8f; }
    m->ambient[3] = 1.0f;
    m->diffuse[3] = 1.0f;
    m->specular[3] = 1.0f;
    m->emission[3] = 1.0f;
    m->shininess = 0.0f;
}

static void set4(float *d, float a, float b, float c, float e) { d[0] = a; d[1] = b; d[2] = c; d[3] = e; }

/* gl_create_context (gl_api.c:81-236): same defaults; the framebuffer is device memory */
GLState *gl_create_context(int32_t width, int32_t height)
{
    if (width <= 0 || height <= 0 || width > FE_MAX_FB_DIM || height > FE_MAX_FB_DIM) return NULL;
    GLState *c = (GLState *)calloc(1, sizeof(GLState));
    if (!c) return NULL;
    if (mtgl_dev_create(width, height, &c->dev) != MTGL_OK) {
        free(c);
        return NULL;
    }
    c->width = width;
    c->height = height;
    set4(c->clear_color, 0.0f, 0.0f, 0.0f, 1.0f);
    c->clear_depth = 1.0;
    c->viewport[0] = 0; c->viewport[1] = 0; c->viewport[2] = width; c->viewport[3] = height;
    set4(c->cur_color, 1.0f, 1.0f, 1.0f, 1.0f);
    c->cur_tex[0] = 0.0f; c->cur_tex[1] = 0.0f;
    c->cur_normal[0] = 0.0f; c->cur_normal[1] = 0.0f; c->cur_normal[2] = 1.0f;
    c->matrix_mode = GL_MODELVIEW;
    for (int i = 0; i < FE_MAX_STACK; i++) {
        fe_mat4_identity(c->mv[i]);
        fe_mat4_identity(c->proj[i]);
        fe_mat4_identity(c->texm[i]);
    }
    c->blend_src = GL_ONE;
    c->blend_dst = GL_ZERO;
    c->cull_mode = GL_BACK;
    c->front_face = GL_CCW;
    c->depth_func = GL_LESS;
    c->depth_mask = GL_TRUE;
    c->alpha_func = GL_ALWAYS;
    c->alpha_ref = 0.0f;
    c->scissor[0] = 0; c->scissor[1] = 0; c->scissor[2] = width; c->scissor[3] = height;
    c->stencil_func = GL_ALWAYS;
    c->stencil_ref = 0;
    c->stencil_mask = 0xFFFFFFFFu;
    c->stencil_fail = c->stencil_zfail = c->stencil_zpass = GL_KEEP;
    c->stencil_writemask = 0xFFFFFFFFu;
    c->stencil_clear = 0;
    c->depth_near = 0.0;
    c->depth_far = 1.0;
    for (int i = 0; i < 4; i++) c->color_mask[i] = GL_TRUE;
    c->line_width = 1.0f;
    c->point_size = 1.0f;
    c->poly_front = c->poly_back = GL_FILL;
    c->tex_env_mode = GL_MODULATE;
    set4(c->tex_env_color, 0.0f, 0.0f, 0.0f, 0.0f);
    c->persp_hint = GL_DONT_CARE;
    c->raster_valid = GL_TRUE;
    c->fog_mode = GL_EXP;
    c->fog_density = 1.0f;
    c->fog_start = 0.0f;
    c->fog_end = 1.0f;
    set4(c->fog_color, 0.0f, 0.0f, 0.0f, 0.0f);
    for (int i = 0; i < FE_MAX_LIGHTS; i++) fe_light_init(&c->lit.lights[i], i);
    fe_material_init(&c->lit.front);
    c->lit.back = c->lit.front;
    set4(c->lit.model_ambient, 0.2f, 0.2f, 0.2f, 1.0f);
    c->color_material_face = GL_FRONT_AND_BACK;
    c->color_material_mode = GL_AMBIENT_AND_DIFFUSE;
    c->shade_model = GL_SMOOTH;
    c->error = GL_NO_ERROR;
    c->vs_dirty = 1;
    return c;
}

void gl_destroy_context(GLState *c)
{
    if (!c) return;
    fe_lists_free(c);
    fe_buffers_free(c);
    fe_textures_free(c);
    mtgl_dev_destroy(c->dev);
    free(c->imm);
    free(c->imm_vs);
    free(c->vstates);
    free(c->host_color);
    if (fe_ctx == c) fe_ctx = NULL;
    free(c);
}

void gl_make_current(GLState *c) { fe_ctx = c; }
GLState *gl_get_current_context(void) { return fe_ctx; }

int mtgl_finish(GLState *c)
{
    if (!c) return MTGL_ERR_INVALID;
    return mtgl_dev_finish(c->dev);
}

int mtgl_read_framebuffer(GLState *c, uint32_t *color, float *depth, uint8_t *stencil)
{
    if (!c) return MTGL_ERR_INVALID;
    return mtgl_dev_read(c->dev, color, depth, stencil);
}

const uint32_t *mtgl_color_buffer(GLState *c)
{
    if (!c) return NULL;
    if (!c->host_color) {
        c->host_color = (uint32_t *)malloc((size_t)c->width * (size_t)c->height * sizeof(uint32_t));
        if (!c->host_color) return NULL;
    }
    if (mtgl_dev_read(c->dev, c->host_color, NULL, NULL) != MTGL_OK) return NULL;
    return c->host_color;
}

int mtgl_framebuffer_size(GLState *c, int32_t *w, int32_t *h)
{
    if (!c) return MTGL_ERR_INVALID;
    if (w) *w = c->width;
    if (h) *h = c->height;
    return MTGL_OK;
}

const char *mtgl_backend_name(void) { return mtgl_dev_backend_name(); }

int mtgl_get_stats(GLState *c, mtgl_stats *out) { return c ? mtgl_dev_stats(c->dev, out) : MTGL_ERR_INVALID; }
int mtgl_reset_stats(GLState *c) { return c ? mtgl_dev_reset_stats(c->dev) : MTGL_ERR_INVALID; }
int mtgl_set_profiling(GLState *c, int enable) { return c ? mtgl_dev_profile(c->dev, enable) : MTGL_ERR_INVALID; }
int mtgl_get_timings(GLState *c, mtgl_timings *out) { return c ? mtgl_dev_timings(c->dev, out) : MTGL_ERR_INVALID; }
void *mtgl_cuda_stream(GLState *c) { return c ? mtgl_dev_stream(c->dev) : NULL; }
int mtgl_set_option(GLState *c, int option, int value)
{
    if (!c) return MTGL_ERR_INVALID;
    int st = mtgl_dev_set_option(c->dev, option, value);
    if (st == MTGL_OK && option == MTGL_OPT_MIPMAP_CHAIN) c->mipmap_chain = value != 0;
    return st;
}

/* the back end of a context, for back-end entry points that take a GLState (not exported) */
mtgl_dev *fe_context_device(GLState *c) { return c ? c->dev : NULL; }

/* ---- capabilities (gl_api.c:351-407) ---- */
static uint32_t cap_flag(GLenum cap)
{
    switch (cap) {
    case GL_DEPTH_TEST: return F_DEPTH_TEST;
    case GL_CULL_FACE: return F_CULL_FACE;
    case GL_BLEND: return F_BLEND;
    case GL_TEXTURE_2D: return F_TEXTURE_2D;
    case GL_LIGHTING: return F_LIGHTING;
    case GL_FOG: return F_FOG;
    case GL_NORMALIZE: return F_NORMALIZE;
    case GL_COLOR_MATERIAL: return F_COLOR_MATERIAL;
    case GL_ALPHA_TEST: return F_ALPHA_TEST;
    case GL_SCISSOR_TEST: return F_SCISSOR_TEST;
    case GL_STENCIL_TEST: return F_STENCIL_TEST;
    default: return 0;
    }
}

static void set_cap(GLenum cap, int on)
{
    uint32_t f = cap_flag(cap);
    fe_state_changed(fe_ctx);
    if (f) {
        if (on) fe_ctx->flags |= f; else fe_ctx->flags &= ~f;
        return;
    }
    if (cap >= GL_LIGHT0 && cap <= GL_LIGHT7) {
        fe_ctx->lit.lights[cap - GL_LIGHT0].enabled = on ? GL_TRUE : GL_FALSE;
        return;
    }
    fe_set_error(fe_ctx, GL_INVALID_ENUM);
}

void glEnable(GLenum cap)
{
    CHECK_CTX();
    if (fe_rec_e(LC_ENABLE, cap)) return;
    set_cap(cap, 1);
}

void glDisable(GLenum cap)
{
    CHECK_CTX();
    if (fe_rec_e(LC_DISABLE, cap)) return;
    set_cap(cap, 0);
}

/* glClear (gl_api.c:409-457): scissor-limited, ignores the write masks */
void glClear(GLbitfield mask)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    int32_t x0, y0, x1, y1;
    if (c->flags & F_SCISSOR_TEST) {
        x0 = c->scissor[0];
        y0 = c->scissor[1];
        x1 = c->scissor[0] + c->scissor[2];
        y1 = c->scissor[1] + c->scissor[3];
        if (x0 < 0) x0 = 0;
        if (y0 < 0) y0 = 0;
        if (x1 > c->width) x1 = c->width;
        if (y1 > c->height) y1 = c->height;
    } else {
        x0 = 0; y0 = 0; x1 = c->width; y1 = c->height;
    }
    uint32_t m = mask & (GL_COLOR_BUFFER_BIT | GL_DEPTH_BUFFER_BIT | GL_STENCIL_BUFFER_BIT);
    if (!m || x0 >= x1 || y0 >= y1) return;
    uint32_t col = fe_color_to_rgba32(c->clear_color);
    float depth = (float)c->clear_depth;
    uint8_t st = (uint8_t)(c->stencil_clear & 0xFF);
    fe_dev_error(c, mtgl_dev_clear(c->dev, m, x0, y0, x1, y1, col, depth, st));
}

void glClearColor(GLclampf r, GLclampf g, GLclampf b, GLclampf a)
{
    CHECK_CTX();
    set4(fe_ctx->clear_color, r, g, b, a);
}

void glClearDepth(GLclampd depth)
{
    CHECK_CTX();
    fe_ctx->clear_depth = depth;
}

void glViewport(GLint x, GLint y, GLsizei w, GLsizei h)
{
    CHECK_CTX();
    fe_ctx->viewport[0] = x; fe_ctx->viewport[1] = y;
    fe_ctx->viewport[2] = w; fe_ctx->viewport[3] = h;
}

/* ---- fixed-function state (gl_api.c:909-1176) ---- */
static int valid_blend_factor(GLenum f, int is_src)
{
    switch (f) {
    case GL_ZERO: case GL_ONE: case GL_SRC_COLOR: case GL_ONE_MINUS_SRC_COLOR:
    case GL_DST_COLOR: case GL_ONE_MINUS_DST_COLOR: case GL_SRC_ALPHA: case GL_ONE_MINUS_SRC_ALPHA:
    case GL_DST_ALPHA: case GL_ONE_MINUS_DST_ALPHA: case GL_CONSTANT_COLOR:
    case GL_ONE_MINUS_CONSTANT_COLOR: case GL_CONSTANT_ALPHA: case GL_ONE_MINUS_CONSTANT_ALPHA:
        return 1;
    case GL_SRC_ALPHA_SATURATE:
        return is_src;
    default:
        return 0;
    }
}

void glBlendFunc(GLenum s, GLenum d)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_BLEND_FUNC, {s, d, 0}, 0, {0}, {0}};
    if (fe_rec(&cmd)) return;
    if (!valid_blend_factor(s, 1) || !valid_blend_factor(d, 0)) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_ctx->blend_src = s;
    fe_ctx->blend_dst = d;
}

void glCullFace(GLenum mode)
{
    CHECK_CTX();
    if (fe_rec_e(LC_CULL_FACE, mode)) return;
    if (mode != GL_FRONT && mode != GL_BACK && mode != GL_FRONT_AND_BACK) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_ctx->cull_mode = mode;
}

void glFrontFace(GLenum mode)
{
    CHECK_CTX();
    if (fe_rec_e(LC_FRONT_FACE, mode)) return;
    if (mode != GL_CW && mode != GL_CCW) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_ctx->front_face = mode;
}

void glDepthFunc(GLenum f)
{
    CHECK_CTX();
    if (fe_rec_e(LC_DEPTH_FUNC, f)) return;
    if (f < GL_NEVER || f > GL_ALWAYS) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_ctx->depth_func = f;
}

void glDepthMask(GLboolean flag)
{
    CHECK_CTX();
    if (fe_rec_e(LC_DEPTH_MASK, flag)) return;
    fe_ctx->depth_mask = flag;
}

void glAlphaFunc(GLenum f, GLclampf ref)
{
    CHECK_CTX();
    if (f < GL_NEVER || f > GL_ALWAYS) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_ctx->alpha_func = f;
    if (ref < 0.0f) ref = 0.0f;
    if (ref > 1.0f) ref = 1.0f;
    fe_ctx->alpha_ref = ref;
}

void glLineWidth(GLfloat w)
{
    CHECK_CTX();
    if (w <= 0.0f || isnan(w) || isinf(w)) {
        fe_set_error(fe_ctx, GL_INVALID_VALUE);
        return;
    }
    fe_ctx->line_width = w;
}

void glPointSize(GLfloat s)
{
    CHECK_CTX();
    if (s <= 0.0f || isnan(s) || isinf(s)) {
        fe_set_error(fe_ctx, GL_INVALID_VALUE);
        return;
    }
    fe_ctx->point_size = s;
}

void glPolygonMode(GLenum face, GLenum mode)
{
    CHECK_CTX();
    if (face != GL_FRONT && face != GL_BACK && face != GL_FRONT_AND_BACK) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    if (mode != GL_POINT && mode != GL_LINE && mode != GL_FILL) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    if (face == GL_FRONT || face == GL_FRONT_AND_BACK) fe_ctx->poly_front = mode;
    if (face == GL_BACK || face == GL_FRONT_AND_BACK) fe_ctx->poly_back = mode;
}

void glScissor(GLint x, GLint y, GLsizei w, GLsizei h)
{
    CHECK_CTX();
    if (w < 0 || h < 0) {
        fe_set_error(fe_ctx, GL_INVALID_VALUE);
        return;
    }
    fe_ctx->scissor[0] = x; fe_ctx->scissor[1] = y;
    fe_ctx->scissor[2] = w; fe_ctx->scissor[3] = h;
}

void glDepthRange(GLclampd n, GLclampd f)
{
    CHECK_CTX();
    if (n < 0.0) n = 0.0;
    if (n > 1.0) n = 1.0;
    if (f < 0.0) f = 0.0;
    if (f > 1.0) f = 1.0;
    fe_ctx->depth_near = n;
    fe_ctx->depth_far = f;
}

void glColorMask(GLboolean r, GLboolean g, GLboolean b, GLboolean a)
{
    CHECK_CTX();
    fe_ctx->color_mask[0] = r; fe_ctx->color_mask[1] = g;
    fe_ctx->color_mask[2] = b; fe_ctx->color_mask[3] = a;
}

static int valid_cmp(GLenum f)
{
    return f >= GL_NEVER && f <= GL_ALWAYS;
}

void glStencilFunc(GLenum f, GLint ref, GLuint mask)
{
    CHECK_CTX();
    if (!valid_cmp(f)) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_ctx->stencil_func = f;
    fe_ctx->stencil_ref = ref;
    fe_ctx->stencil_mask = mask;
}

static int valid_stencil_op(GLenum op)
{
    switch (op) {
    case GL_KEEP: case GL_ZERO: case GL_REPLACE: case GL_INCR: case GL_INCR_WRAP:
    case GL_DECR: case GL_DECR_WRAP: case GL_INVERT:
        return 1;
    default:
        return 0;
    }
}

void glStencilOp(GLenum sfail, GLenum dpfail, GLenum dppass)
{
    CHECK_CTX();
    if (!valid_stencil_op(sfail) || !valid_stencil_op(dpfail) || !valid_stencil_op(dppass)) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_ctx->stencil_fail = sfail;
    fe_ctx->stencil_zfail = dpfail;
    fe_ctx->stencil_zpass = dppass;
}

void glStencilMask(GLuint mask)
{
    CHECK_CTX();
    fe_ctx->stencil_writemask = mask;
}

void glClearStencil(GLint s)
{
    CHECK_CTX();
    fe_ctx->stencil_clear = s;
}

void glPixelStorei(GLenum pname, GLint param)
{
    CHECK_CTX();
    if (pname == GL_PACK_ALIGNMENT || pname == GL_UNPACK_ALIGNMENT) {
        if (param != 1 && param != 2 && param != 4 && param != 8) fe_set_error(fe_ctx, GL_INVALID_VALUE);
    } else {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
    }
}

void glHint(GLenum target, GLenum mode)
{
    CHECK_CTX();
    if (mode != GL_DONT_CARE && mode != GL_FASTEST && mode != GL_NICEST) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    switch (target) {
    case GL_PERSPECTIVE_CORRECTION_HINT: fe_ctx->persp_hint = mode; break;
    case GL_POINT_SMOOTH_HINT: case GL_LINE_SMOOTH_HINT: case GL_FOG_HINT: break;
    default: fe_set_error(fe_ctx, GL_INVALID_ENUM); break;
    }
}

void glFlush(void)
{
    CHECK_CTX();
    fe_dev_error(fe_ctx, mtgl_dev_flush(fe_ctx->dev));
}

void glFinish(void)
{
    CHECK_CTX();
    fe_dev_error(fe_ctx, mtgl_dev_finish(fe_ctx->dev));
}

GLenum glGetError(void)
{
    if (!fe_ctx) return GL_NO_ERROR;
    GLenum e = fe_ctx->error;
    fe_ctx->error = GL_NO_ERROR;
    return e;
}

/* ---- fog (gl_api.c:1429-1512) ---- */
static int valid_fog_mode(GLenum m) { return m == GL_LINEAR || m == GL_EXP || m == GL_EXP2; }

void glFogi(GLenum pname, GLint param)
{
    CHECK_CTX();
    if (pname == GL_FOG_MODE) {
        if (!valid_fog_mode((GLenum)param)) {
            fe_set_error(fe_ctx, GL_INVALID_ENUM);
            return;
        }
        fe_ctx->fog_mode = (GLenum)param;
    } else {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
    }
}

static void fog_scalar(GLenum pname, const GLfloat *p)
{
    switch (pname) {
    case GL_FOG_MODE: {
        GLenum m = (GLenum)fe_f2i(p[0]);
        if (!valid_fog_mode(m)) {
            fe_set_error(fe_ctx, GL_INVALID_ENUM);
            return;
        }
        fe_ctx->fog_mode = m;
        break;
    }
    case GL_FOG_DENSITY:
        if (p[0] < 0.0f) {
            fe_set_error(fe_ctx, GL_INVALID_VALUE);
            return;
        }
        fe_ctx->fog_density = p[0];
        break;
    case GL_FOG_START: fe_ctx->fog_start = p[0]; break;
    case GL_FOG_END: fe_ctx->fog_end = p[0]; break;
    default: fe_set_error(fe_ctx, GL_INVALID_ENUM); break;
    }
}

void glFogf(GLenum pname, GLfloat param)
{
    CHECK_CTX();
    fog_scalar(pname, &param);
}

void glFogfv(GLenum pname, const GLfloat *params)
{
    CHECK_CTX();
    if (pname == GL_FOG_COLOR) {
        set4(fe_ctx->fog_color, params[0], params[1], params[2], params[3]);
        return;
    }
    fog_scalar(pname, params);
}

/* ---- texture environment (gl_api.c:3193-3243) ---- */
void glTexEnvi(GLenum target, GLenum pname, GLint param)
{
    CHECK_CTX();
    if (target != GL_TEXTURE_ENV || pname != GL_TEXTURE_ENV_MODE) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    switch (param) {
    case GL_MODULATE: case GL_DECAL: case GL_REPLACE: case GL_BLEND: case GL_ADD:
        fe_ctx->tex_env_mode = (GLenum)param;
        break;
    default:
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        break;
    }
}

void glTexEnvf(GLenum target, GLenum pname, GLfloat param)
{
    glTexEnvi(target, pname, (GLint)fe_f2i(param));
}

void glTexEnvfv(GLenum target, GLenum pname, const GLfloat *params)
{
    CHECK_CTX();
    if (!params) return;
    if (target != GL_TEXTURE_ENV) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    if (pname == GL_TEXTURE_ENV_MODE)
        glTexEnvi(target, pname, (GLint)fe_f2i(params[0]));
    else if (pname == GL_TEXTURE_ENV_COLOR)
        set4(fe_ctx->tex_env_color, params[0], params[1], params[2], params[3]);
    else
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
}

/* ---- lights and materials (gl_api.c:1945-2262) ---- */
void glLightfv(GLenum light, GLenum pname, const GLfloat *p)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_LIGHTFV, {light, pname, 0}, 0, {p[0], p[1], p[2], p[3]}, {0}};
    if (fe_rec(&cmd)) return;
    if (light < GL_LIGHT0 || light > GL_LIGHT7) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    GLState *c = fe_ctx;
    mtgl_light *l = &c->lit.lights[light - GL_LIGHT0];
    fe_state_changed(c);
    switch (pname) {
    case GL_AMBIENT: set4(l->ambient, p[0], p[1], p[2], p[3]); break;
    case GL_DIFFUSE: set4(l->diffuse, p[0], p[1], p[2], p[3]); break;
    case GL_SPECULAR: set4(l->specular, p[0], p[1], p[2], p[3]); break;
    case GL_POSITION: {
        /* transformed by the modelview current at call time (gl_api.c:1966-1971) */
        float v[4] = {p[0], p[1], p[2], p[3]};
        fe_mat4_mul_vec4(c->mv[c->mv_depth], v, l->position);
        break;
    }
    case GL_SPOT_DIRECTION: {
        float v[4] = {p[0], p[1], p[2], 0.0f}, o[4];
        fe_mat4_mul_vec4(c->mv[c->mv_depth], v, o);
        l->spot_direction[0] = o[0]; l->spot_direction[1] = o[1]; l->spot_direction[2] = o[2];
        break;
    }
    case GL_SPOT_EXPONENT: l->spot_exponent = p[0]; break;
    case GL_SPOT_CUTOFF: l->spot_cutoff = p[0]; break;
    case GL_CONSTANT_ATTENUATION: l->constant_attenuation = p[0]; break;
    case GL_LINEAR_ATTENUATION: l->linear_attenuation = p[0]; break;
    case GL_QUADRATIC_ATTENUATION: l->quadratic_attenuation = p[0]; break;
    default: break; /* the reference ignores unknown pnames silently */
    }
}

void glLightf(GLenum light, GLenum pname, GLfloat param)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_LIGHTF, {light, pname, 0}, 0, {param}, {0}};
    if (fe_rec(&cmd)) return;
    GLfloat p[4] = {param, param, param, param};
    glLightfv(light, pname, p);
}

void glLighti(GLenum light, GLenum pname, GLint param) { glLightf(light, pname, (GLfloat)param); }

void glLightiv(GLenum light, GLenum pname, const GLint *params)
{
    GLfloat p[4] = {(GLfloat)params[0], (GLfloat)params[1], (GLfloat)params[2], (GLfloat)params[3]};
    glLightfv(light, pname, p);
}

void glMaterialfv(GLenum face, GLenum pname, const GLfloat *p)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_MATERIALFV, {face, pname, 0}, 0, {p[0], p[1], p[2], p[3]}, {0}};
    if (fe_rec(&cmd)) return;
    if (face != GL_FRONT && face != GL_BACK && face != GL_FRONT_AND_BACK) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    mtgl_material *mats[2] = {NULL, NULL};
    if (face == GL_FRONT || face == GL_FRONT_AND_BACK) mats[0] = &fe_ctx->lit.front;
    if (face == GL_BACK || face == GL_FRONT_AND_BACK) mats[1] = &fe_ctx->lit.back;
    fe_state_changed(fe_ctx);
    for (int k = 0; k < 2; k++) {
        mtgl_material *m = mats[k];
        if (!m) continue;
        switch (pname) {
        case GL_AMBIENT: set4(m->ambient, p[0], p[1], p[2], p[3]); break;
        case GL_DIFFUSE: set4(m->diffuse, p[0], p[1], p[2], p[3]); break;
        case GL_SPECULAR: set4(m->specular, p[0], p[1], p[2], p[3]); break;
        case GL_EMISSION: set4(m->emission, p[0], p[1], p[2], p[3]); break;
        case GL_SHININESS: m->shininess = p[0]; break;
        case GL_AMBIENT_AND_DIFFUSE:
            set4(m->ambient, p[0], p[1], p[2], p[3]);
            set4(m->diffuse, p[0], p[1], p[2], p[3]);
            break;
        default:
            if (k == 0 || !mats[0]) fe_set_error(fe_ctx, GL_INVALID_ENUM);
            return;
        }
    }
}

void glMaterialf(GLenum face, GLenum pname, GLfloat param)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_MATERIALF, {face, pname, 0}, 0, {param}, {0}};
    if (fe_rec(&cmd)) return;
    GLfloat p[4] = {param, param, param, param};
    glMaterialfv(face, pname, p);
}

void glMateriali(GLenum face, GLenum pname, GLint param) { glMaterialf(face, pname, (GLfloat)param); }

void glMaterialiv(GLenum face, GLenum pname, const GLint *params)
{
    GLfloat p[4] = {(GLfloat)params[0], (GLfloat)params[1], (GLfloat)params[2], (GLfloat)params[3]};
    glMaterialfv(face, pname, p);
}

void glLightModelfv(GLenum pname, const GLfloat *p)
{
    CHECK_CTX();
    fe_state_changed(fe_ctx);
    switch (pname) {
    case GL_LIGHT_MODEL_AMBIENT: set4(fe_ctx->lit.model_ambient, p[0], p[1], p[2], p[3]); break;
    case GL_LIGHT_MODEL_LOCAL_VIEWER: fe_ctx->lit.local_viewer = (p[0] != 0.0f); break;
    case GL_LIGHT_MODEL_TWO_SIDE: fe_ctx->lit.two_side = (p[0] != 0.0f); break;
    default: break;
    }
}

void glLightModelf(GLenum pname, GLfloat param)
{
    GLfloat p[4] = {param, param, param, param};
    glLightModelfv(pname, p);
}

void glLightModeli(GLenum pname, GLint param) { glLightModelf(pname, (GLfloat)param); }

void glLightModeliv(GLenum pname, const GLint *params)
{
    GLfloat p[4] = {(GLfloat)params[0], (GLfloat)params[1], (GLfloat)params[2], (GLfloat)params[3]};
    glLightModelfv(pname, p);
}

void glColorMaterial(GLenum face, GLenum mode)
{
    CHECK_CTX();
    if (face != GL_FRONT && face != GL_BACK && face != GL_FRONT_AND_BACK) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    if (mode != GL_EMISSION && mode != GL_AMBIENT && mode != GL_DIFFUSE && mode != GL_SPECULAR &&
        mode != GL_AMBIENT_AND_DIFFUSE) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_state_changed(fe_ctx);
    fe_ctx->color_material_face = face;
    fe_ctx->color_material_mode = mode;
}

void glShadeModel(GLenum mode)
{
    CHECK_CTX();
    if (fe_rec_e(LC_SHADE_MODEL, mode)) return;
    if (mode != GL_FLAT && mode != GL_SMOOTH && mode != GL_PHONG) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_state_changed(fe_ctx);
    fe_ctx->shade_model = mode;
}

/* ---- state snapshots handed to the back end ---- */

/* Light fields compute_lighting derives per vertex (lighting.h:306-334), derived once here
 * with the same float operations. */
static void derive_lighting(const GLState *c, mtgl_lighting *out)
{
    *out = c->lit;
    out->normalize = (c->flags & F_NORMALIZE) ? 1u : 0u;
    for (int i = 0; i < FE_MAX_LIGHTS; i++) {
        mtgl_light *l = &out->lights[i];
        fe_vec3_normalize(l->position, l->dir_normalized);
        fe_vec3_normalize(l->spot_direction, l->spot_dir_normalized);
        l->cos_cutoff = cosf(l->spot_cutoff * 3.14159265f / 180.0f);
    }
}

/* mat4_normal_matrix (graphics.h:229-260) */
static void normal_matrix(const float *m, float *r)
{
    float a = m[0], b = m[1], c = m[2];
    float d = m[4], e = m[5], f = m[6];
    float g = m[8], h = m[9], i = m[10];
    float det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
    if (fabsf(det) < 1e-10f) {
        fe_mat4_identity(r);
        return;
    }
    float inv_det = 1.0f / det;
    for (int k = 0; k < 16; k++) r[k] = 0.0f;
    r[0] = (e * i - f * h) * inv_det;
    r[1] = (d * i - f * g) * -inv_det;
    r[2] = (d * h - e * g) * inv_det;
    r[4] = (b * i - c * h) * -inv_det;
    r[5] = (a * i - c * g) * inv_det;
    r[6] = (a * h - b * g) * -inv_det;
    r[8] = (b * f - c * e) * inv_det;
    r[9] = (a * f - c * d) * -inv_det;
    r[10] = (a * e - b * d) * inv_det;
    r[15] = 1.0f;
}

void fe_snapshot_vertex(GLState *c, mtgl_vertex_state *vs)
{
    memset(vs, 0, sizeof(*vs));
    memcpy(vs->modelview, c->mv[c->mv_depth], sizeof(vs->modelview));
    memcpy(vs->projection, c->proj[c->proj_depth], sizeof(vs->projection));
    memcpy(vs->texture, c->texm[c->tex_depth], sizeof(vs->texture));
    normal_matrix(vs->modelview, vs->normal_matrix);
    vs->lighting = (c->flags & F_LIGHTING) ? 1u : 0u;
    vs->color_material = (c->flags & F_COLOR_MATERIAL) ? 1u : 0u;
    vs->color_material_face = c->color_material_face;
    vs->color_material_mode = c->color_material_mode;
    vs->phong = (c->shade_model == GL_PHONG) ? 1u : 0u;
    derive_lighting(c, &vs->lit);
}

void fe_snapshot_raster(GLState *c, mtgl_raster_state *rs)
{
    memset(rs, 0, sizeof(*rs));
    memcpy(rs->viewport, c->viewport, sizeof(rs->viewport));
    memcpy(rs->scissor, c->scissor, sizeof(rs->scissor));
    rs->scissor_test = (c->flags & F_SCISSOR_TEST) ? 1u : 0u;
    rs->depth_test = (c->flags & F_DEPTH_TEST) ? 1u : 0u;
    rs->depth_func = c->depth_func;
    rs->depth_mask = c->depth_mask ? 1u : 0u;
    rs->depth_near = c->depth_near;
    rs->depth_far = c->depth_far;
    rs->stencil_test = (c->flags & F_STENCIL_TEST) ? 1u : 0u;
    rs->stencil_func = c->stencil_func;
    rs->stencil_ref = c->stencil_ref;
    rs->stencil_mask = c->stencil_mask;
    rs->stencil_fail = c->stencil_fail;
    rs->stencil_zfail = c->stencil_zfail;
    rs->stencil_zpass = c->stencil_zpass;
    rs->stencil_writemask = c->stencil_writemask;
    rs->blend = (c->flags & F_BLEND) ? 1u : 0u;
    rs->blend_src = c->blend_src;
    rs->blend_dst = c->blend_dst;
    rs->alpha_test = (c->flags & F_ALPHA_TEST) ? 1u : 0u;
    rs->alpha_func = c->alpha_func;
    rs->alpha_ref = c->alpha_ref;
    for (int i = 0; i < 4; i++) rs->color_mask[i] = c->color_mask[i] ? 1u : 0u;
    rs->cull_face = (c->flags & F_CULL_FACE) ? 1u : 0u;
    rs->cull_face_mode = c->cull_mode;
    rs->front_face = c->front_face;
    rs->polygon_mode_front = c->poly_front;
    rs->polygon_mode_back = c->poly_back;
    rs->shade_model = c->shade_model;
    rs->perspective_hint = c->persp_hint;
    rs->fog = (c->flags & F_FOG) ? 1u : 0u;
    rs->fog_mode = c->fog_mode;
    rs->fog_density = c->fog_density;
    rs->fog_start = c->fog_start;
    rs->fog_end = c->fog_end;
    memcpy(rs->fog_color, c->fog_color, sizeof(rs->fog_color));
    rs->tex_env_mode = c->tex_env_mode;
    memcpy(rs->tex_env_color, c->tex_env_color, sizeof(rs->tex_env_color));
    rs->texture = 0;
    if ((c->flags & F_TEXTURE_2D) && c->bound_texture != 0) {
        /* the texture's parameters are read at raster time (raster.c:495-498) */
        fe_texture *t = fe_texture_get(c, c->bound_texture);
        if (t && t->has_image) {
            rs->texture = t->dev;
            rs->tex_min_filter = t->min_filter;
            rs->tex_mag_filter = t->mag_filter;
            rs->tex_wrap_s = t->wrap_s;
            rs->tex_wrap_t = t->wrap_t;
        }
    }
    rs->line_width = c->line_width;
    rs->point_size = c->point_size;
    rs->lighting = (c->flags & F_LIGHTING) ? 1u : 0u;
    derive_lighting(c, &rs->lit);
}
