/*
 * fe_draw.c — vertex specification, vertex arrays and draw calls, raster position and
 * pixel transfer (gl_api.c:614-752, 1180-1424, 1717-1941).
 *
 * glEnd no longer rasterises: it hands the batch to the back end as one draw packet. A
 * glDrawArrays / glDrawElements call becomes one packet whose attribute streams point at
 * client memory or at device-resident buffer objects; the vertex kernel then performs the
 * conversions get_array_element and glColor4f perform per element in the reference.
 * Cases where the reference's per-element replay has observable side effects beyond
 * a plain draw (display-list compilation, a glBegin still open, vertices left over from
 * outside glBegin/glEnd, an invalid mode) take the replay path verbatim.
 */
#include "fe_internal.h"

/* ---- immediate-mode batch ---- */

static void push_vertex_state(GLState *c)
{
    mtgl_vertex_state vs;
    fe_snapshot_vertex(c, &vs);
    c->vs_dirty = 0;
    if (c->vs_count > 0 && memcmp(&c->vstates[c->vs_count - 1], &vs, sizeof(vs)) == 0) return;
    if (c->vs_count == c->vs_cap) {
        uint32_t cap = c->vs_cap ? c->vs_cap * 2 : 4;
        mtgl_vertex_state *n = (mtgl_vertex_state *)realloc(c->vstates, cap * sizeof(*n));
        if (!n) {
            fe_set_error(c, GL_OUT_OF_MEMORY);
            return;
        }
        c->vstates = n;
        c->vs_cap = cap;
    }
    c->vstates[c->vs_count++] = vs;
}

/* color_clamp of the current colour written into the material (gl_api.c:285-312) */
static void apply_color_material(GLState *c, const float *color)
{
    float cl[4];
    for (int i = 0; i < 4; i++) cl[i] = color[i] < 0 ? 0 : (color[i] > 1 ? 1 : color[i]);
    GLenum mode = c->color_material_mode, face = c->color_material_face;
    mtgl_material *mats[2] = {NULL, NULL};
    if (face == GL_FRONT || face == GL_FRONT_AND_BACK) mats[0] = &c->lit.front;
    if (face == GL_BACK || face == GL_FRONT_AND_BACK) mats[1] = &c->lit.back;
    for (int k = 0; k < 2; k++) {
        mtgl_material *m = mats[k];
        if (!m) continue;
        if (mode == GL_AMBIENT || mode == GL_AMBIENT_AND_DIFFUSE) memcpy(m->ambient, cl, sizeof(cl));
        if (mode == GL_DIFFUSE || mode == GL_AMBIENT_AND_DIFFUSE) memcpy(m->diffuse, cl, sizeof(cl));
        if (mode == GL_SPECULAR) memcpy(m->specular, cl, sizeof(cl));
        if (mode == GL_EMISSION) memcpy(m->emission, cl, sizeof(cl));
    }
}

/* emit_vertex (gl_api.c:263-348), host half: capture the vertex; the device transforms it */
static void emit_vertex(float x, float y, float z)
{
    GLState *c = fe_ctx;
    if (c->vs_dirty || c->vs_count == 0) push_vertex_state(c);
    if (c->vs_count == 0) return;
    if ((c->flags & F_LIGHTING) && (c->flags & F_COLOR_MATERIAL)) apply_color_material(c, c->cur_color);
    if (c->imm_count == c->imm_cap) {
        size_t cap = c->imm_cap ? c->imm_cap * 2 : 64;
        fe_vertex *nv = (fe_vertex *)realloc(c->imm, cap * sizeof(fe_vertex));
        if (!nv) {
            fe_set_error(c, GL_OUT_OF_MEMORY);
            return;
        }
        c->imm = nv;
        uint32_t *ns = (uint32_t *)realloc(c->imm_vs, cap * sizeof(uint32_t));
        if (!ns) {
            fe_set_error(c, GL_OUT_OF_MEMORY);
            return;
        }
        c->imm_vs = ns;
        c->imm_cap = cap;
    }
    fe_vertex *v = &c->imm[c->imm_count];
    v->pos[0] = x; v->pos[1] = y; v->pos[2] = z;
    memcpy(v->color, c->cur_color, sizeof(v->color));
    memcpy(v->tex, c->cur_tex, sizeof(v->tex));
    memcpy(v->normal, c->cur_normal, sizeof(v->normal));
    c->imm_vs[c->imm_count] = c->vs_count - 1;
    c->imm_count++;
}

static void host_attrib(mtgl_attrib *a, const void *p, int size)
{
    memset(a, 0, sizeof(*a));
    a->host = p;
    a->size = size;
    a->type = GL_FLOAT;
    a->stride = (int32_t)sizeof(fe_vertex);
    a->enabled = 1;
}

/* flush_* dispatch of glEnd (gl_api.c:648-659): one packet for the whole batch */
void fe_flush_immediate(GLState *c)
{
    if (c->imm_count > 0 && c->vs_count > 0) {
        mtgl_raster_state rs;
        fe_snapshot_raster(c, &rs);
        mtgl_draw d;
        memset(&d, 0, sizeof(d));
        d.mode = c->prim_mode;
        d.first = 0;
        d.count = (int32_t)c->imm_count;
        d.index_min = 0;
        d.index_max = (int64_t)c->imm_count - 1;
        host_attrib(&d.position, c->imm[0].pos, 3);
        host_attrib(&d.color, c->imm[0].color, 4);
        host_attrib(&d.texcoord, c->imm[0].tex, 2);
        host_attrib(&d.normal, c->imm[0].normal, 3);
        memcpy(d.current_color, c->cur_color, sizeof(d.current_color));
        memcpy(d.current_texcoord, c->cur_tex, sizeof(d.current_texcoord));
        memcpy(d.current_normal, c->cur_normal, sizeof(d.current_normal));
        d.vertex_state_ids = c->imm_vs;
        d.vertex_states = c->vstates;
        d.vertex_state_count = c->vs_count;
        d.raster_state = &rs;
        fe_dev_error(c, mtgl_dev_draw(c->dev, &d));
    }
    c->imm_count = 0;
    c->vs_count = 0;
    c->vs_dirty = 1;
}

static void buffer_attrib(mtgl_attrib *a, mtgl_handle vb, uint64_t offset, uint64_t buffer_bytes, int size)
{
    memset(a, 0, sizeof(*a));
    a->buffer = vb;
    a->offset = offset;
    a->bytes = buffer_bytes - offset;
    a->size = size;
    a->type = GL_FLOAT;
    a->stride = (int32_t)sizeof(fe_vertex);
    a->enabled = 1;
}

/* glCallList of a device-resident block (fe_lists.c): what glBegin, the block's commands
 * and glEnd do through the immediate path, with the vertices read from the list's device
 * buffer. The packet glEnd would submit has one vertex state (the block changes no state
 * that the snapshot holds, and the snapshot is taken, as at the first emit_vertex, before
 * GL_COLOR_MATERIAL rewrites the material); an attribute the block never sets comes from
 * the current value, which every vertex would have copied. Afterwards the current
 * attributes hold the block's last values, and GL_COLOR_MATERIAL under lighting leaves the
 * last vertex's colour in the material (emit_vertex, gl_api.c:263-348). Returns 0, having
 * done nothing, when the replay must go through the public entry points instead (a list
 * being compiled, a glBegin still open, vertices emitted outside glBegin/glEnd pending). */
int fe_draw_list_block(GLState *c, mtgl_handle vb, const fe_list_block *b)
{
    if ((c->flags & F_INSIDE_BEGIN_END) || c->list_index != 0 || c->imm_count != 0) return 0;
    if (b->set & CL_COLOR) memcpy(c->cur_color, b->color, sizeof(c->cur_color));
    if (b->set & CL_TEXCOORD) memcpy(c->cur_tex, b->tex, sizeof(c->cur_tex));
    if (b->set & CL_NORMAL) memcpy(c->cur_normal, b->normal, sizeof(c->cur_normal));
    c->prim_mode = b->mode;

    const uint64_t base = (uint64_t)b->first * sizeof(fe_vertex);
    const uint64_t bytes = base + (uint64_t)b->count * sizeof(fe_vertex);
    mtgl_draw d;
    memset(&d, 0, sizeof(d));
    d.mode = b->mode;
    d.count = (int32_t)b->count;
    d.index_max = (int64_t)b->count - 1;
    buffer_attrib(&d.position, vb, base + offsetof(fe_vertex, pos), bytes, 3);
    if (b->set & CL_COLOR) buffer_attrib(&d.color, vb, base + offsetof(fe_vertex, color), bytes, 4);
    if (b->set & CL_TEXCOORD) buffer_attrib(&d.texcoord, vb, base + offsetof(fe_vertex, tex), bytes, 2);
    if (b->set & CL_NORMAL) buffer_attrib(&d.normal, vb, base + offsetof(fe_vertex, normal), bytes, 3);
    memcpy(d.current_color, c->cur_color, sizeof(d.current_color));
    memcpy(d.current_texcoord, c->cur_tex, sizeof(d.current_texcoord));
    memcpy(d.current_normal, c->cur_normal, sizeof(d.current_normal));
    mtgl_vertex_state vs;
    mtgl_raster_state rs;
    fe_snapshot_vertex(c, &vs);
    fe_snapshot_raster(c, &rs);
    d.vertex_states = &vs;
    d.vertex_state_count = 1;
    d.raster_state = &rs;
    fe_dev_error(c, mtgl_dev_draw(c->dev, &d));
    if ((c->flags & F_LIGHTING) && (c->flags & F_COLOR_MATERIAL))
        apply_color_material(c, (b->set & CL_COLOR) ? b->last_color : c->cur_color);
    c->imm_count = 0;
    c->vs_count = 0;
    c->vs_dirty = 1;
    return 1;
}

void glBegin(GLenum mode)
{
    CHECK_CTX();
    if (fe_rec_e(LC_BEGIN, mode)) return;
    if (fe_ctx->flags & F_INSIDE_BEGIN_END) {
        fe_set_error(fe_ctx, GL_INVALID_OPERATION);
        return;
    }
    if (mode > GL_POLYGON) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_ctx->prim_mode = mode;
    fe_ctx->flags |= F_INSIDE_BEGIN_END;
}

void glEnd(void)
{
    CHECK_CTX();
    if (fe_rec_op(LC_END)) return;
    if (!(fe_ctx->flags & F_INSIDE_BEGIN_END)) {
        fe_set_error(fe_ctx, GL_INVALID_OPERATION);
        return;
    }
    fe_ctx->flags &= ~F_INSIDE_BEGIN_END;
    fe_flush_immediate(fe_ctx);
}

void glVertex3f(GLfloat x, GLfloat y, GLfloat z)
{
    CHECK_CTX();
    if (fe_rec_f3(LC_VERTEX, x, y, z)) return;
    emit_vertex(x, y, z);
}

void glVertex2f(GLfloat x, GLfloat y)
{
    CHECK_CTX();
    if (fe_rec_f3(LC_VERTEX, x, y, 0.0f)) return;
    emit_vertex(x, y, 0.0f);
}

void glVertex2i(GLint x, GLint y) { glVertex2f((float)x, (float)y); }
void glVertex3i(GLint x, GLint y, GLint z) { glVertex3f((float)x, (float)y, (float)z); }

static int finite_f(float f) { return !isnan(f) && !isinf(f); }

/* glColor4f (gl_api.c:711-723): NaN/Inf -> 0 (alpha -> 1), then clamp to [0,1] */
static void sanitize_color(float *c)
{
    for (int i = 0; i < 4; i++) {
        if (!finite_f(c[i])) c[i] = (i == 3) ? 1.0f : 0.0f;
        if (c[i] < 0.0f) c[i] = 0.0f; else if (c[i] > 1.0f) c[i] = 1.0f;
    }
}

static void set_color(float r, float g, float b, float a)
{
    fe_list_cmd cmd = {LC_COLOR, {0, 0, 0}, 0, {r, g, b, a}, {0}};
    if (fe_rec(&cmd)) return;
    fe_ctx->cur_color[0] = r; fe_ctx->cur_color[1] = g;
    fe_ctx->cur_color[2] = b; fe_ctx->cur_color[3] = a;
}

void glColor3f(GLfloat r, GLfloat g, GLfloat b)
{
    CHECK_CTX();
    float c[4] = {r, g, b, 1.0f};
    sanitize_color(c);
    set_color(c[0], c[1], c[2], 1.0f);
}

void glColor4f(GLfloat r, GLfloat g, GLfloat b, GLfloat a)
{
    CHECK_CTX();
    float c[4] = {r, g, b, a};
    sanitize_color(c);
    set_color(c[0], c[1], c[2], c[3]);
}

void glColor3ub(GLubyte r, GLubyte g, GLubyte b)
{
    CHECK_CTX();
    set_color(r / 255.0f, g / 255.0f, b / 255.0f, 1.0f);
}

void glColor4ub(GLubyte r, GLubyte g, GLubyte b, GLubyte a)
{
    CHECK_CTX();
    set_color(r / 255.0f, g / 255.0f, b / 255.0f, a / 255.0f);
}

void glTexCoord2f(GLfloat s, GLfloat t)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_TEXCOORD, {0, 0, 0}, 0, {s, t}, {0}};
    if (fe_rec(&cmd)) return;
    fe_ctx->cur_tex[0] = s;
    fe_ctx->cur_tex[1] = t;
}

void glNormal3f(GLfloat x, GLfloat y, GLfloat z)
{
    CHECK_CTX();
    if (fe_rec_f3(LC_NORMAL, x, y, z)) return;
    fe_ctx->cur_normal[0] = x; fe_ctx->cur_normal[1] = y; fe_ctx->cur_normal[2] = z;
}

/* ---- vertex arrays (gl_api.c:1612-1741) ---- */

static void client_state(GLenum array, int on)
{
    uint32_t bit;
    switch (array) {
    case GL_VERTEX_ARRAY: bit = CL_VERTEX; break;
    case GL_COLOR_ARRAY: bit = CL_COLOR; break;
    case GL_TEXTURE_COORD_ARRAY: bit = CL_TEXCOORD; break;
    case GL_NORMAL_ARRAY: bit = CL_NORMAL; break;
    default: fe_set_error(fe_ctx, GL_INVALID_ENUM); return;
    }
    if (on) fe_ctx->client_state |= bit; else fe_ctx->client_state &= ~bit;
}

void glEnableClientState(GLenum a) { CHECK_CTX(); client_state(a, 1); }
void glDisableClientState(GLenum a) { CHECK_CTX(); client_state(a, 0); }

static void set_pointer(fe_array *arr, GLint size, GLenum type, GLsizei stride, const GLvoid *p, GLint lo, GLint hi)
{
    if (size < lo || size > hi) {
        fe_set_error(fe_ctx, GL_INVALID_VALUE);
        return;
    }
    if (type != GL_FLOAT && type != GL_UNSIGNED_BYTE) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    if (stride < 0) {
        fe_set_error(fe_ctx, GL_INVALID_VALUE);
        return;
    }
    arr->size = size;
    arr->type = type;
    arr->stride = stride;
    arr->pointer = p;
}

void glVertexPointer(GLint size, GLenum type, GLsizei stride, const GLvoid *p)
{
    CHECK_CTX();
    set_pointer(&fe_ctx->vp, size, type, stride, p, 2, 4);
}

void glColorPointer(GLint size, GLenum type, GLsizei stride, const GLvoid *p)
{
    CHECK_CTX();
    set_pointer(&fe_ctx->cp, size, type, stride, p, 3, 4);
}

void glTexCoordPointer(GLint size, GLenum type, GLsizei stride, const GLvoid *p)
{
    CHECK_CTX();
    set_pointer(&fe_ctx->tp, size, type, stride, p, 1, 4);
}

void glNormalPointer(GLenum type, GLsizei stride, const GLvoid *p)
{
    CHECK_CTX();
    if (type != GL_FLOAT && type != GL_UNSIGNED_BYTE) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    if (stride < 0) {
        fe_set_error(fe_ctx, GL_INVALID_VALUE);
        return;
    }
    fe_ctx->np.size = 3;
    fe_ctx->np.type = type;
    fe_ctx->np.stride = stride;
    fe_ctx->np.pointer = p;
}

/* get_array_pointer (gl_api.c:1745-1755): with an array buffer bound at draw time every
 * pointer is an offset into it. Returns the host view (shadow copy for buffers). */
static const void *array_base(GLState *c, const fe_array *a, fe_buffer **buf_out)
{
    *buf_out = NULL;
    if (c->bound_array_buffer) {
        fe_buffer *b = fe_buffer_get(c, c->bound_array_buffer);
        if (b && b->shadow) {
            *buf_out = b;
            return b->shadow + (size_t)a->pointer;
        }
        return NULL;
    }
    return a->pointer;
}

static int32_t eff_stride(const fe_array *a)
{
    if (a->stride != 0) return a->stride;
    return a->size * (a->type == GL_FLOAT ? (int32_t)sizeof(GLfloat) : 1);
}

/* get_array_element (gl_api.c:1758-1797) */
static void get_element(const fe_array *a, const void *base, GLint index, float *out, int n)
{
    if (!base || index < 0) {
        for (int i = 0; i < n; i++) out[i] = (i < 3) ? 0.0f : 1.0f;
        return;
    }
    int32_t stride = eff_stride(a);
    if (stride <= 0) {
        for (int i = 0; i < n; i++) out[i] = (i < 3) ? 0.0f : 1.0f;
        return;
    }
    const uint8_t *p = (const uint8_t *)base + (size_t)index * (size_t)stride;
    for (int i = 0; i < a->size && i < n; i++) {
        if (a->type == GL_FLOAT) {
            float v;
            memcpy(&v, p + 4 * i, 4);
            out[i] = v;
        } else {
            out[i] = p[i] / 255.0f;
        }
    }
    for (int i = a->size; i < n; i++) out[i] = (i == 3) ? 1.0f : 0.0f;
}

typedef struct {
    const void *vbase, *cbase, *tbase, *nbase;
    fe_buffer *vbuf, *cbuf, *tbuf, *nbuf;
} array_bases;

static void resolve_bases(GLState *c, array_bases *b)
{
    memset(b, 0, sizeof(*b));
    b->vbase = array_base(c, &c->vp, &b->vbuf);
    if (c->client_state & CL_COLOR) b->cbase = array_base(c, &c->cp, &b->cbuf);
    if (c->client_state & CL_TEXCOORD) b->tbase = array_base(c, &c->tp, &b->tbuf);
    if (c->client_state & CL_NORMAL) b->nbase = array_base(c, &c->np, &b->nbuf);
}

/* The reference's per-element replay through the public entry points (gl_api.c:1818-1851) */
static void replay_element(GLState *c, const array_bases *b, GLint idx)
{
    float v[4], col[4], t[2], n[3];
    get_element(&c->vp, b->vbase, idx, v, 4);
    if (b->cbase) {
        get_element(&c->cp, b->cbase, idx, col, 4);
        glColor4f(col[0], col[1], col[2], col[3]);
    }
    if (b->tbase) {
        get_element(&c->tp, b->tbase, idx, t, 2);
        glTexCoord2f(t[0], t[1]);
    }
    if (b->nbase) {
        get_element(&c->np, b->nbase, idx, n, 3);
        glNormal3f(n[0], n[1], n[2]);
    }
    if (c->vp.size == 2) glVertex2f(v[0], v[1]);
    else glVertex3f(v[0], v[1], v[2]);
}

static void make_attrib(const fe_array *a, const void *base, fe_buffer *buf, mtgl_attrib *out)
{
    memset(out, 0, sizeof(*out));
    if (!base) return;
    out->size = a->size;
    out->type = (int32_t)a->type;
    out->stride = eff_stride(a);
    out->enabled = 1;
    if (buf) {
        out->buffer = buf->dev;
        out->offset = (uint64_t)(size_t)a->pointer;
        out->bytes = (uint64_t)buf->size > out->offset ? (uint64_t)buf->size - out->offset : 0;
    } else {
        out->host = base;
    }
}

/* The host-visible effects of the per-element replay that outlive the draw: the current
 * attributes take the last element's values, and GL_COLOR_MATERIAL leaves the last
 * colour in the material (gl_api.c:285-312, 694-752). */
static void apply_last_element(GLState *c, const array_bases *b, GLint idx)
{
    float col[4], t[2], n[3];
    if (b->cbase) {
        get_element(&c->cp, b->cbase, idx, col, 4);
        sanitize_color(col);
        memcpy(c->cur_color, col, sizeof(col));
    }
    if (b->tbase) {
        get_element(&c->tp, b->tbase, idx, t, 2);
        c->cur_tex[0] = t[0];
        c->cur_tex[1] = t[1];
    }
    if (b->nbase) {
        get_element(&c->np, b->nbase, idx, n, 3);
        memcpy(c->cur_normal, n, sizeof(n));
    }
    if ((c->flags & F_LIGHTING) && (c->flags & F_COLOR_MATERIAL)) apply_color_material(c, c->cur_color);
}

static int fast_path_ok(GLState *c, GLenum mode)
{
    return mode <= GL_POLYGON && !(c->flags & F_INSIDE_BEGIN_END) && c->list_index == 0 && c->imm_count == 0;
}

static void submit_array_draw(GLState *c, mtgl_draw *d, const array_bases *b)
{
    make_attrib(&c->vp, b->vbase, b->vbuf, &d->position);
    make_attrib(&c->cp, b->cbase, b->cbuf, &d->color);
    make_attrib(&c->tp, b->tbase, b->tbuf, &d->texcoord);
    make_attrib(&c->np, b->nbase, b->nbuf, &d->normal);
    d->position_2d = (c->vp.size == 2);
    memcpy(d->current_color, c->cur_color, sizeof(d->current_color));
    memcpy(d->current_texcoord, c->cur_tex, sizeof(d->current_texcoord));
    memcpy(d->current_normal, c->cur_normal, sizeof(d->current_normal));
    mtgl_vertex_state vs;
    mtgl_raster_state rs;
    fe_snapshot_vertex(c, &vs);
    fe_snapshot_raster(c, &rs);
    d->vertex_states = &vs;
    d->vertex_state_count = 1;
    d->vertex_state_ids = NULL;
    d->raster_state = &rs;
    fe_dev_error(c, mtgl_dev_draw(c->dev, d));
}

void glDrawArrays(GLenum mode, GLint first, GLsizei count)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (count < 0) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    array_bases b;
    resolve_bases(c, &b);
    if (!(c->client_state & CL_VERTEX) || !b.vbase) return;

    if (!fast_path_ok(c, mode)) {
        glBegin(mode);
        for (GLsizei i = 0; i < count; i++) replay_element(c, &b, first + i);
        glEnd();
        return;
    }
    if (count == 0) return;
    mtgl_draw d;
    memset(&d, 0, sizeof(d));
    d.mode = mode;
    d.first = first;
    d.count = count;
    d.index_type = 0;
    int64_t lo = first, hi = (int64_t)first + count - 1;
    d.has_negative_index = lo < 0;
    d.index_min = lo < 0 ? 0 : lo;
    d.index_max = hi;
    submit_array_draw(c, &d, &b);
    apply_last_element(c, &b, (GLint)(first + count - 1));
}

static GLuint read_index(const void *data, GLenum type, GLsizei i)
{
    if (type == GL_UNSIGNED_SHORT) { GLushort v; memcpy(&v, (const uint8_t *)data + 2 * (size_t)i, 2); return v; }
    if (type == GL_UNSIGNED_INT) { GLuint v; memcpy(&v, (const uint8_t *)data + 4 * (size_t)i, 4); return v; }
    return ((const GLubyte *)data)[i];
}

/* non-negative (as GLint) index range of an index list */
static void scan_indices(const void *data, GLenum type, GLsizei count, int64_t *mn, int64_t *mx, int *neg)
{
    int64_t lo = INT64_MAX, hi = -1;
    int has_neg = 0;
    for (GLsizei i = 0; i < count; i++) {
        GLint v = (GLint)read_index(data, type, i);
        if (v < 0) { has_neg = 1; continue; }
        if (v < lo) lo = v;
        if (v > hi) hi = v;
    }
    if (hi < 0) { lo = 0; hi = -1; }
    *mn = lo; *mx = hi; *neg = has_neg;
}

void glDrawElements(GLenum mode, GLsizei count, GLenum type, const GLvoid *indices)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (count < 0) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    if (type != GL_UNSIGNED_BYTE && type != GL_UNSIGNED_SHORT && type != GL_UNSIGNED_INT) {
        fe_set_error(c, GL_INVALID_ENUM);
        return;
    }
    array_bases b;
    resolve_bases(c, &b);
    const void *index_data = indices;
    fe_buffer *ibuf = NULL;
    uint64_t ioff = 0;
    if (c->bound_element_buffer) {
        ibuf = fe_buffer_get(c, c->bound_element_buffer);
        if (ibuf && ibuf->shadow) {
            ioff = (uint64_t)(uintptr_t)indices;
            if (ioff >= (uint64_t)ibuf->size) {
                fe_set_error(c, GL_INVALID_VALUE);
                return;
            }
            index_data = ibuf->shadow + ioff;
        } else {
            return;
        }
    }
    if (!(c->client_state & CL_VERTEX) || !b.vbase || !index_data) return;
    int isz = type == GL_UNSIGNED_INT ? 4 : (type == GL_UNSIGNED_SHORT ? 2 : 1);
    if (ibuf && (uint64_t)count * isz > (uint64_t)ibuf->size - ioff) {
        /* the reference reads past the end of the element buffer here (undefined
         * behaviour); this implementation draws only the indices the buffer holds */
        count = (GLsizei)(((uint64_t)ibuf->size - ioff) / isz);
    }

    if (!fast_path_ok(c, mode)) {
        glBegin(mode);
        for (GLsizei i = 0; i < count; i++) replay_element(c, &b, (GLint)read_index(index_data, type, i));
        glEnd();
        return;
    }
    if (count == 0) return;
    mtgl_draw d;
    memset(&d, 0, sizeof(d));
    d.mode = mode;
    d.first = 0;
    d.count = count;
    d.index_type = type;
    int64_t mn, mx;
    int neg;
    if (ibuf) {
        d.index_buffer = ibuf->dev;
        d.index_offset = ioff;
        fe_buffer_index_range(ibuf, ioff, count, type, &mn, &mx, &neg);
    } else {
        d.index_host = index_data;
        scan_indices(index_data, type, count, &mn, &mx, &neg);
    }
    d.index_min = mn;
    d.index_max = mx;
    d.has_negative_index = neg;
    submit_array_draw(c, &d, &b);
    apply_last_element(c, &b, (GLint)read_index(index_data, type, count - 1));
}

void fe_scan_indices(const void *data, GLenum type, GLsizei count, int64_t *mn, int64_t *mx, int *neg)
{
    scan_indices(data, type, count, mn, mx, neg);
}

/* ---- raster position (gl_api.c:1378-1424) ---- */

/* ndc_to_screen (raster.c:59-63) */
static void ndc_to_screen(GLState *c, float x, float y, int32_t *sx, int32_t *sy)
{
    *sx = fe_f2i((x + 1.0f) * 0.5f * (float)c->viewport[2] + (float)c->viewport[0]);
    *sy = fe_f2i((1.0f - y) * 0.5f * (float)c->viewport[3] + (float)c->viewport[1]);
}

static void raster_pos(float x, float y, float z)
{
    GLState *c = fe_ctx;
    float v[4] = {x, y, z, 1.0f}, e[4], clip[4];
    fe_mat4_mul_vec4(c->mv[c->mv_depth], v, e);
    fe_mat4_mul_vec4(c->proj[c->proj_depth], e, clip);
    if (clip[3] <= 0.0f) {
        c->raster_valid = GL_FALSE;
        return;
    }
    float nx = clip[0] / clip[3];
    float ny = clip[1] / clip[3];
    int32_t sx, sy;
    ndc_to_screen(c, nx, ny, &sx, &sy);
    c->raster_x = sx;
    /* two's-complement wrap as on the reference's x86-64 build when sy is INT32_MIN */
    c->raster_y = (GLint)((uint32_t)(c->height - 1) - (uint32_t)sy);
    c->raster_valid = GL_TRUE;
}

void glRasterPos2i(GLint x, GLint y) { CHECK_CTX(); raster_pos((float)x, (float)y, 0.0f); }
void glRasterPos2f(GLfloat x, GLfloat y) { CHECK_CTX(); raster_pos(x, y, 0.0f); }
void glRasterPos3f(GLfloat x, GLfloat y, GLfloat z) { CHECK_CTX(); raster_pos(x, y, z); }

/* ---- pixel transfer ---- */

/* glDrawPixels (gl_api.c:1287-1376): formats are packed on the host, the blit (alpha
 * test, depth test at depth 0, blend, depth write) runs on the device in order. */
void glDrawPixels(GLsizei width, GLsizei height, GLenum format, GLenum type, const GLvoid *pixels)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (type != GL_UNSIGNED_BYTE || !pixels || !c->raster_valid) return;
    if (format != GL_RGBA && format != GL_RGB && format != GL_LUMINANCE && format != GL_LUMINANCE_ALPHA) return;
    if (width <= 0 || height <= 0) return;
    size_t n = (size_t)width * (size_t)height;
    uint32_t *packed = (uint32_t *)malloc(n * sizeof(uint32_t));
    if (!packed) {
        fe_set_error(c, GL_OUT_OF_MEMORY);
        return;
    }
    const uint8_t *s = (const uint8_t *)pixels;
    for (size_t i = 0; i < n; i++) {
        uint32_t r, g, b, a = 255;
        if (format == GL_RGBA) { r = s[4 * i]; g = s[4 * i + 1]; b = s[4 * i + 2]; a = s[4 * i + 3]; }
        else if (format == GL_RGB) { r = s[3 * i]; g = s[3 * i + 1]; b = s[3 * i + 2]; }
        else if (format == GL_LUMINANCE) { r = g = b = s[i]; }
        else { r = g = b = s[2 * i]; a = s[2 * i + 1]; }
        packed[i] = (a << 24) | (b << 16) | (g << 8) | r;
    }
    mtgl_raster_state rs;
    fe_snapshot_raster(c, &rs);
    fe_dev_error(c, mtgl_dev_draw_pixels(c->dev, c->raster_x, c->raster_y, width, height, packed, &rs));
    free(packed);
}

/* glReadPixels (gl_api.c:1180-1230): synchronises, then converts on the host */
void glReadPixels(GLint x, GLint y, GLsizei width, GLsizei height, GLenum format, GLenum type, GLvoid *pixels)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (type != GL_UNSIGNED_BYTE || !pixels || width < 0 || height < 0) return;
    const uint32_t *fb = mtgl_color_buffer(c);
    if (!fb) {
        fe_set_error(c, GL_OUT_OF_MEMORY);
        return;
    }
    uint8_t *dst = (uint8_t *)pixels;
    for (GLsizei row = 0; row < height; row++) {
        GLint fb_y = c->height - 1 - (y + row);
        if (fb_y < 0 || fb_y >= c->height) {
            if (format == GL_RGBA) memset(dst + (size_t)row * width * 4, 0, (size_t)width * 4);
            else if (format == GL_RGB) memset(dst + (size_t)row * width * 3, 0, (size_t)width * 3);
            continue;
        }
        for (GLsizei col = 0; col < width; col++) {
            GLint sx = x + col;
            uint8_t r = 0, g = 0, b = 0, a = 255;
            if (sx >= 0 && sx < c->width) {
                uint32_t p = fb[(size_t)fb_y * c->width + sx];
                r = p & 0xFF; g = (p >> 8) & 0xFF; b = (p >> 16) & 0xFF; a = (p >> 24) & 0xFF;
            }
            if (format == GL_RGBA) {
                size_t i = ((size_t)row * width + col) * 4;
                dst[i] = r; dst[i + 1] = g; dst[i + 2] = b; dst[i + 3] = a;
            } else if (format == GL_RGB) {
                size_t i = ((size_t)row * width + col) * 3;
                dst[i] = r; dst[i + 1] = g; dst[i + 2] = b;
            }
        }
    }
}
