/*
 * fe_objects.c — texture and buffer objects (gl_api.c:756-885, 1516-1610; textures.c:13-269;
 * vbo.c:12-161).
 *
 * Ids are 1-based, deleted slots are reused first, and the tables cap at 256 entries, as
 * in the reference. Texel and vertex storage lives on the device; buffers keep a host
 * shadow copy because glDrawElements needs index ranges and the last element's attributes
 * on the host.
 */
#include "fe_internal.h"

/* ---- textures ---- */

fe_texture *fe_texture_get(GLState *c, GLuint id)
{
    if (id == 0 || id > c->tex_count) return NULL;
    fe_texture *t = &c->textures[id - 1];
    return t->allocated ? t : NULL;
}

static void texture_init_slot(fe_texture *t)
{
    mtgl_handle keep = t->dev;
    memset(t, 0, sizeof(*t));
    t->dev = keep;
    t->min_filter = GL_NEAREST;
    t->mag_filter = GL_NEAREST;
    t->wrap_s = GL_REPEAT;
    t->wrap_t = GL_REPEAT;
    t->allocated = 1;
}

/* texture_alloc (textures.c:58-95) */
static GLuint texture_alloc(GLState *c)
{
    for (size_t i = 0; i < c->tex_count; i++) {
        if (!c->textures[i].allocated) {
            texture_init_slot(&c->textures[i]);
            return (GLuint)(i + 1);
        }
    }
    if (c->tex_count >= FE_MAX_TEXTURES) return 0;
    if (c->tex_count == c->tex_cap) {
        size_t cap = c->tex_cap ? c->tex_cap * 2 : 16;
        if (cap > FE_MAX_TEXTURES) cap = FE_MAX_TEXTURES;
        fe_texture *n = (fe_texture *)realloc(c->textures, cap * sizeof(fe_texture));
        if (!n) return 0;
        memset(n + c->tex_cap, 0, (cap - c->tex_cap) * sizeof(fe_texture));
        c->textures = n;
        c->tex_cap = cap;
    }
    texture_init_slot(&c->textures[c->tex_count]);
    c->tex_count++;
    return (GLuint)c->tex_count;
}

void fe_textures_free(GLState *c)
{
    for (size_t i = 0; i < c->tex_count; i++)
        if (c->textures[i].dev) mtgl_dev_texture_destroy(c->dev, c->textures[i].dev);
    free(c->textures);
    c->textures = NULL;
    c->tex_count = c->tex_cap = 0;
}

void glGenTextures(GLsizei n, GLuint *ids)
{
    CHECK_CTX();
    if (n < 0) {
        fe_set_error(fe_ctx, GL_INVALID_VALUE);
        return;
    }
    for (GLsizei i = 0; i < n; i++) ids[i] = texture_alloc(fe_ctx);
}

void glDeleteTextures(GLsizei n, const GLuint *ids)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (n < 0) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    for (GLsizei i = 0; i < n; i++) {
        if (ids[i] == c->bound_texture) c->bound_texture = 0;
        fe_texture *t = fe_texture_get(c, ids[i]);
        if (!t) continue;
        if (t->dev) {
            mtgl_dev_texture_destroy(c->dev, t->dev);
            t->dev = 0;
        }
        t->width = t->height = 0;
        t->has_image = 0;
        t->allocated = 0;
    }
}

void glBindTexture(GLenum target, GLuint id)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_BIND_TEXTURE, {target, 0, 0}, id, {0}, {0}};
    if (fe_rec(&cmd)) return;
    if (target != GL_TEXTURE_2D) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    fe_ctx->bound_texture = id;
}

/* glTexImage2D (gl_api.c:794-834) + texture_upload_* (textures.c:141-269): level 0 only;
 * every format becomes packed RGBA8 (graphics.h:420-434). Under the MTGL_OPT_MIPMAP_CHAIN
 * extension (no counterpart in the reference) a level above 0 of an uploaded texture
 * replaces that level of its chain: GL_INVALID_OPERATION without a level-0 image,
 * GL_INVALID_VALUE when the chain has no such level or the size is not the level's. */
void glTexImage2D(GLenum target, GLint level, GLint internalformat, GLsizei width, GLsizei height, GLint border,
                  GLenum format, GLenum type, const GLvoid *pixels)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    (void)internalformat;
    (void)border;
    if (target != GL_TEXTURE_2D) {
        fe_set_error(c, GL_INVALID_ENUM);
        return;
    }
    if ((level != 0 && !(c->mipmap_chain && level > 0)) || type != GL_UNSIGNED_BYTE) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    if (width < 0 || height < 0) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    fe_texture *t = fe_texture_get(c, c->bound_texture);
    if (!t) return;
    int comps;
    switch (format) {
    case GL_RGBA: comps = 4; break;
    case GL_RGB: comps = 3; break;
    case GL_LUMINANCE: comps = 1; break;
    case GL_LUMINANCE_ALPHA: comps = 2; break;
    default:
        fe_set_error(c, GL_INVALID_ENUM);
        return;
    }
    /* upload failures (empty or oversized image) leave the texture unchanged */
    if (width <= 0 || height <= 0 || width > FE_MAX_TEXTURE_SIZE || height > FE_MAX_TEXTURE_SIZE) return;
    size_t n = (size_t)width * (size_t)height;
    uint32_t *texels = (uint32_t *)malloc(n * sizeof(uint32_t));
    if (!texels) return;
    const uint8_t *s = (const uint8_t *)pixels;
    for (size_t i = 0; i < n; i++) {
        uint32_t r = 0, g = 0, b = 0, a = 255;
        if (s) {
            if (comps == 4) { r = s[4 * i]; g = s[4 * i + 1]; b = s[4 * i + 2]; a = s[4 * i + 3]; }
            else if (comps == 3) { r = s[3 * i]; g = s[3 * i + 1]; b = s[3 * i + 2]; }
            else if (comps == 1) { r = g = b = s[i]; }
            else { r = g = b = s[2 * i]; a = s[2 * i + 1]; }
        }
        texels[i] = (a << 24) | (b << 16) | (g << 8) | r;
    }
    int st = MTGL_OK;
    if (level > 0) {
        if (!t->has_image || !t->dev) {
            free(texels);
            fe_set_error(c, GL_INVALID_OPERATION);
            return;
        }
        st = mtgl_dev_texture_level(c->dev, t->dev, level, width, height, texels);
        free(texels);
        if (st == MTGL_ERR_INVALID) fe_set_error(c, GL_INVALID_VALUE);
        else if (st != MTGL_OK) fe_dev_error(c, st);
        return;
    }
    if (!t->dev) st = mtgl_dev_texture_create(c->dev, &t->dev);
    if (st == MTGL_OK) st = mtgl_dev_texture_image(c->dev, t->dev, width, height, texels);
    free(texels);
    if (st != MTGL_OK) {
        fe_dev_error(c, st);
        return;
    }
    t->width = width;
    t->height = height;
    t->has_image = 1;
}

void glTexParameteri(GLenum target, GLenum pname, GLint param)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (target != GL_TEXTURE_2D) {
        fe_set_error(c, GL_INVALID_ENUM);
        return;
    }
    fe_texture *t = fe_texture_get(c, c->bound_texture);
    if (!t) return;
    switch (pname) {
    case GL_TEXTURE_MIN_FILTER:
        if (param != GL_NEAREST && param != GL_LINEAR && param != GL_NEAREST_MIPMAP_NEAREST &&
            param != GL_LINEAR_MIPMAP_NEAREST && param != GL_NEAREST_MIPMAP_LINEAR &&
            param != GL_LINEAR_MIPMAP_LINEAR) {
            fe_set_error(c, GL_INVALID_ENUM);
            return;
        }
        t->min_filter = param;
        break;
    case GL_TEXTURE_MAG_FILTER:
        if (param != GL_NEAREST && param != GL_LINEAR) {
            fe_set_error(c, GL_INVALID_ENUM);
            return;
        }
        t->mag_filter = param;
        break;
    case GL_TEXTURE_WRAP_S:
    case GL_TEXTURE_WRAP_T:
        if (param != GL_REPEAT && param != GL_CLAMP && param != GL_CLAMP_TO_EDGE) {
            fe_set_error(c, GL_INVALID_ENUM);
            return;
        }
        if (pname == GL_TEXTURE_WRAP_S) t->wrap_s = param; else t->wrap_t = param;
        break;
    default:
        fe_set_error(c, GL_INVALID_ENUM);
        break;
    }
}

GLboolean glIsTexture(GLuint id)
{
    CHECK_CTX_RET(GL_FALSE);
    if (id == 0) return GL_FALSE;
    return fe_texture_get(fe_ctx, id) ? GL_TRUE : GL_FALSE;
}

/* ---- buffer objects ---- */

fe_buffer *fe_buffer_get(GLState *c, GLuint id)
{
    if (id == 0 || id > c->buf_count) return NULL;
    fe_buffer *b = &c->buffers[id - 1];
    return b->allocated ? b : NULL;
}

void fe_buffers_free(GLState *c)
{
    for (size_t i = 0; i < c->buf_count; i++) {
        if (c->buffers[i].dev) mtgl_dev_buffer_destroy(c->dev, c->buffers[i].dev);
        free(c->buffers[i].shadow);
    }
    free(c->buffers);
    c->buffers = NULL;
    c->buf_count = c->buf_cap = 0;
}

static void buffer_reset(fe_buffer *b)
{
    mtgl_handle keep = b->dev;
    uint64_t ver = b->version;
    memset(b, 0, sizeof(*b));
    b->dev = keep;
    b->version = ver + 1;
    b->allocated = 1;
}

/* buffer_gen (vbo.c:34-92) */
void glGenBuffers(GLsizei n, GLuint *ids)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (n < 0) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    for (GLsizei i = 0; i < n; i++) {
        GLuint found = 0;
        for (size_t j = 0; j < c->buf_count; j++) {
            if (!c->buffers[j].allocated) {
                buffer_reset(&c->buffers[j]);
                found = (GLuint)(j + 1);
                break;
            }
        }
        if (found) {
            ids[i] = found;
            continue;
        }
        if (c->buf_count >= FE_MAX_BUFFERS) {
            ids[i] = 0;
            continue;
        }
        if (c->buf_count == c->buf_cap) {
            size_t cap = c->buf_cap ? c->buf_cap * 2 : 16;
            if (cap > FE_MAX_BUFFERS) cap = FE_MAX_BUFFERS;
            fe_buffer *nb = (fe_buffer *)realloc(c->buffers, cap * sizeof(fe_buffer));
            if (!nb) {
                ids[i] = 0;
                continue;
            }
            memset(nb + c->buf_cap, 0, (cap - c->buf_cap) * sizeof(fe_buffer));
            c->buffers = nb;
            c->buf_cap = cap;
        }
        buffer_reset(&c->buffers[c->buf_count]);
        c->buf_count++;
        ids[i] = (GLuint)c->buf_count;
    }
}

void glDeleteBuffers(GLsizei n, const GLuint *ids)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (n < 0) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    for (GLsizei i = 0; i < n; i++) {
        if (ids[i] == c->bound_array_buffer) c->bound_array_buffer = 0;
        if (ids[i] == c->bound_element_buffer) c->bound_element_buffer = 0;
    }
    for (GLsizei i = 0; i < n; i++) {
        fe_buffer *b = fe_buffer_get(c, ids[i]);
        if (!b) continue;
        if (b->dev) {
            mtgl_dev_buffer_destroy(c->dev, b->dev);
            b->dev = 0;
        }
        free(b->shadow);
        b->shadow = NULL;
        b->size = 0;
        b->allocated = 0;
    }
}

void glBindBuffer(GLenum target, GLuint id)
{
    CHECK_CTX();
    if (target == GL_ARRAY_BUFFER) fe_ctx->bound_array_buffer = id;
    else if (target == GL_ELEMENT_ARRAY_BUFFER) fe_ctx->bound_element_buffer = id;
    else fe_set_error(fe_ctx, GL_INVALID_ENUM);
}

static fe_buffer *target_buffer(GLState *c, GLenum target, int *bad_enum)
{
    *bad_enum = 0;
    if (target == GL_ARRAY_BUFFER) return fe_buffer_get(c, c->bound_array_buffer);
    if (target == GL_ELEMENT_ARRAY_BUFFER) return fe_buffer_get(c, c->bound_element_buffer);
    *bad_enum = 1;
    return NULL;
}

/* glBufferData + buffer_data (gl_api.c:1560-1584, vbo.c:120-151) */
void glBufferData(GLenum target, GLsizeiptr size, const GLvoid *data, GLenum usage)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (size < 0) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    int bad;
    fe_buffer *b = target_buffer(c, target, &bad);
    if (bad) {
        fe_set_error(c, GL_INVALID_ENUM);
        return;
    }
    if (!b) return;
    b->usage = usage;
    b->version++;
    b->rng_valid = 0;
    if (size <= 0) {
        free(b->shadow);
        b->shadow = NULL;
        b->size = 0;
        if (b->dev) fe_dev_error(c, mtgl_dev_buffer_data(c->dev, b->dev, NULL, 0));
        return;
    }
    /* the reference leaves a NULL-data buffer uninitialised; this one zero-fills it */
    uint8_t *shadow = (uint8_t *)(data ? malloc((size_t)size) : calloc(1, (size_t)size));
    if (!shadow) return;
    if (data) memcpy(shadow, data, (size_t)size);
    int st = MTGL_OK;
    if (!b->dev) st = mtgl_dev_buffer_create(c->dev, &b->dev);
    if (st == MTGL_OK) st = mtgl_dev_buffer_data(c->dev, b->dev, shadow, (uint64_t)size);
    if (st != MTGL_OK) {
        free(shadow);
        fe_dev_error(c, st);
        return;
    }
    free(b->shadow);
    b->shadow = shadow;
    b->size = size;
}

void glBufferSubData(GLenum target, GLintptr offset, GLsizeiptr size, const GLvoid *data)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (offset < 0 || size < 0) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    int bad;
    fe_buffer *b = target_buffer(c, target, &bad);
    if (bad) {
        fe_set_error(c, GL_INVALID_ENUM);
        return;
    }
    if (!b) {
        fe_set_error(c, GL_INVALID_OPERATION);
        return;
    }
    if (!b->shadow || !data || offset + size > b->size) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    if (size == 0) return;
    memcpy(b->shadow + offset, data, (size_t)size);
    b->version++;
    b->rng_valid = 0;
    fe_dev_error(c, mtgl_dev_buffer_sub_data(c->dev, b->dev, (uint64_t)offset, data, (uint64_t)size));
}

GLboolean glIsBuffer(GLuint id)
{
    CHECK_CTX_RET(GL_FALSE);
    if (id == 0) return GL_FALSE;
    return fe_buffer_get(fe_ctx, id) ? GL_TRUE : GL_FALSE;
}

void fe_buffer_index_range(fe_buffer *b, uint64_t offset, GLsizei count, GLenum type, int64_t *mn, int64_t *mx,
                           int *neg)
{
    if (b->rng_valid && b->rng_version == b->version && b->rng_offset == offset && b->rng_count == count &&
        b->rng_type == type) {
        *mn = b->rng_min;
        *mx = b->rng_max;
        *neg = b->rng_neg;
        return;
    }
    fe_scan_indices(b->shadow + offset, type, count, mn, mx, neg);
    b->rng_valid = 1;
    b->rng_version = b->version;
    b->rng_offset = offset;
    b->rng_count = count;
    b->rng_type = type;
    b->rng_min = *mn;
    b->rng_max = *mx;
    b->rng_neg = *neg;
}
