/*
 * oracle_backend.c — TEST INFRASTRUCTURE ONLY: the CPU oracle of the GB300 back end.
 *
 * A plain C99 restatement of MyTinyGL's CPU renderer behind the mtgl_dev ABI
 * (include/mytinygl/mtgl_dev.h): the per-vertex stage (gl_api.c:263-348 with
 * lighting.h:53-142), primitive assembly (raster.c:961-1017, 1199-1231), frustum
 * clipping (clipping.h:37-229), render_triangle (raster.c:729-958), the rasterizer and
 * fragment pipeline (raster.c:20-725), points and lines (raster.c:66-296, 776-898,
 * 1019-1196), texture sampling with the lazily built mip level 1 (textures.c:271-563),
 * glClear (gl_api.c:409-457) and glDrawPixels (gl_api.c:1287-1376).
 *
 * It executes every packet immediately, in order, with the reference's float operation
 * order (compiled with -ffp-contract=off, no fast-math) and emulates the x86-64
 * float->int conversions the reference performs, so its output is the reference's
 * output. Linked with the product's C99 front end it forms liboracle_mtgl.so, which the
 * tests, smoke() and bench.py's CPU baseline use as the checker. Nothing in the product
 * links this file.
 *
 * Parity is pinned two ways: against the reference itself, compiled from its sources by
 * oracle/Makefile into oracle/_ref (tests/test_oracle_vs_reference.py), and against
 * golden fixtures rendered by that reference build (tests/golden/).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "GL/gl.h"
#include "mytinygl/mtgl_dev.h"
#include "mytinygl/mytinygl.h"

/* ------------------------------------------------------------------ basics */

typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } v4;
typedef struct { float r, g, b, a; } col;
typedef struct { float x, y; } v2;

/* vertex_t (graphics.h:438-446) */
typedef struct {
    v4 position;
    col color;
    v2 texcoord;
    v3 normal;
    float eye_z;
    v3 eye_pos;
    v3 eye_normal;
} vtx;

/* x86-64 cvttss2si */
static int32_t f2i(float f)
{
    if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int32_t)f;
}

static v3 V3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static v4 V4(float x, float y, float z, float w) { v4 r = {x, y, z, w}; return r; }
static col C4(float r, float g, float b, float a) { col c = {r, g, b, a}; return c; }
static col C4v(const float *p) { col c = {p[0], p[1], p[2], p[3]}; return c; }

static v3 v3_add(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 v3_sub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 v3_scale(v3 v, float s) { return V3(v.x * s, v.y * s, v.z * s); }
static float v3_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float v3_length(v3 v) { return sqrtf(v3_dot(v, v)); }
static v3 v3_normalize(v3 v)
{
    float len = v3_length(v);
    if (len > 0.0f) return v3_scale(v, 1.0f / len);
    return v;
}

static v4 m4_mul_v4(const float *m, v4 v)
{
    return V4(m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w,
              m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w,
              m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w,
              m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w);
}

/* mat4_normal_matrix (graphics.h:229-260) */
static void normal_matrix(const float *m, float *r)
{
    float a = m[0], b = m[1], c = m[2];
    float d = m[4], e = m[5], f = m[6];
    float g = m[8], h = m[9], i = m[10];
    float det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
    for (int k = 0; k < 16; k++) r[k] = (k % 5 == 0) ? 1.0f : 0.0f;
    if (fabsf(det) < 1e-10f) return;
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

static col c_add(col a, col b) { return C4(a.r + b.r, a.g + b.g, a.b + b.b, a.a + b.a); }
static col c_mul(col a, col b) { return C4(a.r * b.r, a.g * b.g, a.b * b.b, a.a * b.a); }
static col c_scale(col c, float s) { return C4(c.r * s, c.g * s, c.b * s, c.a * s); }
static col c_lerp(col a, col b, float t) { return c_add(c_scale(a, 1.0f - t), c_scale(b, t)); }
static col c_lerp_rgb(col a, col b, float t)
{
    return C4(a.r + (b.r - a.r) * t, a.g + (b.g - a.g) * t, a.b + (b.b - a.b) * t, a.a);
}
static col c_clamp(col c)
{
    return C4(c.r < 0 ? 0 : (c.r > 1 ? 1 : c.r), c.g < 0 ? 0 : (c.g > 1 ? 1 : c.g),
              c.b < 0 ? 0 : (c.b > 1 ? 1 : c.b), c.a < 0 ? 0 : (c.a > 1 ? 1 : c.a));
}

/* color_to_rgba32 (graphics.h:337-348) */
static uint32_t c_to_rgba32(col c)
{
    float rf = c.r < 0.0f ? 0.0f : (c.r > 1.0f ? 1.0f : c.r);
    float gf = c.g < 0.0f ? 0.0f : (c.g > 1.0f ? 1.0f : c.g);
    float bf = c.b < 0.0f ? 0.0f : (c.b > 1.0f ? 1.0f : c.b);
    float af = c.a < 0.0f ? 0.0f : (c.a > 1.0f ? 1.0f : c.a);
    uint32_t r = (uint32_t)f2i(rf * 255.0f) & 0xFF;
    uint32_t g = (uint32_t)f2i(gf * 255.0f) & 0xFF;
    uint32_t b = (uint32_t)f2i(bf * 255.0f) & 0xFF;
    uint32_t a = (uint32_t)f2i(af * 255.0f) & 0xFF;
    return (a << 24) | (b << 16) | (g << 8) | r;
}

static col c_from_rgba32(uint32_t p)
{
    return C4((p & 0xFF) / 255.0f, ((p >> 8) & 0xFF) / 255.0f, ((p >> 16) & 0xFF) / 255.0f,
              ((p >> 24) & 0xFF) / 255.0f);
}

static col c_bary(col a, col b, col c, float b0, float b1, float b2)
{
    return C4(a.r * b0 + b.r * b1 + c.r * b2, a.g * b0 + b.g * b1 + c.g * b2,
              a.b * b0 + b.b * b1 + c.b * b2, a.a * b0 + b.a * b1 + c.a * b2);
}
static v3 v3_bary(v3 a, v3 b, v3 c, float b0, float b1, float b2)
{
    return V3(a.x * b0 + b.x * b1 + c.x * b2, a.y * b0 + b.y * b1 + c.y * b2, a.z * b0 + b.z * b1 + c.z * b2);
}

/* vertex_lerp (graphics.h:465-475) */
static vtx vtx_lerp(const vtx *a, const vtx *b, float t)
{
    vtx v;
    v.position = V4(a->position.x + t * (b->position.x - a->position.x),
                    a->position.y + t * (b->position.y - a->position.y),
                    a->position.z + t * (b->position.z - a->position.z),
                    a->position.w + t * (b->position.w - a->position.w));
    v.color = c_lerp(a->color, b->color, t);
    v.texcoord.x = a->texcoord.x + t * (b->texcoord.x - a->texcoord.x);
    v.texcoord.y = a->texcoord.y + t * (b->texcoord.y - a->texcoord.y);
    v.normal = V3(a->normal.x + t * (b->normal.x - a->normal.x), a->normal.y + t * (b->normal.y - a->normal.y),
                  a->normal.z + t * (b->normal.z - a->normal.z));
    v.eye_z = a->eye_z + t * (b->eye_z - a->eye_z);
    v.eye_pos = V3(a->eye_pos.x + t * (b->eye_pos.x - a->eye_pos.x), a->eye_pos.y + t * (b->eye_pos.y - a->eye_pos.y),
                   a->eye_pos.z + t * (b->eye_pos.z - a->eye_pos.z));
    v.eye_normal = V3(a->eye_normal.x + t * (b->eye_normal.x - a->eye_normal.x),
                      a->eye_normal.y + t * (b->eye_normal.y - a->eye_normal.y),
                      a->eye_normal.z + t * (b->eye_normal.z - a->eye_normal.z));
    return v;
}

/* ------------------------------------------------------------------ device state */

typedef struct {
    uint8_t *data;
    uint64_t size;
} obuf;

#define OMAX_CHAIN 16
typedef struct {
    int32_t width, height;
    uint32_t *pixels;
    int32_t mip1_width, mip1_height;
    uint32_t *mip1;
    /* MTGL_OPT_MIPMAP_CHAIN (an extension of this library, not of the reference): levels 2.. */
    int nchain;
    int32_t chain_w[OMAX_CHAIN], chain_h[OMAX_CHAIN];
    uint32_t *chain[OMAX_CHAIN];
} otex;

struct mtgl_dev {
    int32_t w, h;
    uint32_t *color;
    float *depth;
    uint8_t *stencil;
    mtgl_stats stats;
    const mtgl_raster_state *rs; /* raster state of the packet being rendered */
    int mipmap_chain;            /* MTGL_OPT_MIPMAP_CHAIN */
};

const char *mtgl_dev_last_error(void) { return ""; }
const char *mtgl_dev_backend_name(void) { return "cpu-oracle"; }

int mtgl_dev_create(int32_t width, int32_t height, mtgl_dev **out)
{
    mtgl_dev *d = (mtgl_dev *)calloc(1, sizeof(mtgl_dev));
    if (!d) return MTGL_ERR_OOM;
    size_t n = (size_t)width * (size_t)height;
    d->w = width;
    d->h = height;
    d->color = (uint32_t *)calloc(n, 4);
    d->depth = (float *)calloc(n, 4);
    d->stencil = (uint8_t *)calloc(n, 1);
    if (!d->color || !d->depth || !d->stencil) {
        free(d->color); free(d->depth); free(d->stencil); free(d);
        return MTGL_ERR_OOM;
    }
    *out = d;
    return MTGL_OK;
}

int mtgl_dev_destroy(mtgl_dev *d)
{
    if (!d) return MTGL_OK;
    free(d->color); free(d->depth); free(d->stencil); free(d);
    return MTGL_OK;
}

int mtgl_dev_buffer_create(mtgl_dev *d, mtgl_handle *out)
{
    (void)d;
    obuf *b = (obuf *)calloc(1, sizeof(obuf));
    if (!b) return MTGL_ERR_OOM;
    *out = (mtgl_handle)(uintptr_t)b;
    return MTGL_OK;
}

int mtgl_dev_buffer_data(mtgl_dev *d, mtgl_handle h, const void *data, uint64_t bytes)
{
    (void)d;
    obuf *b = (obuf *)(uintptr_t)h;
    if (!b) return MTGL_ERR_INVALID;
    uint8_t *n = bytes ? (uint8_t *)malloc(bytes) : NULL;
    if (bytes && !n) return MTGL_ERR_OOM;
    if (bytes) {
        if (data) memcpy(n, data, bytes); else memset(n, 0, bytes);
    }
    free(b->data);
    b->data = n;
    b->size = bytes;
    return MTGL_OK;
}

int mtgl_dev_buffer_sub_data(mtgl_dev *d, mtgl_handle h, uint64_t offset, const void *data, uint64_t bytes)
{
    (void)d;
    obuf *b = (obuf *)(uintptr_t)h;
    if (!b || offset + bytes > b->size) return MTGL_ERR_INVALID;
    memcpy(b->data + offset, data, bytes);
    return MTGL_OK;
}

int mtgl_dev_buffer_destroy(mtgl_dev *d, mtgl_handle h)
{
    (void)d;
    obuf *b = (obuf *)(uintptr_t)h;
    if (!b) return MTGL_OK;
    free(b->data);
    free(b);
    return MTGL_OK;
}

int mtgl_dev_texture_create(mtgl_dev *d, mtgl_handle *out)
{
    (void)d;
    otex *t = (otex *)calloc(1, sizeof(otex));
    if (!t) return MTGL_ERR_OOM;
    *out = (mtgl_handle)(uintptr_t)t;
    return MTGL_OK;
}

static void free_chain(otex *t)
{
    for (int i = 0; i < t->nchain; i++) free(t->chain[i]);
    t->nchain = 0;
}

static int gen_mip1(otex *t);
static int build_chain(otex *t);

/* texture_upload_* (textures.c:141-174): new base level, mip level 1 invalidated */
int mtgl_dev_texture_image(mtgl_dev *d, mtgl_handle h, int32_t width, int32_t height, const uint32_t *rgba32)
{
    otex *t = (otex *)(uintptr_t)h;
    if (!t || width <= 0 || height <= 0) return MTGL_ERR_INVALID;
    size_t n = (size_t)width * (size_t)height;
    uint32_t *p = (uint32_t *)malloc(n * 4);
    if (!p) return MTGL_ERR_OOM;
    memcpy(p, rgba32, n * 4);
    free(t->pixels);
    free(t->mip1);
    free_chain(t);
    t->mip1 = NULL;
    t->mip1_width = t->mip1_height = 0;
    t->pixels = p;
    t->width = width;
    t->height = height;
    /* the extension builds every level at once (level 1 as the reference builds it) */
    if (d && d->mipmap_chain && gen_mip1(t) == 0 && build_chain(t) != 0) return MTGL_ERR_OOM;
    return MTGL_OK;
}

int mtgl_dev_texture_level(mtgl_dev *d, mtgl_handle h, int32_t level, int32_t width, int32_t height,
                           const uint32_t *rgba32)
{
    (void)d;
    otex *t = (otex *)(uintptr_t)h;
    if (!t || !rgba32 || level < 1 || t->nchain == 0) return MTGL_ERR_INVALID;
    uint32_t *dst = NULL;
    if (level == 1 && t->mip1 && width == t->mip1_width && height == t->mip1_height) dst = t->mip1;
    if (level >= 2 && level - 2 < t->nchain && width == t->chain_w[level - 2] && height == t->chain_h[level - 2])
        dst = t->chain[level - 2];
    if (!dst) return MTGL_ERR_INVALID;
    memcpy(dst, rgba32, (size_t)width * (size_t)height * 4);
    return MTGL_OK;
}

int mtgl_dev_texture_destroy(mtgl_dev *d, mtgl_handle h)
{
    (void)d;
    otex *t = (otex *)(uintptr_t)h;
    if (!t) return MTGL_OK;
    free(t->pixels);
    free(t->mip1);
    free_chain(t);
    free(t);
    return MTGL_OK;
}

/* ------------------------------------------------------------------ framebuffer access (framebuffer.h:92-134) */

static void put_pixel(mtgl_dev *d, int32_t x, int32_t y, uint32_t c)
{
    if (x < 0 || x >= d->w || y < 0 || y >= d->h) return;
    d->color[(size_t)y * d->w + x] = c;
}
static uint32_t get_pixel(mtgl_dev *d, int32_t x, int32_t y)
{
    if (x < 0 || x >= d->w || y < 0 || y >= d->h) return 0;
    return d->color[(size_t)y * d->w + x];
}
static void put_depth(mtgl_dev *d, int32_t x, int32_t y, float v)
{
    if (x < 0 || x >= d->w || y < 0 || y >= d->h) return;
    d->depth[(size_t)y * d->w + x] = v;
}
static float get_depth(mtgl_dev *d, int32_t x, int32_t y)
{
    if (x < 0 || x >= d->w || y < 0 || y >= d->h) return 1.0f;
    return d->depth[(size_t)y * d->w + x];
}
static void put_stencil(mtgl_dev *d, int32_t x, int32_t y, uint8_t s)
{
    if (x < 0 || x >= d->w || y < 0 || y >= d->h) return;
    d->stencil[(size_t)y * d->w + x] = s;
}
static uint8_t get_stencil(mtgl_dev *d, int32_t x, int32_t y)
{
    if (x < 0 || x >= d->w || y < 0 || y >= d->h) return 0;
    return d->stencil[(size_t)y * d->w + x];
}

/* write_pixel_masked (raster.c:20-45) */
static void write_pixel_masked(mtgl_dev *d, int32_t x, int32_t y, col c)
{
    const mtgl_raster_state *rs = d->rs;
    if (rs->color_mask[0] && rs->color_mask[1] && rs->color_mask[2] && rs->color_mask[3]) {
        put_pixel(d, x, y, c_to_rgba32(c));
        return;
    }
    if (!rs->color_mask[0] && !rs->color_mask[1] && !rs->color_mask[2] && !rs->color_mask[3]) return;
    col dst = c_from_rgba32(get_pixel(d, x, y));
    if (rs->color_mask[0]) dst.r = c.r;
    if (rs->color_mask[1]) dst.g = c.g;
    if (rs->color_mask[2]) dst.b = c.b;
    if (rs->color_mask[3]) dst.a = c.a;
    put_pixel(d, x, y, c_to_rgba32(dst));
}

/* ------------------------------------------------------------------ tests and blending (raster.c:343-448) */

static int cmp_test(uint32_t func, float a, float b)
{
    switch (func) {
    case GL_NEVER: return 0;
    case GL_LESS: return a < b;
    case GL_EQUAL: return a == b;
    case GL_LEQUAL: return a <= b;
    case GL_GREATER: return a > b;
    case GL_NOTEQUAL: return a != b;
    case GL_GEQUAL: return a >= b;
    default: return 1;
    }
}

static col blend_factor(uint32_t f, col s, col d)
{
    switch (f) {
    case GL_ZERO: return C4(0, 0, 0, 0);
    case GL_ONE: return C4(1, 1, 1, 1);
    case GL_SRC_COLOR: return s;
    case GL_ONE_MINUS_SRC_COLOR: return C4(1 - s.r, 1 - s.g, 1 - s.b, 1 - s.a);
    case GL_DST_COLOR: return d;
    case GL_ONE_MINUS_DST_COLOR: return C4(1 - d.r, 1 - d.g, 1 - d.b, 1 - d.a);
    case GL_SRC_ALPHA: return C4(s.a, s.a, s.a, s.a);
    case GL_ONE_MINUS_SRC_ALPHA: return C4(1 - s.a, 1 - s.a, 1 - s.a, 1 - s.a);
    case GL_DST_ALPHA: return C4(d.a, d.a, d.a, d.a);
    case GL_ONE_MINUS_DST_ALPHA: return C4(1 - d.a, 1 - d.a, 1 - d.a, 1 - d.a);
    case GL_SRC_ALPHA_SATURATE: {
        float f2 = (s.a < (1 - d.a)) ? s.a : (1 - d.a);
        return C4(f2, f2, f2, 1);
    }
    default: return C4(1, 1, 1, 1);
    }
}

static col blend_colors(const mtgl_raster_state *rs, col s, col d)
{
    col sf = blend_factor(rs->blend_src, s, d);
    col df = blend_factor(rs->blend_dst, s, d);
    return c_clamp(c_add(c_mul(s, sf), c_mul(d, df)));
}

static int stencil_test(uint32_t func, int32_t ref, uint32_t mask, uint8_t val)
{
    int32_t mr = (int32_t)((uint32_t)ref & mask);
    int32_t mv = (int32_t)(val & mask);
    switch (func) {
    case GL_NEVER: return 0;
    case GL_LESS: return mr < mv;
    case GL_EQUAL: return mr == mv;
    case GL_LEQUAL: return mr <= mv;
    case GL_GREATER: return mr > mv;
    case GL_NOTEQUAL: return mr != mv;
    case GL_GEQUAL: return mr >= mv;
    default: return 1;
    }
}

static uint8_t stencil_op(uint32_t op, uint8_t v, int32_t ref)
{
    switch (op) {
    case GL_KEEP: return v;
    case GL_ZERO: return 0;
    case GL_REPLACE: return (uint8_t)(ref & 0xFF);
    case GL_INCR: return v < 255 ? (uint8_t)(v + 1) : 255;
    case GL_INCR_WRAP: return (uint8_t)(v + 1);
    case GL_DECR: return v > 0 ? (uint8_t)(v - 1) : 0;
    case GL_DECR_WRAP: return (uint8_t)(v - 1);
    case GL_INVERT: return (uint8_t)~v;
    default: return v;
    }
}

static void write_stencil_masked(mtgl_dev *d, int32_t x, int32_t y, uint8_t nv, uint32_t wm)
{
    uint8_t old = get_stencil(d, x, y);
    uint8_t m8 = (uint8_t)(wm & 0xFF);
    put_stencil(d, x, y, (uint8_t)((old & ~m8) | (nv & m8)));
}

/* depth range mapping: float NDC term, double range arithmetic, float result (raster.c:548) */
static float map_depth(const mtgl_raster_state *rs, float z)
{
    return (float)((z + 1.0f) * 0.5f * (rs->depth_far - rs->depth_near) + rs->depth_near);
}

static col apply_fog(const mtgl_raster_state *rs, col c, float fog_coord, int triangle)
{
    float f;
    switch (rs->fog_mode) {
    case GL_LINEAR:
        if (rs->fog_end != rs->fog_start) f = (rs->fog_end - fog_coord) / (rs->fog_end - rs->fog_start);
        else f = 1.0f;
        break;
    case GL_EXP: f = expf(-rs->fog_density * fog_coord); break;
    case GL_EXP2: {
        float dd = rs->fog_density * fog_coord;
        f = expf(-dd * dd);
        break;
    }
    default: f = 1.0f; break;
    }
    (void)triangle;
    if (f < 0.0f) f = 0.0f;
    if (f > 1.0f) f = 1.0f;
    return c_lerp_rgb(C4v(rs->fog_color), c, f);
}

/* ------------------------------------------------------------------ lighting (lighting.h:53-142) */

static col compute_lighting(const mtgl_lighting *L, v3 eye_pos, v3 eye_normal, const mtgl_material *mat)
{
    col result = c_add(C4v(mat->emission), c_mul(C4v(mat->ambient), C4v(L->model_ambient)));
    result.a = mat->diffuse[3];
    v3 N = eye_normal;
    if (L->normalize) N = v3_normalize(N);
    for (int i = 0; i < MTGL_MAX_LIGHTS; i++) {
        const mtgl_light *l = &L->lights[i];
        if (!l->enabled) continue;
        v3 Ld;
        float att = 1.0f;
        if (l->position[3] == 0.0f) {
            Ld = v3_normalize(V3(l->position[0], l->position[1], l->position[2]));
        } else {
            v3 lp = V3(l->position[0], l->position[1], l->position[2]);
            v3 to = v3_sub(lp, eye_pos);
            float dist = v3_length(to);
            if (dist < 1e-6f) dist = 1e-6f;
            Ld = v3_scale(to, 1.0f / dist);
            float den = l->constant_attenuation + l->linear_attenuation * dist + l->quadratic_attenuation * dist * dist;
            if (den < 1e-6f) den = 1e-6f;
            att = 1.0f / den;
            if (l->spot_cutoff < 180.0f) {
                v3 sd = v3_normalize(V3(l->spot_direction[0], l->spot_direction[1], l->spot_direction[2]));
                float cos_angle = -v3_dot(Ld, sd);
                float cos_cutoff = cosf(l->spot_cutoff * 3.14159265f / 180.0f);
                if (cos_angle < cos_cutoff) att = 0.0f;
                else att *= powf(cos_angle, l->spot_exponent);
            }
        }
        if (att <= 0.0f) continue;
        result = c_add(result, c_scale(c_mul(C4v(mat->ambient), C4v(l->ambient)), att));
        float NdotL = v3_dot(N, Ld);
        if (NdotL > 0.0f) {
            result = c_add(result, c_scale(c_mul(C4v(mat->diffuse), C4v(l->diffuse)), att * NdotL));
            if (mat->shininess > 0.0f) {
                v3 V = L->local_viewer ? v3_normalize(v3_scale(eye_pos, -1.0f)) : V3(0.0f, 0.0f, 1.0f);
                v3 H = v3_normalize(v3_add(Ld, V));
                float NdotH = v3_dot(N, H);
                if (NdotH > 0.0f) {
                    float spec = powf(NdotH, mat->shininess) * att;
                    result = c_add(result, c_scale(c_mul(C4v(mat->specular), C4v(l->specular)), spec));
                }
            }
        }
    }
    return c_clamp(result);
}

/* ------------------------------------------------------------------ textures (textures.c:271-563) */

/* level `mip` of a texture: 0 the base, 1 the reference's level 1, 2.. the extension's chain */
static void level_of(const otex *t, int mip, const uint32_t **px, int32_t *w, int32_t *h)
{
    if (mip == 0) { *px = t->pixels; *w = t->width; *h = t->height; }
    else if (mip == 1) { *px = t->mip1; *w = t->mip1_width; *h = t->mip1_height; }
    else { *px = t->chain[mip - 2]; *w = t->chain_w[mip - 2]; *h = t->chain_h[mip - 2]; }
}

static uint32_t texel_wrapped(const otex *t, const mtgl_raster_state *rs, int32_t x, int32_t y, int mip)
{
    const uint32_t *px;
    int32_t w, h;
    level_of(t, mip, &px, &w, &h);
    if (rs->tex_wrap_s == GL_REPEAT) x = ((x % w) + w) % w;
    else { if (x < 0) x = 0; else if (x >= w) x = w - 1; }
    if (rs->tex_wrap_t == GL_REPEAT) y = ((y % h) + h) % h;
    else { if (y < 0) y = 0; else if (y >= h) y = h - 1; }
    return px[(size_t)y * w + x];
}

static uint32_t bilinear(uint32_t c00, uint32_t c10, uint32_t c01, uint32_t c11, float fx, float fy)
{
    col top = c_lerp(c_from_rgba32(c00), c_from_rgba32(c10), fx);
    col bot = c_lerp(c_from_rgba32(c01), c_from_rgba32(c11), fx);
    return c_to_rgba32(c_lerp(top, bot, fy));
}

/* texture_generate_mip1 (textures.c:311-354), built on first use */
static int gen_mip1(otex *t)
{
    if (t->mip1) return 0;
    if (!t->pixels || t->width < 2 || t->height < 2) return -1;
    t->mip1_width = t->width / 2;
    t->mip1_height = t->height / 2;
    t->mip1 = (uint32_t *)malloc((size_t)t->mip1_width * t->mip1_height * 4);
    if (!t->mip1) {
        t->mip1_width = t->mip1_height = 0;
        return -1;
    }
    for (int32_t y = 0; y < t->mip1_height; y++)
        for (int32_t x = 0; x < t->mip1_width; x++) {
            int32_t sx = 2 * x, sy = 2 * y;
            col c = c_from_rgba32(t->pixels[(size_t)sy * t->width + sx]);
            c = c_add(c, c_from_rgba32(t->pixels[(size_t)sy * t->width + sx + 1]));
            c = c_add(c, c_from_rgba32(t->pixels[(size_t)(sy + 1) * t->width + sx]));
            c = c_add(c, c_from_rgba32(t->pixels[(size_t)(sy + 1) * t->width + sx + 1]));
            c = c_scale(c, 0.25f);
            t->mip1[(size_t)y * t->mip1_width + x] = c_to_rgba32(c);
        }
    return 0;
}

/* the extension's levels 2..: the 2x2 box filter of texture_generate_mip1 (textures.c:311-354)
 * applied to each level in turn, while both sides of the previous one are at least 2 */
static int build_chain(otex *t)
{
    const uint32_t *src = t->mip1;
    int32_t sw = t->mip1_width, sh = t->mip1_height;
    while (sw >= 2 && sh >= 2 && t->nchain < OMAX_CHAIN) {
        int32_t w = sw / 2, h = sh / 2;
        uint32_t *dst = (uint32_t *)malloc((size_t)w * h * 4);
        if (!dst) return -1;
        for (int32_t y = 0; y < h; y++)
            for (int32_t x = 0; x < w; x++) {
                int32_t sx = 2 * x, sy = 2 * y;
                col c = c_from_rgba32(src[(size_t)sy * sw + sx]);
                c = c_add(c, c_from_rgba32(src[(size_t)sy * sw + sx + 1]));
                c = c_add(c, c_from_rgba32(src[(size_t)(sy + 1) * sw + sx]));
                c = c_add(c, c_from_rgba32(src[(size_t)(sy + 1) * sw + sx + 1]));
                c = c_scale(c, 0.25f);
                dst[(size_t)y * w + x] = c_to_rgba32(c);
            }
        t->chain[t->nchain] = dst;
        t->chain_w[t->nchain] = w;
        t->chain_h[t->nchain] = h;
        t->nchain++;
        src = dst;
        sw = w;
        sh = h;
    }
    return 0;
}

static uint32_t sample_level(otex *t, const mtgl_raster_state *rs, float u, float v, int linear, int mip)
{
    const uint32_t *lpx;
    int32_t w, h;
    level_of(t, mip, &lpx, &w, &h);
    float tx = u * w - 0.5f;
    float ty = v * h - 0.5f;
    if (linear) {
        int32_t x0 = f2i(floorf(tx)), y0 = f2i(floorf(ty));
        int32_t x1 = x0 + 1, y1 = y0 + 1;
        float fx = tx - x0, fy = ty - y0;
        return bilinear(texel_wrapped(t, rs, x0, y0, mip), texel_wrapped(t, rs, x1, y0, mip),
                        texel_wrapped(t, rs, x0, y1, mip), texel_wrapped(t, rs, x1, y1, mip), fx, fy);
    }
    int32_t x = f2i(floorf(tx + 0.5f)), y = f2i(floorf(ty + 0.5f));
    if (x < 0) x = 0;
    if (x >= w) x = w - 1;
    if (y < 0) y = 0;
    if (y >= h) y = h - 1;
    return lpx[(size_t)y * w + x];
}

/* The extension's mipmap filters over the whole chain (levels 0 .. top, lod > 0):
 * *_MIPMAP_NEAREST the level floor(lod + 0.5), *_MIPMAP_LINEAR the blend of levels floor(lod)
 * and floor(lod) + 1 by the fraction, as the reference blends levels 0 and 1; from the top
 * level up, that level alone. */
static uint32_t sample_chain(otex *t, const mtgl_raster_state *rs, float u, float v, float lod, int32_t filter)
{
    int top = 1 + t->nchain;
    int lin = filter == GL_LINEAR_MIPMAP_NEAREST || filter == GL_LINEAR_MIPMAP_LINEAR;
    if (filter == GL_NEAREST_MIPMAP_NEAREST || filter == GL_LINEAR_MIPMAP_NEAREST) {
        int d = lod >= (float)top ? top : (int)(lod + 0.5f);
        if (d > top) d = top;
        return sample_level(t, rs, u, v, lin, d);
    }
    if (lod >= (float)top) return sample_level(t, rs, u, v, lin, top);
    int d = (int)lod;
    float f = lod - (float)d;
    uint32_t c0 = sample_level(t, rs, u, v, lin, d);
    uint32_t c1 = sample_level(t, rs, u, v, lin, d + 1);
    return c_to_rgba32(c_lerp(c_from_rgba32(c0), c_from_rgba32(c1), f));
}

static uint32_t sample_mip1(otex *t, const mtgl_raster_state *rs, float u, float v, int32_t filter)
{
    if (gen_mip1(t) != 0) return 0xFFFFFFFFu;
    int lin = filter == GL_LINEAR || filter == GL_LINEAR_MIPMAP_NEAREST || filter == GL_LINEAR_MIPMAP_LINEAR;
    return sample_level(t, rs, u, v, lin, 1);
}

/* texture_sample_lod (textures.c:457-557) */
static uint32_t sample_lod(otex *t, const mtgl_raster_state *rs, float u, float v, float lod)
{
    if (!t->pixels || t->width <= 0 || t->height <= 0) return 0xFFFFFFFFu;
    if (rs->tex_wrap_s == GL_REPEAT) {
        u = u - (float)f2i(u);
        if (u < 0) u += 1.0f;
    } else {
        if (u < 0.0f) u = 0.0f;
        if (u > 1.0f) u = 1.0f;
    }
    if (rs->tex_wrap_t == GL_REPEAT) {
        v = v - (float)f2i(v);
        if (v < 0) v += 1.0f;
    } else {
        if (v < 0.0f) v = 0.0f;
        if (v > 1.0f) v = 1.0f;
    }
    int32_t filter = (lod > 0.0f) ? rs->tex_min_filter : rs->tex_mag_filter;
    if (lod > 0.0f && filter != GL_NEAREST && filter != GL_LINEAR && t->nchain > 0)
        return sample_chain(t, rs, u, v, lod, filter);
    if (filter == GL_NEAREST_MIPMAP_NEAREST || filter == GL_LINEAR_MIPMAP_NEAREST) {
        if (lod >= 0.5f) return sample_mip1(t, rs, u, v, filter);
        filter = (filter == GL_NEAREST_MIPMAP_NEAREST) ? GL_NEAREST : GL_LINEAR;
    } else if (filter == GL_NEAREST_MIPMAP_LINEAR || filter == GL_LINEAR_MIPMAP_LINEAR) {
        if (lod > 0.0f) {
            float cl = (lod > 1.0f) ? 1.0f : lod;
            int base_linear = (filter == GL_LINEAR_MIPMAP_LINEAR);
            uint32_t c0 = sample_level(t, rs, u, v, base_linear, 0);
            uint32_t c1 = sample_mip1(t, rs, u, v, filter);
            return c_to_rgba32(c_lerp(c_from_rgba32(c0), c_from_rgba32(c1), cl));
        }
        filter = (filter == GL_NEAREST_MIPMAP_LINEAR) ? GL_NEAREST : GL_LINEAR;
    }
    return sample_level(t, rs, u, v, filter == GL_LINEAR, 0);
}

static otex *bound_texture(const mtgl_raster_state *rs)
{
    otex *t = (otex *)(uintptr_t)rs->texture;
    return (t && t->pixels) ? t : NULL;
}

/* ------------------------------------------------------------------ triangles */

static void ndc_to_screen(const mtgl_raster_state *rs, float x, float y, int32_t *sx, int32_t *sy)
{
    *sx = f2i((x + 1.0f) * 0.5f * (float)rs->viewport[2] + (float)rs->viewport[0]);
    *sy = f2i((1.0f - y) * 0.5f * (float)rs->viewport[3] + (float)rs->viewport[1]);
}

static float edge_fn(float ax, float ay, float bx, float by, float px, float py)
{
    return (px - ax) * (by - ay) - (py - ay) * (bx - ax);
}

/* rasterize_triangle_smooth (raster.c:451-725) */
static void raster_smooth(mtgl_dev *dv, int32_t x0, int32_t y0, float z0, float w0i, col c0, v2 uv0, float ez0,
                          int32_t x1, int32_t y1, float z1, float w1i, col c1, v2 uv1, float ez1,
                          int32_t x2, int32_t y2, float z2, float w2i, col c2, v2 uv2, float ez2,
                          v3 ep0, v3 en0, v3 ep1, v3 en1, v3 ep2, v3 en2, int back)
{
    const mtgl_raster_state *rs = dv->rs;
    int32_t minX = x0 < x1 ? (x0 < x2 ? x0 : x2) : (x1 < x2 ? x1 : x2);
    int32_t minY = y0 < y1 ? (y0 < y2 ? y0 : y2) : (y1 < y2 ? y1 : y2);
    int32_t maxX = x0 > x1 ? (x0 > x2 ? x0 : x2) : (x1 > x2 ? x1 : x2);
    int32_t maxY = y0 > y1 ? (y0 > y2 ? y0 : y2) : (y1 > y2 ? y1 : y2);
    if (minX < rs->viewport[0]) minX = rs->viewport[0];
    if (minY < rs->viewport[1]) minY = rs->viewport[1];
    if (maxX >= rs->viewport[0] + rs->viewport[2]) maxX = rs->viewport[0] + rs->viewport[2] - 1;
    if (maxY >= rs->viewport[1] + rs->viewport[3]) maxY = rs->viewport[1] + rs->viewport[3] - 1;
    if (rs->scissor_test) {
        if (minX < rs->scissor[0]) minX = rs->scissor[0];
        if (minY < rs->scissor[1]) minY = rs->scissor[1];
        if (maxX >= rs->scissor[0] + rs->scissor[2]) maxX = rs->scissor[0] + rs->scissor[2] - 1;
        if (maxY >= rs->scissor[1] + rs->scissor[3]) maxY = rs->scissor[1] + rs->scissor[3] - 1;
    }
    if (minX > maxX || minY > maxY) return;
    /* pixels outside the framebuffer read defaults and write nothing (framebuffer.h:92-134) */
    if (minX < 0) minX = 0;
    if (minY < 0) minY = 0;
    if (maxX > dv->w - 1) maxX = dv->w - 1;
    if (maxY > dv->h - 1) maxY = dv->h - 1;

    float area = edge_fn((float)x0, (float)y0, (float)x1, (float)y1, (float)x2, (float)y2);
    if (fabsf(area) < 0.5f) return;
    float inv_area = 1.0f / area;
    int persp = rs->perspective_hint != GL_FASTEST;
    otex *tex = bound_texture(rs);
    float u0w = uv0.x * w0i, v0w = uv0.y * w0i;
    float u1w = uv1.x * w1i, v1w = uv1.y * w1i;
    float u2w = uv2.x * w2i, v2w = uv2.y * w2i;
    float lod = 0.0f;
    if (tex) {
        float screen_area = fabsf(area) * 0.5f;
        float du1 = (uv1.x - uv0.x) * tex->width;
        float dv1 = (uv1.y - uv0.y) * tex->height;
        float du2 = (uv2.x - uv0.x) * tex->width;
        float dv2 = (uv2.y - uv0.y) * tex->height;
        float texel_area = fabsf(du1 * dv2 - du2 * dv1) * 0.5f;
        if (screen_area > 0.0f) {
            float tpp = texel_area / screen_area;
            if (tpp > 0.0f) {
                lod = log2f(tpp) * 0.5f;
                if (lod < 0.0f) lod = 0.0f;
            }
        }
    }
    float fx0 = (float)x0, fy0 = (float)y0, fx1 = (float)x1, fy1 = (float)y1, fx2 = (float)x2, fy2 = (float)y2;
    /* the state the loop reads, held in locals: the framebuffer stores below may alias the
       state block's integer fields as far as the compiler knows */
    const int depth_test = rs->depth_test, depth_write = rs->depth_test && rs->depth_mask;
    const uint32_t depth_func = rs->depth_func;
    const int stencil = rs->stencil_test, blend = rs->blend, fog = rs->fog, flat = rs->shade_model == GL_FLAT;
    const int lit_frag = rs->lighting && (rs->shade_model == GL_PHONG || (back && rs->lit.two_side));
    const int all_mask = rs->color_mask[0] && rs->color_mask[1] && rs->color_mask[2] && rs->color_mask[3];
    uint32_t *const color = dv->color;
    float *const depthbuf = dv->depth;
    const int32_t fbw = dv->w;
    uint64_t frags = 0;
    for (int32_t y = minY; y <= maxY; y++) {
        for (int32_t x = minX; x <= maxX; x++) {
            float px = (float)x, py = (float)y;
            float e0 = edge_fn(fx1, fy1, fx2, fy2, px, py);
            float e1 = edge_fn(fx2, fy2, fx0, fy0, px, py);
            float e2 = edge_fn(fx0, fy0, fx1, fy1, px, py);
            if (!((area > 0 && e0 >= 0 && e1 >= 0 && e2 >= 0) || (area < 0 && e0 <= 0 && e1 <= 0 && e2 <= 0)))
                continue;
            frags++;
            /* (x, y) lies inside the framebuffer: the box was clamped to it above */
            const size_t pi = (size_t)y * fbw + x;
            float b0 = e0 * inv_area, b1 = e1 * inv_area, b2 = e2 * inv_area;
            float z = b0 * z0 + b1 * z1 + b2 * z2;
            float depth = map_depth(rs, z);
            uint8_t sv = 0;
            if (stencil) {
                sv = get_stencil(dv, x, y);
                if (!stencil_test(rs->stencil_func, rs->stencil_ref, rs->stencil_mask, sv)) {
                    write_stencil_masked(dv, x, y, stencil_op(rs->stencil_fail, sv, rs->stencil_ref), rs->stencil_writemask);
                    continue;
                }
            }
            if (depth_test) {
                if (!cmp_test(depth_func, depth, depthbuf[pi])) {
                    if (stencil)
                        write_stencil_masked(dv, x, y, stencil_op(rs->stencil_zfail, sv, rs->stencil_ref),
                                             rs->stencil_writemask);
                    continue;
                }
            }
            if (stencil)
                write_stencil_masked(dv, x, y, stencil_op(rs->stencil_zpass, sv, rs->stencil_ref), rs->stencil_writemask);
            col c = flat ? c2 : c_bary(c0, c1, c2, b0, b1, b2);
            if (lit_frag) {
                if (rs->shade_model == GL_PHONG) {
                    v3 ep = v3_bary(ep0, ep1, ep2, b0, b1, b2);
                    v3 en = v3_bary(en0, en1, en2, b0, b1, b2);
                    const mtgl_material *mat = &rs->lit.front;
                    if (back && rs->lit.two_side) {
                        en = v3_scale(en, -1.0f);
                        mat = &rs->lit.back;
                    }
                    c = compute_lighting(&rs->lit, ep, en, mat);
                } else {
                    v3 ep = v3_bary(ep0, ep1, ep2, b0, b1, b2);
                    v3 en = v3_scale(v3_bary(en0, en1, en2, b0, b1, b2), -1.0f);
                    c = compute_lighting(&rs->lit, ep, en, &rs->lit.back);
                }
            }
            if (tex) {
                float u, v;
                if (persp) {
                    float uow = b0 * u0w + b1 * u1w + b2 * u2w;
                    float vow = b0 * v0w + b1 * v1w + b2 * v2w;
                    float oow = b0 * w0i + b1 * w1i + b2 * w2i;
                    float w = 1.0f / oow;
                    u = uow * w;
                    v = vow * w;
                } else {
                    u = b0 * uv0.x + b1 * uv1.x + b2 * uv2.x;
                    v = b0 * uv0.y + b1 * uv1.y + b2 * uv2.y;
                }
                col tc = c_from_rgba32(sample_lod(tex, rs, u, v, lod));
                if (rs->alpha_test && !cmp_test(rs->alpha_func, tc.a, rs->alpha_ref)) continue;
                switch (rs->tex_env_mode) {
                case GL_REPLACE: c = tc; break;
                case GL_DECAL: c = c_lerp_rgb(c, tc, tc.a); break;
                case GL_BLEND: {
                    col e = C4v(rs->tex_env_color);
                    c = C4(c.r * (1.0f - tc.r) + e.r * tc.r, c.g * (1.0f - tc.g) + e.g * tc.g,
                           c.b * (1.0f - tc.b) + e.b * tc.b, c.a * tc.a);
                    break;
                }
                case GL_ADD: c = C4(c.r + tc.r, c.g + tc.g, c.b + tc.b, c.a * tc.a); break;
                default: c = c_mul(c, tc); break;
                }
            }
            if (fog) c = apply_fog(rs, c, b0 * ez0 + b1 * ez1 + b2 * ez2, 1);
            if (depth_write) depthbuf[pi] = depth;
            if (blend) c = blend_colors(rs, c, c_from_rgba32(color[pi]));
            c = c_clamp(c);
            if (all_mask) color[pi] = c_to_rgba32(c);
            else write_pixel_masked(dv, x, y, c);
        }
    }
    dv->stats.fragments += frags;
}

/* ------------------------------------------------------------------ lines and points */

static void write_line_pixel(mtgl_dev *dv, int32_t px, int32_t py, float depth, col c)
{
    const mtgl_raster_state *rs = dv->rs;
    if (px < 0 || px >= dv->w || py < 0 || py >= dv->h) return;
    if (rs->scissor_test) {
        if (px < rs->scissor[0] || px >= rs->scissor[0] + rs->scissor[2] || py < rs->scissor[1] ||
            py >= rs->scissor[1] + rs->scissor[3])
            return;
    }
    if (rs->depth_test && !cmp_test(rs->depth_func, depth, get_depth(dv, px, py))) return;
    col fc = c;
    if (rs->blend) fc = blend_colors(rs, fc, c_from_rgba32(get_pixel(dv, px, py)));
    if (rs->depth_test && rs->depth_mask) put_depth(dv, px, py, depth);
    write_pixel_masked(dv, px, py, fc);
}

/* draw_line_full (raster.c:107-241). The reference's loop never advances when the alpha
 * test rejects a pixel (its `continue` skips the Bresenham step) and so never ends; the
 * oracle reports MTGL_ERR_UNSUPPORTED for that combination instead of hanging. */
static int draw_line_full(mtgl_dev *dv, int32_t x0, int32_t y0, float z0, int32_t x1, int32_t y1, float z1, col c0,
                          col c1, float ez0, float ez1, v2 uv0, v2 uv1)
{
    const mtgl_raster_state *rs = dv->rs;
    int32_t dx = x1 - x0, dy = y1 - y0;
    int32_t adx = dx < 0 ? -dx : dx, ady = dy < 0 ? -dy : dy;
    int32_t sx = dx < 0 ? -1 : 1, sy = dy < 0 ? -1 : 1;
    int32_t err = adx - ady;
    int32_t total = adx > ady ? adx : ady;
    if (total == 0) total = 1;
    int32_t step = 0;
    int lw = f2i(rs->line_width + 0.5f);
    if (lw < 1) lw = 1;
    int half = lw / 2;
    int ex = adx > ady ? 0 : 1, ey = adx > ady ? 1 : 0;
    otex *tex = bound_texture(rs);
    int32_t cx = x0, cy = y0;
    for (;;) {
        float t = (float)step / (float)total;
        float z = z0 + t * (z1 - z0);
        float depth = map_depth(rs, z);
        col c = c_lerp(c0, c1, t);
        if (tex) {
            float u = uv0.x + t * (uv1.x - uv0.x);
            float v = uv0.y + t * (uv1.y - uv0.y);
            col tc = c_from_rgba32(sample_lod(tex, rs, u, v, 0.0f));
            if (rs->alpha_test && !cmp_test(rs->alpha_func, tc.a, rs->alpha_ref)) return MTGL_ERR_UNSUPPORTED;
            c = c_mul(c, tc);
        } else if (rs->alpha_test) {
            if (!cmp_test(rs->alpha_func, c.a, rs->alpha_ref)) return MTGL_ERR_UNSUPPORTED;
        }
        if (rs->fog) c = apply_fog(rs, c, -(ez0 + t * (ez1 - ez0)), 0);
        if (lw == 1) {
            if (cx >= 0 && cx < dv->w && cy >= 0 && cy < dv->h) write_line_pixel(dv, cx, cy, depth, c);
        } else {
            for (int w = -half; w < lw - half; w++) write_line_pixel(dv, cx + w * ex, cy + w * ey, depth, c);
        }
        if (cx == x1 && cy == y1) break;
        int32_t e2 = err * 2;
        if (e2 > -ady) { err -= ady; cx += sx; }
        if (e2 < adx) { err += adx; cy += sy; }
        step++;
    }
    return MTGL_OK;
}

/* clip_line (clipping.h:138-229) */
static int outcode(v4 v)
{
    int c = 0;
    if (v.x < -v.w) c |= 1; else if (v.x > v.w) c |= 2;
    if (v.y < -v.w) c |= 4; else if (v.y > v.w) c |= 8;
    if (v.z < -v.w) c |= 16; else if (v.z > v.w) c |= 32;
    return c;
}

static void snap(vtx *v, int plane)
{
    switch (plane) {
    case 2: v->position.x = -v->position.w; break;
    case 3: v->position.x = v->position.w; break;
    case 4: v->position.y = -v->position.w; break;
    case 5: v->position.y = v->position.w; break;
    case 0: v->position.z = -v->position.w; break;
    case 1: v->position.z = v->position.w; break;
    }
}

static int clip_line(vtx *v0, vtx *v1)
{
    int c0 = outcode(v0->position), c1 = outcode(v1->position);
    for (;;) {
        if (!(c0 | c1)) return 1;
        if (c0 & c1) return 0;
        int co = c0 ? c0 : c1;
        v4 *p0 = &v0->position, *p1 = &v1->position;
        float d0 = 0, d1 = 0;
        int plane = -1;
        if (co & 1) { d0 = p0->x + p0->w; d1 = p1->x + p1->w; plane = 2; }
        else if (co & 2) { d0 = p0->w - p0->x; d1 = p1->w - p1->x; plane = 3; }
        else if (co & 4) { d0 = p0->y + p0->w; d1 = p1->y + p1->w; plane = 4; }
        else if (co & 8) { d0 = p0->w - p0->y; d1 = p1->w - p1->y; plane = 5; }
        else if (co & 16) { d0 = p0->z + p0->w; d1 = p1->z + p1->w; plane = 0; }
        else if (co & 32) { d0 = p0->w - p0->z; d1 = p1->w - p1->z; plane = 1; }
        float denom = d0 - d1;
        if (fabsf(denom) < 1e-10f) return 0;
        float t = d0 / denom;
        vtx cl = vtx_lerp(v0, v1, t);
        snap(&cl, plane);
        if (co == c0) { *v0 = cl; c0 = outcode(v0->position); }
        else { *v1 = cl; c1 = outcode(v1->position); }
    }
}

/* draw_line_segment (raster.c:244-285) */
static int draw_line_segment(mtgl_dev *dv, const vtx *s0, const vtx *s1)
{
    vtx v0 = *s0, v1 = *s1;
    if (!clip_line(&v0, &v1)) return MTGL_OK;
    float z0, z1;
    if (fabsf(v0.position.w) >= 1e-6f) {
        float iw = 1.0f / v0.position.w;
        v0.position.x *= iw; v0.position.y *= iw; z0 = v0.position.z * iw;
    } else {
        v0.position.x = 0.0f; v0.position.y = 0.0f; z0 = 0.0f;
    }
    if (fabsf(v1.position.w) >= 1e-6f) {
        float iw = 1.0f / v1.position.w;
        v1.position.x *= iw; v1.position.y *= iw; z1 = v1.position.z * iw;
    } else {
        v1.position.x = 0.0f; v1.position.y = 0.0f; z1 = 0.0f;
    }
    int32_t x0, y0, x1, y1;
    ndc_to_screen(dv->rs, v0.position.x, v0.position.y, &x0, &y0);
    ndc_to_screen(dv->rs, v1.position.x, v1.position.y, &x1, &y1);
    return draw_line_full(dv, x0, y0, z0, x1, y1, z1, v0.color, v1.color, v0.eye_z, v1.eye_z, v0.texcoord, v1.texcoord);
}

/* draw_point_at_screen (raster.c:777-844) */
static void draw_point_at_screen(mtgl_dev *dv, int32_t x, int32_t y, float z, col c, float eye_z)
{
    const mtgl_raster_state *rs = dv->rs;
    if (x < 0 || x >= dv->w || y < 0 || y >= dv->h) return;
    if (rs->scissor_test) {
        if (x < rs->scissor[0] || x >= rs->scissor[0] + rs->scissor[2] || y < rs->scissor[1] ||
            y >= rs->scissor[1] + rs->scissor[3])
            return;
    }
    float depth = map_depth(rs, z);
    if (rs->depth_test && !cmp_test(rs->depth_func, depth, get_depth(dv, x, y))) return;
    if (rs->alpha_test && !cmp_test(rs->alpha_func, c.a, rs->alpha_ref)) return;
    if (rs->fog) c = apply_fog(rs, c, -eye_z, 0);
    if (rs->depth_test && rs->depth_mask) put_depth(dv, x, y, depth);
    if (rs->blend) c = blend_colors(rs, c, c_from_rgba32(get_pixel(dv, x, y)));
    write_pixel_masked(dv, x, y, c);
}

static void phong_vertex_colors(mtgl_dev *dv, const vtx *a, const vtx *b, const vtx *c, col *o)
{
    const mtgl_raster_state *rs = dv->rs;
    o[0] = a->color; o[1] = b->color; o[2] = c->color;
    if (rs->lighting && rs->shade_model == GL_PHONG) {
        o[0] = compute_lighting(&rs->lit, a->eye_pos, a->eye_normal, &rs->lit.front);
        o[1] = compute_lighting(&rs->lit, b->eye_pos, b->eye_normal, &rs->lit.front);
        o[2] = compute_lighting(&rs->lit, c->eye_pos, c->eye_normal, &rs->lit.front);
    }
}

/* ------------------------------------------------------------------ render_triangle (raster.c:729-958) */

static void perspective_divide(vtx *v)
{
    if (fabsf(v->position.w) < 1e-6f) {
        v->position = V4(0.0f, 0.0f, 0.0f, 1.0f);
        return;
    }
    float iw = 1.0f / v->position.w;
    v->position.x *= iw;
    v->position.y *= iw;
    v->position.z *= iw;
    v->position.w = iw;
}

static float plane_dist(const v4 *v, int plane)
{
    switch (plane) {
    case 0: return v->z + v->w;
    case 1: return v->w - v->z;
    case 2: return v->x + v->w;
    case 3: return v->w - v->x;
    case 4: return v->y + v->w;
    default: return v->w - v->y;
    }
}

/* clip_polygon_plane_id (clipping.h:50-99) */
static int clip_plane(const vtx *in, int n, vtx *out, int plane)
{
    if (n == 0) return 0;
    int m = 0;
    const vtx *prev = &in[n - 1];
    float pd = plane_dist(&prev->position, plane);
    for (int i = 0; i < n; i++) {
        const vtx *cur = &in[i];
        float cd = plane_dist(&cur->position, plane);
        if (pd >= 0) {
            if (cd >= 0) {
                out[m++] = *cur;
            } else {
                float den = pd - cd;
                if (fabsf(den) > 1e-10f) {
                    out[m] = vtx_lerp(prev, cur, pd / den);
                    snap(&out[m], plane);
                    m++;
                }
            }
        } else if (cd >= 0) {
            float den = pd - cd;
            if (fabsf(den) > 1e-10f) {
                out[m] = vtx_lerp(prev, cur, pd / den);
                snap(&out[m], plane);
                m++;
            }
            out[m++] = *cur;
        }
        prev = cur;
        pd = cd;
    }
    return m;
}

static int cull(const mtgl_raster_state *rs, float sa)
{
    if (!rs->cull_face) return 0;
    int front = (rs->front_face == GL_CCW) ? (sa < 0) : (sa > 0);
    if (rs->cull_face_mode == GL_FRONT) return front;
    if (rs->cull_face_mode == GL_BACK) return !front;
    return 1;
}

static int render_triangle(mtgl_dev *dv, const vtx *a, const vtx *b, const vtx *cc)
{
    const mtgl_raster_state *rs = dv->rs;
    vtx t0[12], t1[12];
    t0[0] = *a; t0[1] = *b; t0[2] = *cc;
    int n = clip_plane(t0, 3, t1, 0);
    if (n) n = clip_plane(t1, n, t0, 1);
    if (n) n = clip_plane(t0, n, t1, 2);
    if (n) n = clip_plane(t1, n, t0, 3);
    if (n) n = clip_plane(t0, n, t1, 4);
    if (n) n = clip_plane(t1, n, t0, 5);
    if (n < 3) return MTGL_OK;
    vtx *cl = t0;
    for (int j = 0; j < n; j++) perspective_divide(&cl[j]);
    for (int j = 1; j + 1 < n; j++) {
        int32_t x0, y0, x1, y1, x2, y2;
        ndc_to_screen(rs, cl[0].position.x, cl[0].position.y, &x0, &y0);
        ndc_to_screen(rs, cl[j].position.x, cl[j].position.y, &x1, &y1);
        ndc_to_screen(rs, cl[j + 1].position.x, cl[j + 1].position.y, &x2, &y2);
        /* int differences wrap like the reference's x86-64 build */
        float sa = (float)(int32_t)((uint32_t)x1 - (uint32_t)x0) * (float)(int32_t)((uint32_t)y2 - (uint32_t)y0) -
                   (float)(int32_t)((uint32_t)x2 - (uint32_t)x0) * (float)(int32_t)((uint32_t)y1 - (uint32_t)y0);
        if (cull(rs, sa)) continue;
        int back = (rs->front_face == GL_CCW) ? (sa >= 0) : (sa < 0);
        uint32_t pm = back ? rs->polygon_mode_back : rs->polygon_mode_front;
        const vtx *p0 = &cl[0], *p1 = &cl[j], *p2 = &cl[j + 1];
        if (pm == GL_POINT) {
            col co[3];
            phong_vertex_colors(dv, p0, p1, p2, co);
            draw_point_at_screen(dv, x0, y0, p0->position.z, co[0], p0->eye_z);
            draw_point_at_screen(dv, x1, y1, p1->position.z, co[1], p1->eye_z);
            draw_point_at_screen(dv, x2, y2, p2->position.z, co[2], p2->eye_z);
        } else if (pm == GL_LINE) {
            col co[3];
            phong_vertex_colors(dv, p0, p1, p2, co);
            int st = draw_line_full(dv, x0, y0, p0->position.z, x1, y1, p1->position.z, co[0], co[1], p0->eye_z,
                                    p1->eye_z, p0->texcoord, p1->texcoord);
            if (st == MTGL_OK)
                st = draw_line_full(dv, x1, y1, p1->position.z, x2, y2, p2->position.z, co[1], co[2], p1->eye_z,
                                    p2->eye_z, p1->texcoord, p2->texcoord);
            if (st == MTGL_OK)
                st = draw_line_full(dv, x2, y2, p2->position.z, x0, y0, p0->position.z, co[2], co[0], p2->eye_z,
                                    p0->eye_z, p2->texcoord, p0->texcoord);
            if (st != MTGL_OK) return st;
        } else {
            dv->stats.setup_triangles++;
            raster_smooth(dv, x0, y0, p0->position.z, p0->position.w, p0->color, p0->texcoord, p0->eye_z,
                          x1, y1, p1->position.z, p1->position.w, p1->color, p1->texcoord, p1->eye_z,
                          x2, y2, p2->position.z, p2->position.w, p2->color, p2->texcoord, p2->eye_z,
                          p0->eye_pos, p0->eye_normal, p1->eye_pos, p1->eye_normal, p2->eye_pos, p2->eye_normal, back);
        }
    }
    return MTGL_OK;
}

/* flush_points (raster.c:1020-1164) */
static void draw_points(mtgl_dev *dv, const vtx *v, int32_t n)
{
    const mtgl_raster_state *rs = dv->rs;
    int ps = f2i(rs->point_size + 0.5f);
    if (ps < 1) ps = 1;
    int half = ps / 2;
    otex *tex = bound_texture(rs);
    for (int32_t i = 0; i < n; i++) {
        v4 p = v[i].position;
        if (p.x < -p.w || p.x > p.w || p.y < -p.w || p.y > p.w || p.z < -p.w || p.z > p.w || p.w <= 0.0f) continue;
        float nx = p.x / p.w, ny = p.y / p.w, nz = p.z / p.w;
        int32_t cx, cy;
        ndc_to_screen(rs, nx, ny, &cx, &cy);
        float depth = map_depth(rs, nz);
        col c = v[i].color;
        if (tex) {
            col tc = c_from_rgba32(sample_lod(tex, rs, v[i].texcoord.x, v[i].texcoord.y, 0.0f));
            if (rs->alpha_test && !cmp_test(rs->alpha_func, tc.a, rs->alpha_ref)) continue;
            c = c_mul(c, tc);
        } else if (rs->alpha_test) {
            if (!cmp_test(rs->alpha_func, c.a, rs->alpha_ref)) continue;
        }
        if (rs->fog) c = apply_fog(rs, c, -v[i].eye_z, 0);
        int32_t xs = cx - half, ys = cy - half;
        for (int32_t py = ys; py < ys + ps; py++)
            for (int32_t px = xs; px < xs + ps; px++) {
                if (px < 0 || px >= dv->w || py < 0 || py >= dv->h) continue;
                if (rs->scissor_test) {
                    if (px < rs->scissor[0] || px >= rs->scissor[0] + rs->scissor[2] || py < rs->scissor[1] ||
                        py >= rs->scissor[1] + rs->scissor[3])
                        continue;
                }
                if (rs->depth_test && !cmp_test(rs->depth_func, depth, get_depth(dv, px, py))) continue;
                col fc = c;
                if (rs->blend) fc = blend_colors(rs, fc, c_from_rgba32(get_pixel(dv, px, py)));
                if (rs->depth_test && rs->depth_mask) put_depth(dv, px, py, depth);
                write_pixel_masked(dv, px, py, fc);
            }
    }
}

/* ------------------------------------------------------------------ per-vertex stage */

static int fetch_attr(const mtgl_attrib *a, int64_t index, float *out, int n)
{
    /* get_array_element (gl_api.c:1758-1797) */
    if (index < 0) {
        for (int i = 0; i < n; i++) out[i] = (i < 3) ? 0.0f : 1.0f;
        return 1;
    }
    const uint8_t *base;
    uint64_t limit;
    if (a->buffer) {
        obuf *b = (obuf *)(uintptr_t)a->buffer;
        base = b->data ? b->data + a->offset : NULL;
        limit = a->bytes;
    } else {
        base = (const uint8_t *)a->host;
        limit = UINT64_MAX;
    }
    int comp = a->type == GL_FLOAT ? 4 : 1;
    uint64_t off = (uint64_t)index * (uint64_t)a->stride;
    if (!base || a->stride <= 0 || off + (uint64_t)a->size * comp > limit) {
        /* beyond the buffer: the reference reads undefined memory; the oracle reads zeros */
        for (int i = 0; i < n; i++) out[i] = (i == 3) ? 1.0f : 0.0f;
        return 0;
    }
    const uint8_t *p = base + off;
    for (int i = 0; i < a->size && i < n; i++) {
        if (a->type == GL_FLOAT) { float f; memcpy(&f, p + 4 * i, 4); out[i] = f; }
        else out[i] = p[i] / 255.0f;
    }
    for (int i = a->size; i < n; i++) out[i] = (i == 3) ? 1.0f : 0.0f;
    return 1;
}

static void sanitize_color(float *c)
{
    for (int i = 0; i < 4; i++) {
        if (isnan(c[i]) || isinf(c[i])) c[i] = (i == 3) ? 1.0f : 0.0f;
        if (c[i] < 0.0f) c[i] = 0.0f; else if (c[i] > 1.0f) c[i] = 1.0f;
    }
}

/* emit_vertex (gl_api.c:263-348) for element `index` of the packet */
static vtx vertex_stage(const mtgl_draw *d, const mtgl_vertex_state *vs, int64_t index)
{
    float p[4], cc[4], t[2], nn[3];
    fetch_attr(&d->position, index, p, 4);
    float x = p[0], y = p[1], z = d->position_2d ? 0.0f : p[2];
    if (d->color.enabled) { fetch_attr(&d->color, index, cc, 4); sanitize_color(cc); }
    else memcpy(cc, d->current_color, sizeof(cc));
    if (d->texcoord.enabled) fetch_attr(&d->texcoord, index, t, 2);
    else memcpy(t, d->current_texcoord, sizeof(t));
    if (d->normal.enabled) fetch_attr(&d->normal, index, nn, 3);
    else memcpy(nn, d->current_normal, sizeof(nn));

    v4 obj = V4(x, y, z, 1.0f);
    v4 eye = m4_mul_v4(vs->modelview, obj);
    float eye_z = -eye.z;
    v3 eye_pos = V3(eye.x, eye.y, eye.z);
    float nm[16];
    normal_matrix(vs->modelview, nm);
    v4 n4 = m4_mul_v4(nm, V4(nn[0], nn[1], nn[2], 0.0f));
    v3 eye_normal = v3_normalize(V3(n4.x, n4.y, n4.z));
    col vc = C4v(cc);
    mtgl_material front = vs->lit.front;
    if (vs->lighting && vs->color_material) {
        col k = c_clamp(vc);
        float kk[4] = {k.r, k.g, k.b, k.a};
        uint32_t mode = vs->color_material_mode, face = vs->color_material_face;
        if (face == GL_FRONT || face == GL_FRONT_AND_BACK) {
            if (mode == GL_AMBIENT || mode == GL_AMBIENT_AND_DIFFUSE) memcpy(front.ambient, kk, sizeof(kk));
            if (mode == GL_DIFFUSE || mode == GL_AMBIENT_AND_DIFFUSE) memcpy(front.diffuse, kk, sizeof(kk));
            if (mode == GL_SPECULAR) memcpy(front.specular, kk, sizeof(kk));
            if (mode == GL_EMISSION) memcpy(front.emission, kk, sizeof(kk));
        }
    }
    if (vs->lighting && !vs->phong) vc = compute_lighting(&vs->lit, eye_pos, eye_normal, &front);
    v4 pos = m4_mul_v4(vs->projection, m4_mul_v4(vs->modelview, obj));
    v4 t4 = m4_mul_v4(vs->texture, V4(t[0], t[1], 0.0f, 1.0f));
    v2 tc;
    if (t4.w != 0.0f && t4.w != 1.0f) { tc.x = t4.x / t4.w; tc.y = t4.y / t4.w; }
    else { tc.x = t4.x; tc.y = t4.y; }
    vtx out;
    out.position = pos;
    out.color = vc;
    out.texcoord = tc;
    out.normal = V3(nn[0], nn[1], nn[2]);
    out.eye_z = eye_z;
    out.eye_pos = eye_pos;
    out.eye_normal = eye_normal;
    return out;
}

static int64_t element_index(const mtgl_draw *d, int32_t k)
{
    if (!d->index_type) return (int64_t)d->first + k;
    const uint8_t *base;
    if (d->index_buffer) {
        obuf *b = (obuf *)(uintptr_t)d->index_buffer;
        base = b->data + d->index_offset;
    } else {
        base = (const uint8_t *)d->index_host;
    }
    uint32_t v;
    if (d->index_type == GL_UNSIGNED_INT) memcpy(&v, base + 4 * (size_t)k, 4);
    else if (d->index_type == GL_UNSIGNED_SHORT) { uint16_t s; memcpy(&s, base + 2 * (size_t)k, 2); v = s; }
    else v = base[k];
    return (int64_t)(int32_t)v; /* GLuint index passed as GLint (gl_api.c:1758) */
}

int mtgl_dev_draw(mtgl_dev *dv, const mtgl_draw *d)
{
    if (!dv || !d || !d->raster_state || !d->vertex_states || d->count < 0) return MTGL_ERR_INVALID;
    int32_t n = d->count;
    vtx *v = (vtx *)malloc((size_t)(n > 0 ? n : 1) * sizeof(vtx));
    if (!v) return MTGL_ERR_OOM;
    for (int32_t k = 0; k < n; k++) {
        uint32_t s = d->vertex_state_ids ? d->vertex_state_ids[k] : 0;
        if (s >= d->vertex_state_count) s = 0;
        v[k] = vertex_stage(d, &d->vertex_states[s], element_index(d, k));
    }
    dv->rs = d->raster_state;
    dv->stats.draws++;
    int st = MTGL_OK;
    switch (d->mode) {
    case GL_POINTS: draw_points(dv, v, n); break;
    case GL_LINES:
        for (int32_t i = 0; i + 1 < n && st == MTGL_OK; i += 2) st = draw_line_segment(dv, &v[i], &v[i + 1]);
        break;
    case GL_LINE_STRIP:
        for (int32_t i = 0; i + 1 < n && st == MTGL_OK; i++) st = draw_line_segment(dv, &v[i], &v[i + 1]);
        break;
    case GL_LINE_LOOP:
        if (n < 2) break;
        for (int32_t i = 0; i + 1 < n && st == MTGL_OK; i++) st = draw_line_segment(dv, &v[i], &v[i + 1]);
        if (st == MTGL_OK) st = draw_line_segment(dv, &v[n - 1], &v[0]);
        break;
    case GL_TRIANGLES:
        for (int32_t i = 0; i + 2 < n && st == MTGL_OK; i += 3) {
            dv->stats.input_triangles++;
            st = render_triangle(dv, &v[i], &v[i + 1], &v[i + 2]);
        }
        break;
    case GL_TRIANGLE_STRIP:
        for (int32_t i = 0; i + 2 < n && st == MTGL_OK; i++) {
            dv->stats.input_triangles++;
            st = (i % 2 == 0) ? render_triangle(dv, &v[i], &v[i + 1], &v[i + 2])
                              : render_triangle(dv, &v[i + 1], &v[i], &v[i + 2]);
        }
        break;
    case GL_TRIANGLE_FAN:
    case GL_POLYGON:
        for (int32_t i = 1; i + 1 < n && st == MTGL_OK; i++) {
            dv->stats.input_triangles++;
            st = render_triangle(dv, &v[0], &v[i], &v[i + 1]);
        }
        break;
    case GL_QUADS:
        for (int32_t i = 0; i + 3 < n && st == MTGL_OK; i += 4) {
            dv->stats.input_triangles += 2;
            st = render_triangle(dv, &v[i], &v[i + 1], &v[i + 2]);
            if (st == MTGL_OK) st = render_triangle(dv, &v[i], &v[i + 2], &v[i + 3]);
        }
        break;
    case GL_QUAD_STRIP:
        for (int32_t i = 0; i + 3 < n && st == MTGL_OK; i += 2) {
            dv->stats.input_triangles += 2;
            st = render_triangle(dv, &v[i], &v[i + 1], &v[i + 3]);
            if (st == MTGL_OK) st = render_triangle(dv, &v[i], &v[i + 3], &v[i + 2]);
        }
        break;
    default: break;
    }
    dv->rs = NULL;
    free(v);
    return st;
}

/* ------------------------------------------------------------------ clear, pixels, readback */

int mtgl_dev_clear(mtgl_dev *d, uint32_t mask, int32_t x0, int32_t y0, int32_t x1, int32_t y1, uint32_t color,
                   float depth, uint8_t stencil)
{
    for (int32_t y = y0; y < y1; y++)
        for (int32_t x = x0; x < x1; x++) {
            size_t i = (size_t)y * d->w + x;
            if (mask & GL_COLOR_BUFFER_BIT) d->color[i] = color;
            if (mask & GL_DEPTH_BUFFER_BIT) d->depth[i] = depth;
            if (mask & GL_STENCIL_BUFFER_BIT) d->stencil[i] = stencil;
        }
    return MTGL_OK;
}

int mtgl_dev_draw_pixels(mtgl_dev *d, int32_t rx, int32_t ry, int32_t width, int32_t height, const uint32_t *rgba32,
                         const mtgl_raster_state *rs)
{
    for (int32_t row = 0; row < height; row++) {
        int32_t fy = d->h - 1 - (ry + row);
        if (fy < 0 || fy >= d->h) continue;
        for (int32_t colx = 0; colx < width; colx++) {
            int32_t fx = rx + colx;
            if (fx < 0 || fx >= d->w) continue;
            uint32_t p = rgba32[(size_t)row * width + colx];
            uint32_t a = p >> 24;
            if (rs->alpha_test && !cmp_test(rs->alpha_func, a / 255.0f, rs->alpha_ref)) continue;
            if (rs->depth_test && !cmp_test(rs->depth_func, 0.0f, get_depth(d, fx, fy))) continue;
            col s = C4((p & 0xFF) / 255.0f, ((p >> 8) & 0xFF) / 255.0f, ((p >> 16) & 0xFF) / 255.0f, a / 255.0f);
            if (rs->blend) {
                col dst = c_from_rgba32(d->color[(size_t)fy * d->w + fx]);
                col sf = blend_factor(rs->blend_src, s, dst);
                col df = blend_factor(rs->blend_dst, s, dst);
                s = c_clamp(c_add(c_mul(s, sf), c_mul(dst, df)));
            }
            if (rs->depth_test && rs->depth_mask) put_depth(d, fx, fy, 0.0f);
            d->color[(size_t)fy * d->w + fx] = c_to_rgba32(s);
        }
    }
    return MTGL_OK;
}

int mtgl_dev_flush(mtgl_dev *d) { (void)d; return MTGL_OK; }
int mtgl_dev_finish(mtgl_dev *d) { (void)d; return MTGL_OK; }
int mtgl_dev_in_batch(const mtgl_dev *d) { (void)d; return 0; }

int mtgl_dev_read(mtgl_dev *d, uint32_t *color, float *depth, uint8_t *stencil)
{
    size_t n = (size_t)d->w * (size_t)d->h;
    if (color) memcpy(color, d->color, n * 4);
    if (depth) memcpy(depth, d->depth, n * 4);
    if (stencil) memcpy(stencil, d->stencil, n);
    return MTGL_OK;
}

int mtgl_dev_stats(mtgl_dev *d, mtgl_stats *out)
{
    *out = d->stats;
    return MTGL_OK;
}

int mtgl_dev_reset_stats(mtgl_dev *d)
{
    memset(&d->stats, 0, sizeof(d->stats));
    return MTGL_OK;
}

int mtgl_dev_profile(mtgl_dev *d, int enable)
{
    (void)d;
    (void)enable;
    return MTGL_OK;
}

int mtgl_dev_timings(mtgl_dev *d, mtgl_timings *out)
{
    (void)d;
    memset(out, 0, sizeof(*out));
    return MTGL_OK;
}

void *mtgl_dev_stream(mtgl_dev *d)
{
    (void)d;
    return NULL;
}

/* The CPU oracle renders every packet as it arrives; nothing is ever queued. */
int mtgl_flush_noalloc(GLState *ctx)
{
    return ctx ? MTGL_OK : MTGL_ERR_INVALID;
}

int mtgl_dev_debug_bounds(void) { return 0; }

int mtgl_dev_set_option(mtgl_dev *d, int option, int value)
{
    if (option == MTGL_OPT_MIPMAP_CHAIN) {
        if (d) d->mipmap_chain = value != 0;
        return MTGL_OK;
    }
    return option == MTGL_OPT_DEPTH_REJECTION ? MTGL_OK : MTGL_ERR_INVALID;
}

/* ------------------------------------------------------------------ batches
 * The oracle renders every packet as it arrives, so by the time contexts are handed to a
 * batch their frames are complete: a batch only counts what it is given. */
struct mtgl_batch {
    mtgl_batch_config cfg;
    mtgl_batch_stats stats;
};

void mtgl_dev_batch_defaults(mtgl_batch_config *cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->tile_size = 16;
    cfg->record_factor = 1.5f;
    cfg->pair_factor = 8.0f;
    cfg->use_graph = 1;
    cfg->order_by_cost = 1;
    cfg->readback_kernel = 1;
}

int mtgl_dev_batch_create(const mtgl_batch_config *cfg, mtgl_batch **out)
{
    mtgl_batch *b;
    if (!out) return MTGL_ERR_INVALID;
    b = (mtgl_batch *)calloc(1, sizeof(*b));
    if (!b) return MTGL_ERR_OOM;
    mtgl_dev_batch_defaults(&b->cfg);
    if (cfg && cfg->tile_size) b->cfg.tile_size = cfg->tile_size;
    b->stats.tile_size = b->cfg.tile_size;
    *out = b;
    return MTGL_OK;
}

int mtgl_dev_batch_destroy(mtgl_batch *b)
{
    free(b);
    return MTGL_OK;
}

int mtgl_dev_batch_submit(mtgl_batch *b, mtgl_dev *const *devs, int32_t n)
{
    if (!b || n < 0 || (n > 0 && !devs)) return MTGL_ERR_INVALID;
    b->stats.batches++;
    b->stats.frames += (uint64_t)n;
    return MTGL_OK;
}

int mtgl_dev_batch_wait(mtgl_batch *b) { return b ? MTGL_OK : MTGL_ERR_INVALID; }
int mtgl_dev_batch_query(mtgl_batch *b) { return b ? 1 : -MTGL_ERR_INVALID; }
int mtgl_dev_batch_begin(mtgl_batch *b) { return b ? MTGL_OK : MTGL_ERR_INVALID; }
int mtgl_dev_batch_launch(mtgl_batch *b) { return b ? MTGL_OK : MTGL_ERR_INVALID; }

/* The oracle's contexts hold their own framebuffers and render at once: a pass recorded
 * on one context cannot be retargeted. */
int mtgl_dev_batch_add(mtgl_batch *b, mtgl_dev *src, mtgl_dev *target)
{
    if (!b || !src || !target) return MTGL_ERR_INVALID;
    return src == target ? MTGL_OK : MTGL_ERR_UNSUPPORTED;
}

int mtgl_dev_batch_readback(mtgl_batch *b, mtgl_dev *target, uint32_t *host_color)
{
    if (!b || !target || !host_color) return MTGL_ERR_INVALID;
    return mtgl_dev_read(target, host_color, NULL, NULL);
}

int mtgl_dev_batch_stats(mtgl_batch *b, mtgl_batch_stats *out)
{
    if (!b || !out) return MTGL_ERR_INVALID;
    *out = b->stats;
    return MTGL_OK;
}

int mtgl_dev_batch_reset_stats(mtgl_batch *b)
{
    int32_t ts;
    if (!b) return MTGL_ERR_INVALID;
    ts = b->stats.tile_size;
    memset(&b->stats, 0, sizeof(b->stats));
    b->stats.tile_size = ts;
    return MTGL_OK;
}

void *mtgl_dev_batch_stream(mtgl_batch *b)
{
    (void)b;
    return NULL;
}

int mtgl_dev_batch_profile(mtgl_batch *b, int enable)
{
    (void)enable;
    return b ? MTGL_OK : MTGL_ERR_INVALID;
}

int mtgl_dev_batch_timings(mtgl_batch *b, mtgl_timings *out)
{
    if (!b || !out) return MTGL_ERR_INVALID;
    memset(out, 0, sizeof(*out));
    return MTGL_OK;
}

int mtgl_batch_render(mtgl_batch *b, GLState *const *ctxs, int32_t n)
{
    if (!b || n < 0 || (n > 0 && !ctxs)) return MTGL_ERR_INVALID;
    b->stats.batches++;
    b->stats.frames += (uint64_t)n;
    return MTGL_OK;
}

int mtgl_batch_render_read(mtgl_batch *b, GLState *const *ctxs, uint32_t *const *colors, int32_t n)
{
    int st = mtgl_batch_render(b, ctxs, n);
    for (int32_t i = 0; st == MTGL_OK && colors && i < n; i++)
        if (colors[i]) st = mtgl_read_framebuffer(ctxs[i], colors[i], NULL, NULL);
    return st;
}
