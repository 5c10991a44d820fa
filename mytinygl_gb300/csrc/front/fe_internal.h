/*
 * fe_internal.h — state of the C99 GL front end.
 *
 * The front end owns everything MyTinyGL keeps in GLState (src/mytinygl.h:86-225) except
 * the framebuffer and the texel/vertex storage the kernels read: those live behind the
 * mtgl_dev ABI. It validates arguments, keeps the matrix stacks, lights, materials and
 * object tables, records display lists, and turns glEnd / glDrawArrays / glDrawElements
 * into draw packets.
 *
 * Host-side float math (matrix products, normal matrix, light derivations) uses the same
 * operation order as the reference (src/graphics.h) and is compiled with
 * -ffp-contract=off, so the matrices handed to the device are bit-identical to the ones the
 * reference would use.
 */
#ifndef MTGL_FE_INTERNAL_H
#define MTGL_FE_INTERNAL_H

#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "GL/gl.h"
#include "mytinygl/mtgl_dev.h"
#include "mytinygl/mytinygl.h"

#define FE_MAX_STACK 24         /* MAX_MATRIX_STACK_DEPTH, mytinygl.h:21 */
#define FE_MAX_LIGHTS 8         /* MAX_LIGHTS, mytinygl.h:22 */
#define FE_MAX_CALL_DEPTH 64    /* MAX_LIST_CALL_DEPTH, mytinygl.h:23 */
#define FE_MAX_TEXTURES 256     /* GL_MAX_TEXTURES, textures.h:18 */
#define FE_MAX_TEXTURE_SIZE 2048 /* MYTGL_MAX_TEXTURE_SIZE, textures.h:17 */
#define FE_MAX_BUFFERS 256      /* GL_MAX_BUFFERS, vbo.h:17 */
#define FE_MAX_LISTS 1024       /* GL_MAX_LISTS, lists.h:18 */
#define FE_MAX_FB_DIM 16384     /* MYTGL_MAX_FRAMEBUFFER_DIM, framebuffer.h:30 */

/* enable bits (same meaning as mytinygl.h:26-37) */
#define F_INSIDE_BEGIN_END (1u << 0)
#define F_DEPTH_TEST (1u << 1)
#define F_CULL_FACE (1u << 2)
#define F_BLEND (1u << 3)
#define F_TEXTURE_2D (1u << 4)
#define F_LIGHTING (1u << 5)
#define F_FOG (1u << 6)
#define F_NORMALIZE (1u << 7)
#define F_COLOR_MATERIAL (1u << 8)
#define F_ALPHA_TEST (1u << 9)
#define F_SCISSOR_TEST (1u << 10)
#define F_STENCIL_TEST (1u << 11)

#define CL_VERTEX (1u << 0)
#define CL_COLOR (1u << 1)
#define CL_TEXCOORD (1u << 2)
#define CL_NORMAL (1u << 3)

typedef struct {
    GLint size;
    GLenum type;
    GLsizei stride;
    const void *pointer;
} fe_array;

/* One immediate-mode vertex as emit_vertex receives it: object position (w is 1, as every
 * glVertex* entry point passes), the current colour, texcoord and normal. */
typedef struct {
    float pos[3];
    float color[4];
    float tex[2];
    float normal[3];
} fe_vertex;

typedef struct {
    int allocated;
    mtgl_handle dev;
    int32_t width, height;   /* 0 until an image is uploaded */
    int has_image;
    int32_t min_filter, mag_filter, wrap_s, wrap_t;
} fe_texture;

typedef struct {
    int allocated;
    mtgl_handle dev;
    uint8_t *shadow;         /* host copy: glDrawElements index ranges, last-vertex state */
    GLsizeiptr size;
    GLenum usage;
    uint64_t version;
    /* last glDrawElements index-range scan of this buffer (content version + request) */
    uint64_t rng_version, rng_offset;
    GLsizei rng_count;
    GLenum rng_type;
    int64_t rng_min, rng_max;
    int rng_neg, rng_valid;
} fe_buffer;

/* display list command (opcode set of lists.h:21-53) */
typedef enum {
    LC_END = 0, LC_BEGIN, LC_VERTEX, LC_COLOR, LC_TEXCOORD, LC_NORMAL, LC_TRANSLATE, LC_ROTATE, LC_SCALE,
    LC_PUSH, LC_POP, LC_LOAD_IDENTITY, LC_MULT_MATRIX, LC_LOAD_MATRIX, LC_MATRIX_MODE, LC_ORTHO, LC_FRUSTUM,
    LC_ENABLE, LC_DISABLE, LC_BIND_TEXTURE, LC_BLEND_FUNC, LC_DEPTH_FUNC, LC_DEPTH_MASK, LC_CULL_FACE,
    LC_FRONT_FACE, LC_SHADE_MODEL, LC_LIGHTF, LC_LIGHTFV, LC_MATERIALF, LC_MATERIALFV, LC_CALL_LIST
} fe_list_op;

typedef struct {
    fe_list_op op;
    GLenum e[3];
    GLuint u;
    float f[16];
    double d[6];
} fe_list_cmd;

/* A glBegin/glEnd block of a display list whose vertices live in the list's device buffer.
 * Its commands are glVertex / glColor / glTexCoord / glNormal only, and each attribute is
 * either never set inside the block (every vertex takes the current value at call time) or
 * set before the block's first vertex (every vertex takes values recorded in the list). */
typedef struct {
    size_t begin, end;           /* indices of its LC_BEGIN and LC_END commands */
    GLenum mode;
    uint32_t first, count;       /* its vertices in the device buffer */
    uint32_t set;                /* CL_COLOR / CL_TEXCOORD / CL_NORMAL set inside the block */
    float color[4], tex[2], normal[3];  /* values current after the block (when set) */
    float last_color[4];         /* colour of the block's last vertex (when CL_COLOR is set) */
} fe_list_block;

typedef struct {
    int allocated;
    int valid;
    fe_list_cmd *cmds;
    size_t count, cap;
    mtgl_handle vb;              /* device copy of the blocks' vertices (fe_vertex layout) */
    fe_list_block *blocks;       /* in command order */
    size_t nblocks;
} fe_list;

struct GLState {
    mtgl_dev *dev;
    int32_t width, height;
    int mipmap_chain; /* MTGL_OPT_MIPMAP_CHAIN: glTexImage2D accepts levels above 0 */

    float clear_color[4];
    double clear_depth;
    GLint stencil_clear;

    GLint viewport[4];

    float cur_color[4], cur_tex[2], cur_normal[3];

    GLenum matrix_mode;
    float mv[FE_MAX_STACK][16], proj[FE_MAX_STACK][16], texm[FE_MAX_STACK][16];
    GLint mv_depth, proj_depth, tex_depth;

    GLenum prim_mode;
    uint32_t flags;

    GLenum blend_src, blend_dst;
    GLenum cull_mode, front_face;
    GLenum depth_func;
    GLboolean depth_mask;
    GLenum alpha_func;
    float alpha_ref;
    GLint scissor[4];
    GLenum stencil_func;
    GLint stencil_ref;
    GLuint stencil_mask;
    GLenum stencil_fail, stencil_zfail, stencil_zpass;
    GLuint stencil_writemask;
    double depth_near, depth_far;
    GLboolean color_mask[4];
    float line_width, point_size;
    GLenum poly_front, poly_back;

    fe_texture *textures;
    size_t tex_count, tex_cap;
    GLuint bound_texture;
    GLenum tex_env_mode;
    float tex_env_color[4];
    GLenum persp_hint;

    GLint raster_x, raster_y;
    GLboolean raster_valid;

    GLenum fog_mode;
    float fog_density, fog_start, fog_end, fog_color[4];

    mtgl_lighting lit;           /* lights (with enable bits), materials, light model */
    GLenum color_material_face, color_material_mode;
    GLenum shade_model;

    fe_buffer *buffers;
    size_t buf_count, buf_cap;
    GLuint bound_array_buffer, bound_element_buffer;

    uint32_t client_state;
    fe_array vp, cp, tp, np;

    fe_list *lists;
    size_t list_count, list_cap;
    GLuint list_base, list_index;
    GLenum list_mode;
    GLuint list_call_depth;

    /* immediate-mode batch: vertices emitted since the last glEnd */
    fe_vertex *imm;
    uint32_t *imm_vs;            /* per-vertex index into vstates */
    size_t imm_count, imm_cap;
    mtgl_vertex_state *vstates;  /* distinct per-vertex states of the batch */
    uint32_t vs_count, vs_cap;
    int vs_dirty;

    GLenum error;
    uint32_t *host_color;        /* mtgl_color_buffer() mirror */
    int dev_status;
};

/* the calling thread's current context (gl_api.c:14-23) */
extern __thread GLState *fe_ctx;

#define CHECK_CTX() do { if (!fe_ctx) return; } while (0)
#define CHECK_CTX_RET(v) do { if (!fe_ctx) return (v); } while (0)

void fe_set_error(GLState *c, GLenum e);
void fe_dev_error(GLState *c, int status);   /* map an mtgl_status to a GL error */
void fe_state_changed(GLState *c);           /* per-vertex state may have changed */

/* ---- float helpers with the reference's operation order (src/graphics.h) ---- */
static inline void fe_mat4_identity(float *m)
{
    for (int i = 0; i < 16; i++) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}

/* mat4_mul (graphics.h:140-152): r = a * b */
static inline void fe_mat4_mul(const float *a, const float *b, float *r)
{
    float t[16];
    for (int col = 0; col < 4; col++)
        for (int row = 0; row < 4; row++)
            t[col * 4 + row] = a[0 * 4 + row] * b[col * 4 + 0] + a[1 * 4 + row] * b[col * 4 + 1] +
                               a[2 * 4 + row] * b[col * 4 + 2] + a[3 * 4 + row] * b[col * 4 + 3];
    memcpy(r, t, sizeof(t));
}

/* mat4_mul_vec4 (graphics.h:131-138) */
static inline void fe_mat4_mul_vec4(const float *m, const float *v, float *o)
{
    float x = m[0] * v[0] + m[4] * v[1] + m[8] * v[2] + m[12] * v[3];
    float y = m[1] * v[0] + m[5] * v[1] + m[9] * v[2] + m[13] * v[3];
    float z = m[2] * v[0] + m[6] * v[1] + m[10] * v[2] + m[14] * v[3];
    float w = m[3] * v[0] + m[7] * v[1] + m[11] * v[2] + m[15] * v[3];
    o[0] = x; o[1] = y; o[2] = z; o[3] = w;
}

/* vec3_normalize (graphics.h:54-60) */
static inline void fe_vec3_normalize(const float *v, float *o)
{
    float len = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (len > 0.0f) {
        float s = 1.0f / len;
        o[0] = v[0] * s; o[1] = v[1] * s; o[2] = v[2] * s;
    } else {
        o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
    }
}

/* x86-64 cvttss2si: NaN and out-of-range inputs give INT32_MIN. The reference is built
 * for x86-64, so every float->int conversion it performs is restated through this. */
static inline int32_t fe_f2i(float f)
{
    if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int32_t)f;
}

/* color_to_rgba32 (graphics.h:337-348) */
static inline uint32_t fe_color_to_rgba32(const float *c)
{
    uint32_t out = 0;
    for (int i = 0; i < 4; i++) {
        float v = c[i] < 0.0f ? 0.0f : (c[i] > 1.0f ? 1.0f : c[i]);
        uint32_t b = (uint32_t)fe_f2i(v * 255.0f) & 0xFFu;
        out |= b << (8 * i);
    }
    return out;
}

/* front-end internals shared between translation units */
void fe_flush_immediate(GLState *c);          /* glEnd body: submit the batch */
int fe_draw_list_block(GLState *c, mtgl_handle vb, const fe_list_block *b); /* 0: replay instead */
void fe_snapshot_raster(GLState *c, mtgl_raster_state *rs);
void fe_snapshot_vertex(GLState *c, mtgl_vertex_state *vs);
fe_texture *fe_texture_get(GLState *c, GLuint id);
fe_buffer *fe_buffer_get(GLState *c, GLuint id);
fe_list *fe_list_get(GLState *c, GLuint id);
void fe_scan_indices(const void *data, GLenum type, GLsizei count, int64_t *mn, int64_t *mx, int *neg);
void fe_buffer_index_range(fe_buffer *b, uint64_t offset, GLsizei count, GLenum type, int64_t *mn, int64_t *mx,
                           int *neg);
void fe_textures_free(GLState *c);
void fe_buffers_free(GLState *c);
void fe_lists_free(GLState *c);
void fe_light_init(mtgl_light *l, int index);
void fe_material_init(mtgl_material *m);

/* display-list recording: returns 1 when the call must not execute (GL_COMPILE) */
int fe_rec(fe_list_cmd *cmd);
int fe_rec_op(fe_list_op op);
int fe_rec_e(fe_list_op op, GLenum a);
int fe_rec_f3(fe_list_op op, float x, float y, float z);

#endif
