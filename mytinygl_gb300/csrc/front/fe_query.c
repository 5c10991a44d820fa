/*
 * fe_query.c — state queries (gl_api.c:2505-3189, 2144-2251).
 *
 * Same pnames, value conventions (stack depth reported +1, float queries falling back to
 * the integer query, boolean queries of enable bits) and error behaviour as the reference.
 */
#include "fe_internal.h"

void glGetIntegerv(GLenum pname, GLint *p)
{
    CHECK_CTX();
    if (!p) return;
    GLState *c = fe_ctx;
    switch (pname) {
    case GL_VIEWPORT: for (int i = 0; i < 4; i++) p[i] = c->viewport[i]; break;
    case GL_MATRIX_MODE: p[0] = (GLint)c->matrix_mode; break;
    case GL_MODELVIEW_STACK_DEPTH: p[0] = c->mv_depth + 1; break;
    case GL_PROJECTION_STACK_DEPTH: p[0] = c->proj_depth + 1; break;
    case GL_TEXTURE_STACK_DEPTH: p[0] = c->tex_depth + 1; break;
    case GL_SHADE_MODEL: p[0] = (GLint)c->shade_model; break;
    case GL_COLOR_MATERIAL_FACE: p[0] = (GLint)c->color_material_face; break;
    case GL_COLOR_MATERIAL_PARAMETER: p[0] = (GLint)c->color_material_mode; break;
    case GL_FOG_MODE: p[0] = (GLint)c->fog_mode; break;
    case GL_LIGHT_MODEL_LOCAL_VIEWER: p[0] = (GLint)c->lit.local_viewer; break;
    case GL_LIGHT_MODEL_TWO_SIDE: p[0] = (GLint)c->lit.two_side; break;
    case GL_CULL_FACE_MODE: p[0] = (GLint)c->cull_mode; break;
    case GL_FRONT_FACE: p[0] = (GLint)c->front_face; break;
    case GL_POLYGON_MODE: p[0] = (GLint)c->poly_front; p[1] = (GLint)c->poly_back; break;
    case GL_TEXTURE_BINDING_2D: p[0] = (GLint)c->bound_texture; break;
    case GL_TEXTURE_ENV_MODE: p[0] = (GLint)c->tex_env_mode; break;
    case GL_SCISSOR_BOX: for (int i = 0; i < 4; i++) p[i] = c->scissor[i]; break;
    case GL_ALPHA_TEST_FUNC: p[0] = (GLint)c->alpha_func; break;
    case GL_STENCIL_FUNC: p[0] = (GLint)c->stencil_func; break;
    case GL_STENCIL_VALUE_MASK: p[0] = (GLint)c->stencil_mask; break;
    case GL_STENCIL_REF: p[0] = c->stencil_ref; break;
    case GL_STENCIL_FAIL: p[0] = (GLint)c->stencil_fail; break;
    case GL_STENCIL_PASS_DEPTH_FAIL: p[0] = (GLint)c->stencil_zfail; break;
    case GL_STENCIL_PASS_DEPTH_PASS: p[0] = (GLint)c->stencil_zpass; break;
    case GL_STENCIL_WRITEMASK: p[0] = (GLint)c->stencil_writemask; break;
    case GL_STENCIL_CLEAR_VALUE: p[0] = c->stencil_clear; break;
    case GL_DEPTH_FUNC: p[0] = (GLint)c->depth_func; break;
    case GL_DEPTH_WRITEMASK: p[0] = c->depth_mask; break;
    case GL_BLEND_SRC: p[0] = (GLint)c->blend_src; break;
    case GL_BLEND_DST: p[0] = (GLint)c->blend_dst; break;
    case GL_COLOR_WRITEMASK: for (int i = 0; i < 4; i++) p[i] = c->color_mask[i]; break;
    case GL_UNPACK_ALIGNMENT: case GL_PACK_ALIGNMENT: p[0] = 4; break;
    case GL_PERSPECTIVE_CORRECTION_HINT: p[0] = (GLint)c->persp_hint; break;
    case GL_FOG_HINT: case GL_LINE_SMOOTH_HINT: case GL_POINT_SMOOTH_HINT: case GL_POLYGON_SMOOTH_HINT:
        p[0] = GL_DONT_CARE;
        break;
    case GL_ARRAY_BUFFER_BINDING: p[0] = (GLint)c->bound_array_buffer; break;
    case GL_ELEMENT_ARRAY_BUFFER_BINDING: p[0] = (GLint)c->bound_element_buffer; break;
    case GL_VERTEX_ARRAY_SIZE: p[0] = c->vp.size; break;
    case GL_VERTEX_ARRAY_TYPE: p[0] = (GLint)c->vp.type; break;
    case GL_VERTEX_ARRAY_STRIDE: p[0] = c->vp.stride; break;
    case GL_COLOR_ARRAY_SIZE: p[0] = c->cp.size; break;
    case GL_COLOR_ARRAY_TYPE: p[0] = (GLint)c->cp.type; break;
    case GL_COLOR_ARRAY_STRIDE: p[0] = c->cp.stride; break;
    case GL_NORMAL_ARRAY_TYPE: p[0] = (GLint)c->np.type; break;
    case GL_NORMAL_ARRAY_STRIDE: p[0] = c->np.stride; break;
    case GL_TEXTURE_COORD_ARRAY_SIZE: p[0] = c->tp.size; break;
    case GL_TEXTURE_COORD_ARRAY_TYPE: p[0] = (GLint)c->tp.type; break;
    case GL_TEXTURE_COORD_ARRAY_STRIDE: p[0] = c->tp.stride; break;
    case GL_LIST_BASE: p[0] = (GLint)c->list_base; break;
    case GL_LIST_INDEX: p[0] = (GLint)c->list_index; break;
    case GL_LIST_MODE: p[0] = c->list_index ? (GLint)c->list_mode : 0; break;
    case GL_CURRENT_RASTER_POSITION: p[0] = c->raster_x; p[1] = c->raster_y; p[2] = 0; p[3] = 1; break;
    case GL_CURRENT_RASTER_POSITION_VALID: p[0] = c->raster_valid; break;
    case GL_RENDER_MODE: p[0] = 0x1C00; break;
    case GL_MAX_LIGHTS: p[0] = FE_MAX_LIGHTS; break;
    case GL_MAX_CLIP_PLANES: p[0] = 6; break;
    case GL_MAX_TEXTURE_SIZE: p[0] = FE_MAX_TEXTURE_SIZE; break;
    case GL_MAX_3D_TEXTURE_SIZE: case GL_MAX_CUBE_MAP_TEXTURE_SIZE: p[0] = 0; break;
    case GL_MAX_PIXEL_MAP_TABLE: p[0] = 256; break;
    case GL_MAX_ATTRIB_STACK_DEPTH: case GL_MAX_CLIENT_ATTRIB_STACK_DEPTH: p[0] = 16; break;
    case GL_MAX_MODELVIEW_STACK_DEPTH: case GL_MAX_PROJECTION_STACK_DEPTH: case GL_MAX_TEXTURE_STACK_DEPTH:
        p[0] = FE_MAX_STACK;
        break;
    case GL_MAX_NAME_STACK_DEPTH: p[0] = 64; break;
    case GL_MAX_VIEWPORT_DIMS: p[0] = FE_MAX_FB_DIM; p[1] = FE_MAX_FB_DIM; break;
    case GL_MAX_TEXTURE_UNITS: p[0] = 1; break;
    case GL_MAX_ELEMENTS_VERTICES: case GL_MAX_ELEMENTS_INDICES: p[0] = 65536; break;
    case GL_SUBPIXEL_BITS: p[0] = 4; break;
    case GL_INDEX_BITS: p[0] = 0; break;
    case GL_RED_BITS: case GL_GREEN_BITS: case GL_BLUE_BITS: case GL_ALPHA_BITS: p[0] = 8; break;
    case GL_DEPTH_BITS: p[0] = 32; break;
    case GL_STENCIL_BITS: p[0] = 8; break;
    case GL_ACCUM_RED_BITS: case GL_ACCUM_GREEN_BITS: case GL_ACCUM_BLUE_BITS: case GL_ACCUM_ALPHA_BITS:
        p[0] = 0;
        break;
    case GL_AUX_BUFFERS: p[0] = 0; break;
    case GL_DOUBLEBUFFER: p[0] = GL_TRUE; break;
    case GL_STEREO: p[0] = GL_FALSE; break;
    case GL_RGBA_MODE: p[0] = GL_TRUE; break;
    case GL_INDEX_MODE: p[0] = GL_FALSE; break;
    case GL_SAMPLE_BUFFERS: case GL_SAMPLES: p[0] = 0; break;
    default: fe_set_error(c, GL_INVALID_ENUM); break;
    }
}

static void copy4(GLfloat *p, const float *v) { for (int i = 0; i < 4; i++) p[i] = v[i]; }

void glGetFloatv(GLenum pname, GLfloat *p)
{
    CHECK_CTX();
    if (!p) return;
    GLState *c = fe_ctx;
    switch (pname) {
    case GL_MODELVIEW_MATRIX: memcpy(p, c->mv[c->mv_depth], 16 * sizeof(float)); break;
    case GL_PROJECTION_MATRIX: memcpy(p, c->proj[c->proj_depth], 16 * sizeof(float)); break;
    case GL_TEXTURE_MATRIX: memcpy(p, c->texm[c->tex_depth], 16 * sizeof(float)); break;
    case GL_CURRENT_COLOR: case GL_CURRENT_RASTER_COLOR: copy4(p, c->cur_color); break;
    case GL_CURRENT_NORMAL: p[0] = c->cur_normal[0]; p[1] = c->cur_normal[1]; p[2] = c->cur_normal[2]; break;
    case GL_CURRENT_TEXTURE_COORDS: p[0] = c->cur_tex[0]; p[1] = c->cur_tex[1]; break;
    case GL_CURRENT_RASTER_POSITION:
        p[0] = (GLfloat)c->raster_x; p[1] = (GLfloat)c->raster_y; p[2] = 0.0f; p[3] = 1.0f;
        break;
    case GL_DEPTH_RANGE: p[0] = (GLfloat)c->depth_near; p[1] = (GLfloat)c->depth_far; break;
    case GL_VIEWPORT: for (int i = 0; i < 4; i++) p[i] = (GLfloat)c->viewport[i]; break;
    case GL_DEPTH_CLEAR_VALUE: p[0] = (GLfloat)c->clear_depth; break;
    case GL_COLOR_CLEAR_VALUE: copy4(p, c->clear_color); break;
    case GL_FOG_COLOR: copy4(p, c->fog_color); break;
    case GL_FOG_DENSITY: p[0] = c->fog_density; break;
    case GL_FOG_START: p[0] = c->fog_start; break;
    case GL_FOG_END: p[0] = c->fog_end; break;
    case GL_LIGHT_MODEL_AMBIENT: copy4(p, c->lit.model_ambient); break;
    case GL_ALPHA_TEST_REF: p[0] = c->alpha_ref; break;
    case GL_BLEND_COLOR: p[0] = p[1] = p[2] = p[3] = 0.0f; break;
    case GL_POINT_SIZE: p[0] = c->point_size; break;
    case GL_POINT_SIZE_RANGE: p[0] = 1.0f; p[1] = 64.0f; break;
    case GL_POINT_SIZE_GRANULARITY: p[0] = 1.0f; break;
    case GL_LINE_WIDTH: p[0] = c->line_width; break;
    case GL_LINE_WIDTH_RANGE: p[0] = 1.0f; p[1] = 16.0f; break;
    case GL_LINE_WIDTH_GRANULARITY: p[0] = 1.0f; break;
    case GL_POLYGON_OFFSET_FACTOR: case GL_POLYGON_OFFSET_UNITS: p[0] = 0.0f; break;
    case GL_TEXTURE_ENV_COLOR: copy4(p, c->tex_env_color); break;
    case GL_SCISSOR_BOX: for (int i = 0; i < 4; i++) p[i] = (GLfloat)c->scissor[i]; break;
    case GL_MAX_TEXTURE_LOD_BIAS: p[0] = 2.0f; break;
    default: {
        /* integer query, first value converted (gl_api.c:2977-2990) */
        GLint ip[4] = {0, 0, 0, 0};
        GLenum saved = c->error;
        c->error = GL_NO_ERROR;
        glGetIntegerv(pname, ip);
        if (c->error == GL_NO_ERROR) {
            p[0] = (GLfloat)ip[0];
            c->error = saved;
        } else {
            c->error = saved;
            fe_set_error(c, GL_INVALID_ENUM);
        }
        break;
    }
    }
}

void glGetDoublev(GLenum pname, GLdouble *p)
{
    CHECK_CTX();
    if (!p) return;
    GLfloat f[16];
    memset(f, 0, sizeof(f));
    glGetFloatv(pname, f);
    int n = 1;
    switch (pname) {
    case GL_MODELVIEW_MATRIX: case GL_PROJECTION_MATRIX: case GL_TEXTURE_MATRIX: n = 16; break;
    case GL_CURRENT_COLOR: case GL_CURRENT_RASTER_COLOR: case GL_CURRENT_RASTER_POSITION: case GL_VIEWPORT:
    case GL_SCISSOR_BOX: case GL_COLOR_CLEAR_VALUE: case GL_FOG_COLOR: case GL_LIGHT_MODEL_AMBIENT:
    case GL_BLEND_COLOR: case GL_TEXTURE_ENV_COLOR: case GL_COLOR_WRITEMASK:
        n = 4;
        break;
    case GL_CURRENT_NORMAL: n = 3; break;
    case GL_CURRENT_TEXTURE_COORDS: case GL_DEPTH_RANGE: case GL_POINT_SIZE_RANGE: case GL_LINE_WIDTH_RANGE:
    case GL_MAX_VIEWPORT_DIMS: case GL_POLYGON_MODE:
        n = 2;
        break;
    default: break;
    }
    for (int i = 0; i < n; i++) p[i] = (GLdouble)f[i];
}

static GLboolean flag_set(uint32_t f) { return (fe_ctx->flags & f) ? GL_TRUE : GL_FALSE; }

void glGetBooleanv(GLenum pname, GLboolean *p)
{
    CHECK_CTX();
    if (!p) return;
    GLState *c = fe_ctx;
    switch (pname) {
    case GL_DEPTH_TEST: p[0] = flag_set(F_DEPTH_TEST); return;
    case GL_CULL_FACE: p[0] = flag_set(F_CULL_FACE); return;
    case GL_BLEND: p[0] = flag_set(F_BLEND); return;
    case GL_TEXTURE_2D: p[0] = flag_set(F_TEXTURE_2D); return;
    case GL_LIGHTING: p[0] = flag_set(F_LIGHTING); return;
    case GL_FOG: p[0] = flag_set(F_FOG); return;
    case GL_NORMALIZE: p[0] = flag_set(F_NORMALIZE); return;
    case GL_COLOR_MATERIAL: p[0] = flag_set(F_COLOR_MATERIAL); return;
    case GL_ALPHA_TEST: p[0] = flag_set(F_ALPHA_TEST); return;
    case GL_SCISSOR_TEST: p[0] = flag_set(F_SCISSOR_TEST); return;
    case GL_STENCIL_TEST: p[0] = flag_set(F_STENCIL_TEST); return;
    case GL_DEPTH_WRITEMASK: p[0] = c->depth_mask; return;
    case GL_COLOR_WRITEMASK: for (int i = 0; i < 4; i++) p[i] = c->color_mask[i]; return;
    case GL_DOUBLEBUFFER: p[0] = GL_TRUE; return;
    case GL_STEREO: p[0] = GL_FALSE; return;
    case GL_RGBA_MODE: p[0] = GL_TRUE; return;
    case GL_INDEX_MODE: p[0] = GL_FALSE; return;
    case GL_CURRENT_RASTER_POSITION_VALID: p[0] = c->raster_valid; return;
    case GL_LIGHT_MODEL_LOCAL_VIEWER: p[0] = (GLboolean)c->lit.local_viewer; return;
    case GL_LIGHT_MODEL_TWO_SIDE: p[0] = (GLboolean)c->lit.two_side; return;
    case GL_VERTEX_ARRAY: p[0] = (c->client_state & CL_VERTEX) ? GL_TRUE : GL_FALSE; return;
    case GL_COLOR_ARRAY: p[0] = (c->client_state & CL_COLOR) ? GL_TRUE : GL_FALSE; return;
    case GL_NORMAL_ARRAY: p[0] = (c->client_state & CL_NORMAL) ? GL_TRUE : GL_FALSE; return;
    case GL_TEXTURE_COORD_ARRAY: p[0] = (c->client_state & CL_TEXCOORD) ? GL_TRUE : GL_FALSE; return;
    default: break;
    }
    if (pname >= GL_LIGHT0 && pname <= GL_LIGHT7) {
        p[0] = (GLboolean)c->lit.lights[pname - GL_LIGHT0].enabled;
        return;
    }
    GLint ip[16];
    memset(ip, 0, sizeof(ip));
    glGetIntegerv(pname, ip);
    p[0] = ip[0] != 0 ? GL_TRUE : GL_FALSE;
}

GLboolean glIsEnabled(GLenum cap)
{
    CHECK_CTX_RET(GL_FALSE);
    switch (cap) {
    case GL_DEPTH_TEST: return flag_set(F_DEPTH_TEST);
    case GL_CULL_FACE: return flag_set(F_CULL_FACE);
    case GL_BLEND: return flag_set(F_BLEND);
    case GL_TEXTURE_2D: return flag_set(F_TEXTURE_2D);
    case GL_LIGHTING: return flag_set(F_LIGHTING);
    case GL_FOG: return flag_set(F_FOG);
    case GL_NORMALIZE: return flag_set(F_NORMALIZE);
    case GL_COLOR_MATERIAL: return flag_set(F_COLOR_MATERIAL);
    case GL_ALPHA_TEST: return flag_set(F_ALPHA_TEST);
    case GL_SCISSOR_TEST: return flag_set(F_SCISSOR_TEST);
    case GL_STENCIL_TEST: return flag_set(F_STENCIL_TEST);
    default:
        if (cap >= GL_LIGHT0 && cap <= GL_LIGHT7) return (GLboolean)fe_ctx->lit.lights[cap - GL_LIGHT0].enabled;
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return GL_FALSE;
    }
}

const GLubyte *glGetString(GLenum name)
{
    CHECK_CTX_RET(NULL);
    switch (name) {
    case GL_VENDOR: return (const GLubyte *)"mytinygl-gb300";
    case GL_RENDERER: return (const GLubyte *)"MyTinyGL fixed-function pipeline on GB300 (sm_103a)";
    case GL_VERSION: return (const GLubyte *)"1.5 mytinygl-gb300";
    case GL_EXTENSIONS: return (const GLubyte *)"";
    default:
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return NULL;
    }
}

void glGetLightfv(GLenum light, GLenum pname, GLfloat *p)
{
    CHECK_CTX();
    if (!p) return;
    if (light < GL_LIGHT0 || light > GL_LIGHT7) {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    const mtgl_light *l = &fe_ctx->lit.lights[light - GL_LIGHT0];
    switch (pname) {
    case GL_AMBIENT: copy4(p, l->ambient); break;
    case GL_DIFFUSE: copy4(p, l->diffuse); break;
    case GL_SPECULAR: copy4(p, l->specular); break;
    case GL_POSITION: copy4(p, l->position); break;
    case GL_SPOT_DIRECTION: p[0] = l->spot_direction[0]; p[1] = l->spot_direction[1]; p[2] = l->spot_direction[2]; break;
    case GL_SPOT_EXPONENT: p[0] = l->spot_exponent; break;
    case GL_SPOT_CUTOFF: p[0] = l->spot_cutoff; break;
    case GL_CONSTANT_ATTENUATION: p[0] = l->constant_attenuation; break;
    case GL_LINEAR_ATTENUATION: p[0] = l->linear_attenuation; break;
    case GL_QUADRATIC_ATTENUATION: p[0] = l->quadratic_attenuation; break;
    default: fe_set_error(fe_ctx, GL_INVALID_ENUM); break;
    }
}

void glGetMaterialfv(GLenum face, GLenum pname, GLfloat *p)
{
    CHECK_CTX();
    if (!p) return;
    const mtgl_material *m;
    if (face == GL_FRONT) m = &fe_ctx->lit.front;
    else if (face == GL_BACK) m = &fe_ctx->lit.back;
    else {
        fe_set_error(fe_ctx, GL_INVALID_ENUM);
        return;
    }
    switch (pname) {
    case GL_AMBIENT: copy4(p, m->ambient); break;
    case GL_DIFFUSE: copy4(p, m->diffuse); break;
    case GL_SPECULAR: copy4(p, m->specular); break;
    case GL_EMISSION: copy4(p, m->emission); break;
    case GL_SHININESS: p[0] = m->shininess; break;
    default: fe_set_error(fe_ctx, GL_INVALID_ENUM); break;
    }
}
