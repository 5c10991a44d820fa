/*
 * fe_matrix.c — matrix stacks (gl_api.c:483-611).
 *
 * Three 24-deep stacks; every operation post-multiplies the current matrix with the
 * reference's float mat4_mul and the reference's matrix builders (graphics.h:154-224), so
 * the matrices reaching the vertex kernel are bit-identical.
 */
#include "fe_internal.h"

static float *cur_matrix(GLState *c)
{
    switch (c->matrix_mode) {
    case GL_PROJECTION: return c->proj[c->proj_depth];
    case GL_TEXTURE: return c->texm[c->tex_depth];
    default: return c->mv[c->mv_depth];
    }
}

static GLint *cur_depth(GLState *c)
{
    switch (c->matrix_mode) {
    case GL_PROJECTION: return &c->proj_depth;
    case GL_TEXTURE: return &c->tex_depth;
    default: return &c->mv_depth;
    }
}

static void post_multiply(const float *m)
{
    float *cur = cur_matrix(fe_ctx);
    fe_mat4_mul(cur, m, cur);
    fe_state_changed(fe_ctx);
}

void glMatrixMode(GLenum mode)
{
    CHECK_CTX();
    if (fe_rec_e(LC_MATRIX_MODE, mode)) return;
    fe_ctx->matrix_mode = mode;
}

void glLoadIdentity(void)
{
    CHECK_CTX();
    if (fe_rec_op(LC_LOAD_IDENTITY)) return;
    fe_mat4_identity(cur_matrix(fe_ctx));
    fe_state_changed(fe_ctx);
}

void glPushMatrix(void)
{
    CHECK_CTX();
    if (fe_rec_op(LC_PUSH)) return;
    GLint *d = cur_depth(fe_ctx);
    if (*d >= FE_MAX_STACK - 1) {
        fe_set_error(fe_ctx, GL_STACK_OVERFLOW);
        return;
    }
    float tmp[16];
    memcpy(tmp, cur_matrix(fe_ctx), sizeof(tmp));
    (*d)++;
    memcpy(cur_matrix(fe_ctx), tmp, sizeof(tmp));
    fe_state_changed(fe_ctx);
}

void glPopMatrix(void)
{
    CHECK_CTX();
    if (fe_rec_op(LC_POP)) return;
    GLint *d = cur_depth(fe_ctx);
    if (*d <= 0) {
        fe_set_error(fe_ctx, GL_STACK_UNDERFLOW);
        return;
    }
    (*d)--;
    fe_state_changed(fe_ctx);
}

/* mat4_ortho (graphics.h:188-205): float parameters, identity when degenerate */
static void ortho_matrix(float l, float r, float b, float t, float n, float f, float *m)
{
    float rl = r - l, tb = t - b, fn = f - n;
    fe_mat4_identity(m);
    if (rl == 0.0f || tb == 0.0f || fn == 0.0f) return;
    m[0] = 2.0f / rl;
    m[5] = 2.0f / tb;
    m[10] = -2.0f / fn;
    m[12] = -(r + l) / rl;
    m[13] = -(t + b) / tb;
    m[14] = -(f + n) / fn;
}

/* mat4_frustum (graphics.h:207-224) */
static void frustum_matrix(float l, float r, float b, float t, float n, float f, float *m)
{
    float rl = r - l, tb = t - b, fn = f - n;
    fe_mat4_identity(m);
    if (rl == 0.0f || tb == 0.0f || fn == 0.0f) return;
    for (int i = 0; i < 16; i++) m[i] = 0.0f;
    m[0] = 2.0f * n / rl;
    m[5] = 2.0f * n / tb;
    m[8] = (r + l) / rl;
    m[9] = (t + b) / tb;
    m[10] = -(f + n) / fn;
    m[11] = -1.0f;
    m[14] = -2.0f * f * n / fn;
}

void glOrtho(GLdouble left, GLdouble right, GLdouble bottom, GLdouble top, GLdouble n, GLdouble f)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_ORTHO, {0, 0, 0}, 0, {0}, {left, right, bottom, top, n, f}};
    if (fe_rec(&cmd)) return;
    float m[16];
    ortho_matrix((float)left, (float)right, (float)bottom, (float)top, (float)n, (float)f, m);
    post_multiply(m);
}

void glFrustum(GLdouble left, GLdouble right, GLdouble bottom, GLdouble top, GLdouble n, GLdouble f)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_FRUSTUM, {0, 0, 0}, 0, {0}, {left, right, bottom, top, n, f}};
    if (fe_rec(&cmd)) return;
    float m[16];
    frustum_matrix((float)left, (float)right, (float)bottom, (float)top, (float)n, (float)f, m);
    post_multiply(m);
}

void glTranslatef(GLfloat x, GLfloat y, GLfloat z)
{
    CHECK_CTX();
    if (fe_rec_f3(LC_TRANSLATE, x, y, z)) return;
    float m[16];
    fe_mat4_identity(m);
    m[12] = x; m[13] = y; m[14] = z;
    post_multiply(m);
}

/* mat4_rotate (graphics.h:172-186) */
void glRotatef(GLfloat angle, GLfloat x, GLfloat y, GLfloat z)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_ROTATE, {0, 0, 0}, 0, {angle, x, y, z}, {0}};
    if (fe_rec(&cmd)) return;
    float m[16];
    float rad = angle * 3.14159265358979f / 180.0f;
    float c = cosf(rad);
    float s = sinf(rad);
    float len = sqrtf(x * x + y * y + z * z);
    fe_mat4_identity(m);
    if (len != 0) {
        x /= len; y /= len; z /= len;
        m[0] = x * x * (1 - c) + c;  m[1] = y * x * (1 - c) + z * s; m[2] = x * z * (1 - c) - y * s; m[3] = 0;
        m[4] = x * y * (1 - c) - z * s; m[5] = y * y * (1 - c) + c;  m[6] = y * z * (1 - c) + x * s; m[7] = 0;
        m[8] = x * z * (1 - c) + y * s; m[9] = y * z * (1 - c) - x * s; m[10] = z * z * (1 - c) + c; m[11] = 0;
        m[12] = 0; m[13] = 0; m[14] = 0; m[15] = 1;
    }
    post_multiply(m);
}

void glScalef(GLfloat x, GLfloat y, GLfloat z)
{
    CHECK_CTX();
    if (fe_rec_f3(LC_SCALE, x, y, z)) return;
    float m[16];
    fe_mat4_identity(m);
    m[0] = x; m[5] = y; m[10] = z;
    post_multiply(m);
}

void glMultMatrixf(const GLfloat *mult)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_MULT_MATRIX, {0, 0, 0}, 0, {0}, {0}};
    memcpy(cmd.f, mult, sizeof(cmd.f));
    if (fe_rec(&cmd)) return;
    float m[16];
    memcpy(m, mult, sizeof(m));
    post_multiply(m);
}

void glLoadMatrixf(const GLfloat *m)
{
    CHECK_CTX();
    fe_list_cmd cmd = {LC_LOAD_MATRIX, {0, 0, 0}, 0, {0}, {0}};
    memcpy(cmd.f, m, sizeof(cmd.f));
    if (fe_rec(&cmd)) return;
    memcpy(cur_matrix(fe_ctx), m, 16 * sizeof(float));
    fe_state_changed(fe_ctx);
}
