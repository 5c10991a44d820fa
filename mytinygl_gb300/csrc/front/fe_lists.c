/*
 * fe_lists.c — display lists (gl_api.c:2268-2499, lists.c:14-425).
 *
 * Recording and replay follow the reference: the same 31 commands are recorded (calls
 * such as glClear, fog or glTexImage2D are not, and execute immediately even under
 * GL_COMPILE); replay re-issues the public entry points, so replayed geometry reaches the
 * device through the same immediate-mode path. Ids are allocated as contiguous ranges,
 * first-fit over freed slots, capped at 1024; nested glCallList stops at depth 64.
 */
#include "fe_internal.h"

fe_list *fe_list_get(GLState *c, GLuint id)
{
    if (id == 0 || id > c->list_count) return NULL;
    fe_list *l = &c->lists[id - 1];
    return l->allocated ? l : NULL;
}

void fe_lists_free(GLState *c)
{
    for (size_t i = 0; i < c->list_count; i++) free(c->lists[i].cmds);
    free(c->lists);
    c->lists = NULL;
    c->list_count = c->list_cap = 0;
}

/* record_cmd (lists.c:185-197) */
int fe_rec(fe_list_cmd *cmd)
{
    GLState *c = fe_ctx;
    if (!c || c->list_index == 0) return 0;
    fe_list *l = fe_list_get(c, c->list_index);
    if (l) {
        if (l->count == l->cap) {
            size_t cap = l->cap ? l->cap * 2 : 64;
            fe_list_cmd *n = (fe_list_cmd *)realloc(l->cmds, cap * sizeof(fe_list_cmd));
            if (n) {
                l->cmds = n;
                l->cap = cap;
            }
        }
        if (l->count < l->cap) l->cmds[l->count++] = *cmd;
    }
    return c->list_mode == GL_COMPILE;
}

int fe_rec_op(fe_list_op op)
{
    if (!fe_ctx || fe_ctx->list_index == 0) return 0;
    fe_list_cmd cmd;
    memset(&cmd, 0, sizeof(cmd));
    cmd.op = op;
    return fe_rec(&cmd);
}

int fe_rec_e(fe_list_op op, GLenum a)
{
    if (!fe_ctx || fe_ctx->list_index == 0) return 0;
    fe_list_cmd cmd;
    memset(&cmd, 0, sizeof(cmd));
    cmd.op = op;
    cmd.e[0] = a;
    return fe_rec(&cmd);
}

int fe_rec_f3(fe_list_op op, float x, float y, float z)
{
    if (!fe_ctx || fe_ctx->list_index == 0) return 0;
    fe_list_cmd cmd;
    memset(&cmd, 0, sizeof(cmd));
    cmd.op = op;
    cmd.f[0] = x;
    cmd.f[1] = y;
    cmd.f[2] = z;
    return fe_rec(&cmd);
}

/* list_alloc_range (lists.c:59-120) */
GLuint glGenLists(GLsizei range)
{
    CHECK_CTX_RET(0);
    GLState *c = fe_ctx;
    if (range < 0) {
        fe_set_error(c, GL_INVALID_VALUE);
        return 0;
    }
    if (range == 0) return 0;
    /* first contiguous run of freed slots */
    size_t run = 0, start = 0;
    for (size_t i = 0; i < c->list_count; i++) {
        if (!c->lists[i].allocated) {
            if (run == 0) start = i;
            if (++run >= (size_t)range) {
                for (GLsizei k = 0; k < range; k++) {
                    fe_list *l = &c->lists[start + k];
                    free(l->cmds);
                    memset(l, 0, sizeof(*l));
                    l->allocated = 1;
                }
                return (GLuint)(start + 1);
            }
        } else {
            run = 0;
        }
    }
    if (c->list_count + (size_t)range > FE_MAX_LISTS) return 0;
    if (c->list_count + (size_t)range > c->list_cap) {
        size_t cap = c->list_cap ? c->list_cap * 2 : 16;
        while (cap < c->list_count + (size_t)range) cap *= 2;
        if (cap > FE_MAX_LISTS) cap = FE_MAX_LISTS;
        fe_list *n = (fe_list *)realloc(c->lists, cap * sizeof(fe_list));
        if (!n) return 0;
        memset(n + c->list_cap, 0, (cap - c->list_cap) * sizeof(fe_list));
        c->lists = n;
        c->list_cap = cap;
    }
    GLuint first = (GLuint)(c->list_count + 1);
    for (GLsizei k = 0; k < range; k++) {
        fe_list *l = &c->lists[c->list_count + k];
        memset(l, 0, sizeof(*l));
        l->allocated = 1;
    }
    c->list_count += (size_t)range;
    return first;
}

void glDeleteLists(GLuint list, GLsizei range)
{
    CHECK_CTX();
    if (range < 0) {
        fe_set_error(fe_ctx, GL_INVALID_VALUE);
        return;
    }
    for (GLsizei i = 0; i < range; i++) {
        fe_list *l = fe_list_get(fe_ctx, list + (GLuint)i);
        if (!l) continue;
        free(l->cmds);
        memset(l, 0, sizeof(*l));
    }
}

void glNewList(GLuint list, GLenum mode)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (c->list_index != 0) {
        fe_set_error(c, GL_INVALID_OPERATION);
        return;
    }
    if (mode != GL_COMPILE && mode != GL_COMPILE_AND_EXECUTE) {
        fe_set_error(c, GL_INVALID_ENUM);
        return;
    }
    fe_list *l = fe_list_get(c, list);
    if (!l) {
        fe_set_error(c, GL_INVALID_VALUE);
        return;
    }
    l->count = 0;
    l->valid = 0;
    c->list_index = list;
    c->list_mode = mode;
}

void glEndList(void)
{
    CHECK_CTX();
    GLState *c = fe_ctx;
    if (c->list_index == 0) {
        fe_set_error(c, GL_INVALID_OPERATION);
        return;
    }
    fe_list *l = fe_list_get(c, c->list_index);
    if (l) l->valid = 1;
    c->list_index = 0;
    c->list_mode = 0;
}

/* execute_list (gl_api.c:2331-2439) */
static void execute_list(GLuint id)
{
    fe_list *l = fe_list_get(fe_ctx, id);
    if (!l || !l->valid) return;
    for (size_t i = 0; i < l->count; i++) {
        /* re-fetch each step: a replayed call may grow another list's storage */
        l = fe_list_get(fe_ctx, id);
        if (!l || i >= l->count) return;
        fe_list_cmd cmd = l->cmds[i];
        switch (cmd.op) {
        case LC_BEGIN: glBegin(cmd.e[0]); break;
        case LC_END: glEnd(); break;
        case LC_VERTEX: glVertex3f(cmd.f[0], cmd.f[1], cmd.f[2]); break;
        case LC_COLOR: glColor4f(cmd.f[0], cmd.f[1], cmd.f[2], cmd.f[3]); break;
        case LC_TEXCOORD: glTexCoord2f(cmd.f[0], cmd.f[1]); break;
        case LC_NORMAL: glNormal3f(cmd.f[0], cmd.f[1], cmd.f[2]); break;
        case LC_TRANSLATE: glTranslatef(cmd.f[0], cmd.f[1], cmd.f[2]); break;
        case LC_ROTATE: glRotatef(cmd.f[0], cmd.f[1], cmd.f[2], cmd.f[3]); break;
        case LC_SCALE: glScalef(cmd.f[0], cmd.f[1], cmd.f[2]); break;
        case LC_PUSH: glPushMatrix(); break;
        case LC_POP: glPopMatrix(); break;
        case LC_LOAD_IDENTITY: glLoadIdentity(); break;
        case LC_MULT_MATRIX: glMultMatrixf(cmd.f); break;
        case LC_LOAD_MATRIX: glLoadMatrixf(cmd.f); break;
        case LC_MATRIX_MODE: glMatrixMode(cmd.e[0]); break;
        case LC_ENABLE: glEnable(cmd.e[0]); break;
        case LC_DISABLE: glDisable(cmd.e[0]); break;
        case LC_BIND_TEXTURE: glBindTexture(cmd.e[0], cmd.u); break;
        case LC_BLEND_FUNC: glBlendFunc(cmd.e[0], cmd.e[1]); break;
        case LC_DEPTH_FUNC: glDepthFunc(cmd.e[0]); break;
        case LC_DEPTH_MASK: glDepthMask((GLboolean)cmd.e[0]); break;
        case LC_CULL_FACE: glCullFace(cmd.e[0]); break;
        case LC_FRONT_FACE: glFrontFace(cmd.e[0]); break;
        case LC_SHADE_MODEL: glShadeModel(cmd.e[0]); break;
        case LC_LIGHTF: glLightf(cmd.e[0], cmd.e[1], cmd.f[0]); break;
        case LC_LIGHTFV: glLightfv(cmd.e[0], cmd.e[1], cmd.f); break;
        case LC_MATERIALF: glMaterialf(cmd.e[0], cmd.e[1], cmd.f[0]); break;
        case LC_MATERIALFV: glMaterialfv(cmd.e[0], cmd.e[1], cmd.f); break;
        case LC_CALL_LIST: glCallList(cmd.u); break;
        case LC_ORTHO: glOrtho(cmd.d[0], cmd.d[1], cmd.d[2], cmd.d[3], cmd.d[4], cmd.d[5]); break;
        case LC_FRUSTUM: glFrustum(cmd.d[0], cmd.d[1], cmd.d[2], cmd.d[3], cmd.d[4], cmd.d[5]); break;
        }
    }
}

void glCallList(GLuint list)
{
    CHECK_CTX();
    fe_list_cmd cmd;
    memset(&cmd, 0, sizeof(cmd));
    cmd.op = LC_CALL_LIST;
    cmd.u = list;
    if (fe_rec(&cmd)) return;
    if (fe_ctx->list_call_depth >= FE_MAX_CALL_DEPTH) {
        fe_set_error(fe_ctx, GL_STACK_OVERFLOW);
        return;
    }
    fe_ctx->list_call_depth++;
    execute_list(list);
    fe_ctx->list_call_depth--;
}

void glCallLists(GLsizei n, GLenum type, const GLvoid *lists)
{
    CHECK_CTX();
    if (n < 0) {
        fe_set_error(fe_ctx, GL_INVALID_VALUE);
        return;
    }
    for (GLsizei i = 0; i < n; i++) {
        GLuint off;
        switch (type) {
        case GL_UNSIGNED_BYTE: off = ((const GLubyte *)lists)[i]; break;
        case GL_UNSIGNED_SHORT: off = ((const GLushort *)lists)[i]; break;
        case GL_UNSIGNED_INT: off = ((const GLuint *)lists)[i]; break;
        default:
            fe_set_error(fe_ctx, GL_INVALID_ENUM);
            return;
        }
        glCallList(fe_ctx->list_base + off);
    }
}

void glListBase(GLuint base)
{
    CHECK_CTX();
    fe_ctx->list_base = base;
}

GLboolean glIsList(GLuint list)
{
    CHECK_CTX_RET(GL_FALSE);
    fe_list *l = fe_list_get(fe_ctx, list);
    return (l && l->valid) ? GL_TRUE : GL_FALSE;
}
