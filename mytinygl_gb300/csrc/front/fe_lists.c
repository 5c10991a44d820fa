/*
 * fe_lists.c — display lists (gl_api.c:2268-2499, lists.c:14-425).
 *
 * Recording and replay follow the reference: the same 31 commands are recorded (calls
 * such as glClear, fog or glTexImage2D are not, and execute immediately even under
 * GL_COMPILE); replay re-issues the public entry points, so replayed geometry reaches the
 * device through the same immediate-mode path. Ids are allocated as contiguous ranges,
 * first-fit over freed slots, capped at 1024; nested glCallList stops at depth 64.
 *
 * Device-resident blocks: at glEndList the vertices of every glBegin/glEnd block whose
 * attributes do not depend on where in the block the caller's current values would show
 * (fe_list_block) are uploaded once into one device buffer per list, and glCallList draws
 * such a block from there (fe_draw_list_block) instead of re-emitting its vertices, which
 * would stage them from host memory again on every call. Everything else replays.
 */
#include "fe_internal.h"

fe_list *fe_list_get(GLState *c, GLuint id)
{
    if (id == 0 || id > c->list_count) return NULL;
    fe_list *l = &c->lists[id - 1];
    return l->allocated ? l : NULL;
}

/* drops the device-resident blocks of a list */
static void drop_blocks(GLState *c, fe_list *l)
{
    if (l->vb) (void)mtgl_dev_buffer_destroy(c->dev, l->vb);
    free(l->blocks);
    l->vb = 0;
    l->blocks = NULL;
    l->nblocks = 0;
}

/* a list slot back to its never-allocated state */
static void clear_list(GLState *c, fe_list *l)
{
    drop_blocks(c, l);
    free(l->cmds);
    memset(l, 0, sizeof(*l));
}

void fe_lists_free(GLState *c)
{
    for (size_t i = 0; i < c->list_count; i++) clear_list(c, &c->lists[i]);
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

/* Scans the block opened by the LC_BEGIN at `b`. Returns its vertex count, or 0 when it
 * cannot be device-resident: another command before LC_END, no LC_END, an invalid mode, no
 * vertex, or an attribute set after a vertex that took the caller's current value. With
 * `out`, writes the vertices (fe_vertex layout; attributes the block never sets are left
 * zero, the draw takes them from the current values; a block that turns out not to
 * qualify may have written some). Colours are stored as recorded:
 * LC_COLOR holds glColor's sanitised values, which replaying through glColor4f keeps. */
static uint32_t scan_block(const fe_list *l, size_t b, fe_list_block *blk, fe_vertex *out)
{
    const fe_list_cmd *cmd = l->cmds;
    const uint32_t attribs = CL_COLOR | CL_TEXCOORD | CL_NORMAL;
    uint32_t set = 0, inherited = 0, n = 0;
    fe_vertex cur;
    memset(&cur, 0, sizeof(cur));
    memset(blk, 0, sizeof(*blk));
    if (cmd[b].e[0] > GL_POLYGON) return 0;
    for (size_t i = b + 1; i < l->count; i++) {
        const fe_list_cmd *m = &cmd[i];
        switch (m->op) {
        case LC_VERTEX:
            if (n == UINT32_MAX / 2) return 0;
            inherited |= attribs & ~set;
            memcpy(cur.pos, m->f, sizeof(cur.pos));
            if (out) out[n] = cur;
            if (set & CL_COLOR) memcpy(blk->last_color, cur.color, sizeof(blk->last_color));
            n++;
            break;
        case LC_COLOR:
            if (inherited & CL_COLOR) return 0;
            set |= CL_COLOR;
            memcpy(cur.color, m->f, sizeof(cur.color));
            break;
        case LC_TEXCOORD:
            if (inherited & CL_TEXCOORD) return 0;
            set |= CL_TEXCOORD;
            memcpy(cur.tex, m->f, sizeof(cur.tex));
            break;
        case LC_NORMAL:
            if (inherited & CL_NORMAL) return 0;
            set |= CL_NORMAL;
            memcpy(cur.normal, m->f, sizeof(cur.normal));
            break;
        case LC_END:
            if (n == 0) return 0;
            blk->begin = b;
            blk->end = i;
            blk->mode = cmd[b].e[0];
            blk->count = n;
            blk->set = set;
            memcpy(blk->color, cur.color, sizeof(blk->color));
            memcpy(blk->tex, cur.tex, sizeof(blk->tex));
            memcpy(blk->normal, cur.normal, sizeof(blk->normal));
            return n;
        default:
            return 0;
        }
    }
    return 0;
}

/* glEndList: uploads the list's device-resident blocks (nothing on failure: they replay) */
static void build_blocks(GLState *c, fe_list *l)
{
    size_t nblocks = 0;
    uint64_t nverts = 0;
    fe_list_block blk;
    for (size_t i = 0; i < l->count; i++) {
        if (l->cmds[i].op != LC_BEGIN) continue;
        uint32_t n = scan_block(l, i, &blk, NULL);
        if (!n) continue;
        nblocks++;
        nverts += n;
        i = blk.end;
    }
    if (nblocks == 0 || nverts > (uint64_t)INT32_MAX) return;
    fe_list_block *blocks = (fe_list_block *)malloc(nblocks * sizeof(fe_list_block));
    fe_vertex *verts = (fe_vertex *)malloc((size_t)nverts * sizeof(fe_vertex));
    mtgl_handle vb = 0;
    if (blocks && verts) {
        size_t nb = 0;
        uint32_t first = 0;
        for (size_t i = 0; i < l->count; i++) {
            if (l->cmds[i].op != LC_BEGIN) continue;
            uint32_t n = scan_block(l, i, &blk, NULL);
            if (!n) continue;
            (void)scan_block(l, i, &blk, verts + first);
            blk.first = first;
            first += n;
            blocks[nb++] = blk;
            i = blk.end;
        }
        if (mtgl_dev_buffer_create(c->dev, &vb) != MTGL_OK) vb = 0;
        if (vb && mtgl_dev_buffer_data(c->dev, vb, verts, nverts * sizeof(fe_vertex)) != MTGL_OK) {
            (void)mtgl_dev_buffer_destroy(c->dev, vb);
            vb = 0;
        }
    }
    free(verts);
    if (!vb) {
        free(blocks);
        return;
    }
    l->vb = vb;
    l->blocks = blocks;
    l->nblocks = nblocks;
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
                    clear_list(c, l);
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
        clear_list(fe_ctx, l);
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
    drop_blocks(c, l);
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
    if (l) build_blocks(c, l);
}

/* execute_list (gl_api.c:2331-2439) */
static void execute_list(GLuint id)
{
    fe_list *l = fe_list_get(fe_ctx, id);
    if (!l || !l->valid) return;
    size_t k = 0;  /* next device-resident block */
    for (size_t i = 0; i < l->count; i++) {
        /* re-fetch each step: a replayed call may grow another list's storage */
        l = fe_list_get(fe_ctx, id);
        if (!l || i >= l->count) return;
        fe_list_cmd cmd = l->cmds[i];
        switch (cmd.op) {
        case LC_BEGIN:
            while (k < l->nblocks && l->blocks[k].begin < i) k++;
            if (k < l->nblocks && l->blocks[k].begin == i && fe_draw_list_block(fe_ctx, l->vb, &l->blocks[k])) {
                i = l->blocks[k].end;
                break;
            }
            glBegin(cmd.e[0]);
            break;
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
