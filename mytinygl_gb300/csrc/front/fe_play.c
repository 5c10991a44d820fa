/* fe_play.c — GENERATED by mytinygl_gb300/gen_play.py from include/GL/gl.h; do not edit.
 *
 * Native player of GL command streams (no counterpart in the reference). A stream is a
 * sequence of records: u32 function id (index of the entry point in sorted name order),
 * u32 argument count, then one 8-byte slot per argument: int64 for integers, enums and
 * pointers, IEEE double for GLfloat/GLdouble arguments. Playing a stream calls the same
 * public entry points an application would, in order, on the given context. */
#include <stdint.h>
#include <stddef.h>
#include <string.h>

#include "GL/gl.h"
#include "mytinygl/mytinygl.h"

typedef union {
    int64_t i;
    double f;
} play_arg;

#define PLAY_FUNCTIONS 111

static const uint8_t k_play_nargs[PLAY_FUNCTIONS] = {
    2, 1, 2, 2, 2, 4, 4, 1, 3, 1, 4, 1, 1, 3, 3, 4, 4, 4, 2, 4, 1, 2, 2, 2,
    1, 1, 2, 1, 1, 3, 4, 5, 1, 1, 0, 0, 0, 0, 2, 2, 2, 1, 6, 2, 1, 2, 2, 2,
    0, 2, 2, 3, 3, 1, 2, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 1, 1, 0, 1, 3,
    3, 3, 3, 1, 1, 2, 3, 3, 6, 2, 1, 2, 0, 0, 2, 2, 3, 7, 4, 3, 4, 1, 3, 1,
    3, 2, 4, 3, 3, 3, 9, 3, 3, 2, 2, 3, 3, 4, 4,
};

static void play_call(uint32_t fid, const play_arg *a)
{
    switch (fid) {
    case 0: (void)glAlphaFunc((GLenum)a[0].i, (GLclampf)a[1].f); break;
    case 1: (void)glBegin((GLenum)a[0].i); break;
    case 2: (void)glBindBuffer((GLenum)a[0].i, (GLuint)a[1].i); break;
    case 3: (void)glBindTexture((GLenum)a[0].i, (GLuint)a[1].i); break;
    case 4: (void)glBlendFunc((GLenum)a[0].i, (GLenum)a[1].i); break;
    case 5: (void)glBufferData((GLenum)a[0].i, (GLsizeiptr)a[1].i, (const GLvoid *)(uintptr_t)a[2].i, (GLenum)a[3].i); break;
    case 6: (void)glBufferSubData((GLenum)a[0].i, (GLintptr)a[1].i, (GLsizeiptr)a[2].i, (const GLvoid *)(uintptr_t)a[3].i); break;
    case 7: (void)glCallList((GLuint)a[0].i); break;
    case 8: (void)glCallLists((GLsizei)a[0].i, (GLenum)a[1].i, (const GLvoid *)(uintptr_t)a[2].i); break;
    case 9: (void)glClear((GLbitfield)a[0].i); break;
    case 10: (void)glClearColor((GLclampf)a[0].f, (GLclampf)a[1].f, (GLclampf)a[2].f, (GLclampf)a[3].f); break;
    case 11: (void)glClearDepth((GLclampd)a[0].f); break;
    case 12: (void)glClearStencil((GLint)a[0].i); break;
    case 13: (void)glColor3f((GLfloat)a[0].f, (GLfloat)a[1].f, (GLfloat)a[2].f); break;
    case 14: (void)glColor3ub((GLubyte)a[0].i, (GLubyte)a[1].i, (GLubyte)a[2].i); break;
    case 15: (void)glColor4f((GLfloat)a[0].f, (GLfloat)a[1].f, (GLfloat)a[2].f, (GLfloat)a[3].f); break;
    case 16: (void)glColor4ub((GLubyte)a[0].i, (GLubyte)a[1].i, (GLubyte)a[2].i, (GLubyte)a[3].i); break;
    case 17: (void)glColorMask((GLboolean)a[0].i, (GLboolean)a[1].i, (GLboolean)a[2].i, (GLboolean)a[3].i); break;
    case 18: (void)glColorMaterial((GLenum)a[0].i, (GLenum)a[1].i); break;
    case 19: (void)glColorPointer((GLint)a[0].i, (GLenum)a[1].i, (GLsizei)a[2].i, (const GLvoid *)(uintptr_t)a[3].i); break;
    case 20: (void)glCullFace((GLenum)a[0].i); break;
    case 21: (void)glDeleteBuffers((GLsizei)a[0].i, (const GLuint *)(uintptr_t)a[1].i); break;
    case 22: (void)glDeleteLists((GLuint)a[0].i, (GLsizei)a[1].i); break;
    case 23: (void)glDeleteTextures((GLsizei)a[0].i, (const GLuint *)(uintptr_t)a[1].i); break;
    case 24: (void)glDepthFunc((GLenum)a[0].i); break;
    case 25: (void)glDepthMask((GLboolean)a[0].i); break;
    case 26: (void)glDepthRange((GLclampd)a[0].f, (GLclampd)a[1].f); break;
    case 27: (void)glDisable((GLenum)a[0].i); break;
    case 28: (void)glDisableClientState((GLenum)a[0].i); break;
    case 29: (void)glDrawArrays((GLenum)a[0].i, (GLint)a[1].i, (GLsizei)a[2].i); break;
    case 30: (void)glDrawElements((GLenum)a[0].i, (GLsizei)a[1].i, (GLenum)a[2].i, (const GLvoid *)(uintptr_t)a[3].i); break;
    case 31: (void)glDrawPixels((GLsizei)a[0].i, (GLsizei)a[1].i, (GLenum)a[2].i, (GLenum)a[3].i, (const GLvoid *)(uintptr_t)a[4].i); break;
    case 32: (void)glEnable((GLenum)a[0].i); break;
    case 33: (void)glEnableClientState((GLenum)a[0].i); break;
    case 34: (void)glEnd(); break;
    case 35: (void)glEndList(); break;
    case 36: (void)glFinish(); break;
    case 37: (void)glFlush(); break;
    case 38: (void)glFogf((GLenum)a[0].i, (GLfloat)a[1].f); break;
    case 39: (void)glFogfv((GLenum)a[0].i, (const GLfloat *)(uintptr_t)a[1].i); break;
    case 40: (void)glFogi((GLenum)a[0].i, (GLint)a[1].i); break;
    case 41: (void)glFrontFace((GLenum)a[0].i); break;
    case 42: (void)glFrustum((GLdouble)a[0].f, (GLdouble)a[1].f, (GLdouble)a[2].f, (GLdouble)a[3].f, (GLdouble)a[4].f, (GLdouble)a[5].f); break;
    case 43: (void)glGenBuffers((GLsizei)a[0].i, (GLuint *)(uintptr_t)a[1].i); break;
    case 44: (void)glGenLists((GLsizei)a[0].i); break;
    case 45: (void)glGenTextures((GLsizei)a[0].i, (GLuint *)(uintptr_t)a[1].i); break;
    case 46: (void)glGetBooleanv((GLenum)a[0].i, (GLboolean *)(uintptr_t)a[1].i); break;
    case 47: (void)glGetDoublev((GLenum)a[0].i, (GLdouble *)(uintptr_t)a[1].i); break;
    case 48: (void)glGetError(); break;
    case 49: (void)glGetFloatv((GLenum)a[0].i, (GLfloat *)(uintptr_t)a[1].i); break;
    case 50: (void)glGetIntegerv((GLenum)a[0].i, (GLint *)(uintptr_t)a[1].i); break;
    case 51: (void)glGetLightfv((GLenum)a[0].i, (GLenum)a[1].i, (GLfloat *)(uintptr_t)a[2].i); break;
    case 52: (void)glGetMaterialfv((GLenum)a[0].i, (GLenum)a[1].i, (GLfloat *)(uintptr_t)a[2].i); break;
    case 53: (void)glGetString((GLenum)a[0].i); break;
    case 54: (void)glHint((GLenum)a[0].i, (GLenum)a[1].i); break;
    case 55: (void)glIsBuffer((GLuint)a[0].i); break;
    case 56: (void)glIsEnabled((GLenum)a[0].i); break;
    case 57: (void)glIsList((GLuint)a[0].i); break;
    case 58: (void)glIsTexture((GLuint)a[0].i); break;
    case 59: (void)glLightModelf((GLenum)a[0].i, (GLfloat)a[1].f); break;
    case 60: (void)glLightModelfv((GLenum)a[0].i, (const GLfloat *)(uintptr_t)a[1].i); break;
    case 61: (void)glLightModeli((GLenum)a[0].i, (GLint)a[1].i); break;
    case 62: (void)glLightModeliv((GLenum)a[0].i, (const GLint *)(uintptr_t)a[1].i); break;
    case 63: (void)glLightf((GLenum)a[0].i, (GLenum)a[1].i, (GLfloat)a[2].f); break;
    case 64: (void)glLightfv((GLenum)a[0].i, (GLenum)a[1].i, (const GLfloat *)(uintptr_t)a[2].i); break;
    case 65: (void)glLighti((GLenum)a[0].i, (GLenum)a[1].i, (GLint)a[2].i); break;
    case 66: (void)glLightiv((GLenum)a[0].i, (GLenum)a[1].i, (const GLint *)(uintptr_t)a[2].i); break;
    case 67: (void)glLineWidth((GLfloat)a[0].f); break;
    case 68: (void)glListBase((GLuint)a[0].i); break;
    case 69: (void)glLoadIdentity(); break;
    case 70: (void)glLoadMatrixf((const GLfloat *)(uintptr_t)a[0].i); break;
    case 71: (void)glMaterialf((GLenum)a[0].i, (GLenum)a[1].i, (GLfloat)a[2].f); break;
    case 72: (void)glMaterialfv((GLenum)a[0].i, (GLenum)a[1].i, (const GLfloat *)(uintptr_t)a[2].i); break;
    case 73: (void)glMateriali((GLenum)a[0].i, (GLenum)a[1].i, (GLint)a[2].i); break;
    case 74: (void)glMaterialiv((GLenum)a[0].i, (GLenum)a[1].i, (const GLint *)(uintptr_t)a[2].i); break;
    case 75: (void)glMatrixMode((GLenum)a[0].i); break;
    case 76: (void)glMultMatrixf((const GLfloat *)(uintptr_t)a[0].i); break;
    case 77: (void)glNewList((GLuint)a[0].i, (GLenum)a[1].i); break;
    case 78: (void)glNormal3f((GLfloat)a[0].f, (GLfloat)a[1].f, (GLfloat)a[2].f); break;
    case 79: (void)glNormalPointer((GLenum)a[0].i, (GLsizei)a[1].i, (const GLvoid *)(uintptr_t)a[2].i); break;
    case 80: (void)glOrtho((GLdouble)a[0].f, (GLdouble)a[1].f, (GLdouble)a[2].f, (GLdouble)a[3].f, (GLdouble)a[4].f, (GLdouble)a[5].f); break;
    case 81: (void)glPixelStorei((GLenum)a[0].i, (GLint)a[1].i); break;
    case 82: (void)glPointSize((GLfloat)a[0].f); break;
    case 83: (void)glPolygonMode((GLenum)a[0].i, (GLenum)a[1].i); break;
    case 84: (void)glPopMatrix(); break;
    case 85: (void)glPushMatrix(); break;
    case 86: (void)glRasterPos2f((GLfloat)a[0].f, (GLfloat)a[1].f); break;
    case 87: (void)glRasterPos2i((GLint)a[0].i, (GLint)a[1].i); break;
    case 88: (void)glRasterPos3f((GLfloat)a[0].f, (GLfloat)a[1].f, (GLfloat)a[2].f); break;
    case 89: (void)glReadPixels((GLint)a[0].i, (GLint)a[1].i, (GLsizei)a[2].i, (GLsizei)a[3].i, (GLenum)a[4].i, (GLenum)a[5].i, (GLvoid *)(uintptr_t)a[6].i); break;
    case 90: (void)glRotatef((GLfloat)a[0].f, (GLfloat)a[1].f, (GLfloat)a[2].f, (GLfloat)a[3].f); break;
    case 91: (void)glScalef((GLfloat)a[0].f, (GLfloat)a[1].f, (GLfloat)a[2].f); break;
    case 92: (void)glScissor((GLint)a[0].i, (GLint)a[1].i, (GLsizei)a[2].i, (GLsizei)a[3].i); break;
    case 93: (void)glShadeModel((GLenum)a[0].i); break;
    case 94: (void)glStencilFunc((GLenum)a[0].i, (GLint)a[1].i, (GLuint)a[2].i); break;
    case 95: (void)glStencilMask((GLuint)a[0].i); break;
    case 96: (void)glStencilOp((GLenum)a[0].i, (GLenum)a[1].i, (GLenum)a[2].i); break;
    case 97: (void)glTexCoord2f((GLfloat)a[0].f, (GLfloat)a[1].f); break;
    case 98: (void)glTexCoordPointer((GLint)a[0].i, (GLenum)a[1].i, (GLsizei)a[2].i, (const GLvoid *)(uintptr_t)a[3].i); break;
    case 99: (void)glTexEnvf((GLenum)a[0].i, (GLenum)a[1].i, (GLfloat)a[2].f); break;
    case 100: (void)glTexEnvfv((GLenum)a[0].i, (GLenum)a[1].i, (const GLfloat *)(uintptr_t)a[2].i); break;
    case 101: (void)glTexEnvi((GLenum)a[0].i, (GLenum)a[1].i, (GLint)a[2].i); break;
    case 102: (void)glTexImage2D((GLenum)a[0].i, (GLint)a[1].i, (GLint)a[2].i, (GLsizei)a[3].i, (GLsizei)a[4].i, (GLint)a[5].i, (GLenum)a[6].i, (GLenum)a[7].i, (const GLvoid *)(uintptr_t)a[8].i); break;
    case 103: (void)glTexParameteri((GLenum)a[0].i, (GLenum)a[1].i, (GLint)a[2].i); break;
    case 104: (void)glTranslatef((GLfloat)a[0].f, (GLfloat)a[1].f, (GLfloat)a[2].f); break;
    case 105: (void)glVertex2f((GLfloat)a[0].f, (GLfloat)a[1].f); break;
    case 106: (void)glVertex2i((GLint)a[0].i, (GLint)a[1].i); break;
    case 107: (void)glVertex3f((GLfloat)a[0].f, (GLfloat)a[1].f, (GLfloat)a[2].f); break;
    case 108: (void)glVertex3i((GLint)a[0].i, (GLint)a[1].i, (GLint)a[2].i); break;
    case 109: (void)glVertexPointer((GLint)a[0].i, (GLenum)a[1].i, (GLsizei)a[2].i, (const GLvoid *)(uintptr_t)a[3].i); break;
    case 110: (void)glViewport((GLint)a[0].i, (GLint)a[1].i, (GLsizei)a[2].i, (GLsizei)a[3].i); break;
    default: break;
    }
}

int mtgl_play_function_count(void) { return PLAY_FUNCTIONS; }

int mtgl_play(GLState *ctx, const void *stream, size_t bytes)
{
    const uint8_t *p = (const uint8_t *)stream;
    size_t at = 0;
    if (!ctx || (bytes && !stream)) return MTGL_ERR_INVALID;
    gl_make_current(ctx);
    while (at < bytes) {
        uint32_t hdr[2];
        play_arg a[16];
        if (bytes - at < sizeof(hdr)) return MTGL_ERR_INVALID;
        memcpy(hdr, p + at, sizeof(hdr));
        at += sizeof(hdr);
        if (hdr[0] >= PLAY_FUNCTIONS || hdr[1] != k_play_nargs[hdr[0]] || hdr[1] > 16) return MTGL_ERR_INVALID;
        if (bytes - at < (size_t)hdr[1] * 8u) return MTGL_ERR_INVALID;
        memcpy(a, p + at, (size_t)hdr[1] * 8u);
        at += (size_t)hdr[1] * 8u;
        play_call(hdr[0], a);
    }
    return MTGL_OK;
}
