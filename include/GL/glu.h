/*
 * glu.h — the GLU helpers MyTinyGL ships as static inline functions
 * (include/GL/glu.h:18-252), restated so programs written against the reference compile
 * unchanged. The arithmetic (double precision, then the float conversions at the GL
 * boundary) follows the reference so the resulting matrices are the same; gluUnProject
 * keeps the reference's model*proj multiplication order (glu.h:199).
 */
#ifndef MYTINYGL_GB300_GLU_H
#define MYTINYGL_GB300_GLU_H

#include "gl.h"
#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* C = A * B, column-major 4x4 in double precision. */
static inline void mtglu_mat4_mul(const GLdouble A[16], const GLdouble B[16], GLdouble C[16])
{
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            C[c * 4 + r] = A[0 * 4 + r] * B[c * 4 + 0] + A[1 * 4 + r] * B[c * 4 + 1] +
                           A[2 * 4 + r] * B[c * 4 + 2] + A[3 * 4 + r] * B[c * 4 + 3];
}

/* Gauss-Jordan inverse with partial pivoting on the column-major matrix; 0 if singular. */
static inline int mtglu_mat4_invert(const GLdouble src[16], GLdouble dst[16])
{
    GLdouble a[16], b[16];
    for (int i = 0; i < 16; i++) { a[i] = src[i]; b[i] = (i % 5 == 0) ? 1.0 : 0.0; }
    for (int col = 0; col < 4; col++) {
        int piv = col;
        GLdouble best = fabs(a[col * 4 + col]);
        for (int r = col + 1; r < 4; r++)
            if (fabs(a[col * 4 + r]) > best) { best = fabs(a[col * 4 + r]); piv = r; }
        if (best < 1e-12) return 0;
        if (piv != col)
            for (int k = 0; k < 4; k++) {
                GLdouble t = a[k * 4 + col]; a[k * 4 + col] = a[k * 4 + piv]; a[k * 4 + piv] = t;
                t = b[k * 4 + col]; b[k * 4 + col] = b[k * 4 + piv]; b[k * 4 + piv] = t;
            }
        GLdouble s = 1.0 / a[col * 4 + col];
        for (int k = 0; k < 4; k++) { a[k * 4 + col] *= s; b[k * 4 + col] *= s; }
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            GLdouble f = a[col * 4 + r];
            for (int k = 0; k < 4; k++) {
                a[k * 4 + r] -= f * a[k * 4 + col];
                b[k * 4 + r] -= f * b[k * 4 + col];
            }
        }
    }
    for (int i = 0; i < 16; i++) dst[i] = b[i];
    return 1;
}

static inline void mtglu_transform(const GLdouble m[16], const GLdouble v[4], GLdouble out[4])
{
    for (int r = 0; r < 4; r++)
        out[r] = m[r] * v[0] + m[4 + r] * v[1] + m[8 + r] * v[2] + m[12 + r] * v[3];
}

/* Symmetric perspective frustum (glu.h:114-119). */
static inline void gluPerspective(GLdouble fovy, GLdouble aspect, GLdouble zNear, GLdouble zFar)
{
    GLdouble h = zNear * tan(fovy * M_PI / 360.0);
    GLdouble w = h * aspect;
    glFrustum(-w, w, -h, h, zNear, zFar);
}

/* View matrix from eye, target and up (glu.h:125-158). */
static inline void gluLookAt(GLdouble ex, GLdouble ey, GLdouble ez, GLdouble tx, GLdouble ty, GLdouble tz,
                             GLdouble ux, GLdouble uy, GLdouble uz)
{
    GLdouble f[3] = {tx - ex, ty - ey, tz - ez};
    GLdouble fl = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (fl > 0.0) { f[0] /= fl; f[1] /= fl; f[2] /= fl; }
    GLdouble s[3] = {f[1] * uz - f[2] * uy, f[2] * ux - f[0] * uz, f[0] * uy - f[1] * ux};
    GLdouble sl = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    if (sl > 0.0) { s[0] /= sl; s[1] /= sl; s[2] /= sl; }
    GLdouble u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    GLfloat m[16] = {
        (GLfloat)s[0], (GLfloat)u[0], (GLfloat)(-f[0]), 0.0f,
        (GLfloat)s[1], (GLfloat)u[1], (GLfloat)(-f[1]), 0.0f,
        (GLfloat)s[2], (GLfloat)u[2], (GLfloat)(-f[2]), 0.0f,
        0.0f, 0.0f, 0.0f, 1.0f};
    glMultMatrixf(m);
    glTranslatef((GLfloat)(-ex), (GLfloat)(-ey), (GLfloat)(-ez));
}

static inline void gluOrtho2D(GLdouble left, GLdouble right, GLdouble bottom, GLdouble top)
{
    glOrtho(left, right, bottom, top, -1.0, 1.0);
}

/* Object -> window coordinates (glu.h:168-190). */
static inline GLint gluProject(GLdouble ox, GLdouble oy, GLdouble oz, const GLdouble model[16],
                               const GLdouble proj[16], const GLint viewport[4],
                               GLdouble *wx, GLdouble *wy, GLdouble *wz)
{
    GLdouble o[4] = {ox, oy, oz, 1.0}, e[4], c[4];
    mtglu_transform(model, o, e);
    mtglu_transform(proj, e, c);
    if (c[3] == 0.0) return GL_FALSE;
    GLdouble nx = c[0] / c[3], ny = c[1] / c[3], nz = c[2] / c[3];
    *wx = viewport[0] + viewport[2] * (nx + 1.0) * 0.5;
    *wy = viewport[1] + viewport[3] * (ny + 1.0) * 0.5;
    *wz = (nz + 1.0) * 0.5;
    return GL_TRUE;
}

/* Window -> object coordinates (glu.h:196-224), same multiplication order as the reference. */
static inline GLint gluUnProject(GLdouble wx, GLdouble wy, GLdouble wz, const GLdouble model[16],
                                 const GLdouble proj[16], const GLint viewport[4],
                                 GLdouble *ox, GLdouble *oy, GLdouble *oz)
{
    GLdouble m[16], inv[16];
    mtglu_mat4_mul(model, proj, m);
    if (!mtglu_mat4_invert(m, inv)) return GL_FALSE;
    GLdouble n[4] = {(wx - viewport[0]) / viewport[2] * 2.0 - 1.0,
                     (wy - viewport[1]) / viewport[3] * 2.0 - 1.0, wz * 2.0 - 1.0, 1.0};
    GLdouble o[4];
    mtglu_transform(inv, n, o);
    if (o[3] == 0.0) return GL_FALSE;
    *ox = o[0] / o[3];
    *oy = o[1] / o[3];
    *oz = o[2] / o[3];
    return GL_TRUE;
}

/* Picking region (glu.h:230-246). */
static inline void gluPickMatrix(GLdouble x, GLdouble y, GLdouble width, GLdouble height, const GLint viewport[4])
{
    if (width <= 0.0 || height <= 0.0) return;
    GLfloat tx = (GLfloat)((viewport[2] - 2.0 * (x - viewport[0])) / width);
    GLfloat ty = (GLfloat)((viewport[3] - 2.0 * (y - viewport[1])) / height);
    GLfloat sx = (GLfloat)(viewport[2] / width);
    GLfloat sy = (GLfloat)(viewport[3] / height);
    glTranslatef(tx, ty, 0.0f);
    glScalef(sx, sy, 1.0f);
}

#ifdef __cplusplus
}
#endif

#endif /* MYTINYGL_GB300_GLU_H */
