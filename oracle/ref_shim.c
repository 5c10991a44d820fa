/*
 * ref_shim.c — TEST INFRASTRUCTURE ONLY. Compiled together with MyTinyGL's own sources
 * (oracle/Makefile, target `ref`) so the unmodified reference exposes the same
 * framebuffer-read entry points as libmytinygl_gb300.so (include/mytinygl/mytinygl.h).
 * It reads ctx->framebuffer (src/mytinygl.h:210, src/framebuffer.h:19-25) directly.
 */
#include <stdint.h>
#include <string.h>
#include "mytinygl.h"

int mtgl_finish(GLState *ctx) { return ctx ? 0 : 1; }

int mtgl_read_framebuffer(GLState *ctx, uint32_t *color, float *depth, uint8_t *stencil)
{
    if (!ctx) return 1;
    size_t n = (size_t)ctx->framebuffer.width * (size_t)ctx->framebuffer.height;
    if (color) memcpy(color, ctx->framebuffer.color, n * sizeof(uint32_t));
    if (depth) memcpy(depth, ctx->framebuffer.depth, n * sizeof(float));
    if (stencil) memcpy(stencil, ctx->framebuffer.stencil, n);
    return 0;
}

int mtgl_framebuffer_size(GLState *ctx, int32_t *w, int32_t *h)
{
    if (!ctx) return 1;
    if (w) *w = ctx->framebuffer.width;
    if (h) *h = ctx->framebuffer.height;
    return 0;
}

const uint32_t *mtgl_color_buffer(GLState *ctx) { return ctx ? ctx->framebuffer.color : 0; }

const char *mtgl_backend_name(void) { return "reference"; }

int mtgl_get_stats(GLState *ctx, void *out) { (void)ctx; (void)out; return 1; }
int mtgl_reset_stats(GLState *ctx) { (void)ctx; return 1; }
int mtgl_set_profiling(GLState *ctx, int enable) { (void)ctx; (void)enable; return 1; }
int mtgl_get_timings(GLState *ctx, void *out) { (void)ctx; (void)out; return 1; }
void *mtgl_cuda_stream(GLState *ctx) { (void)ctx; return 0; }
int mtgl_set_option(GLState *ctx, int option, int value) { (void)ctx; (void)option; (void)value; return 1; }
