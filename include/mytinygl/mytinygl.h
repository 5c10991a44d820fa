/*
 * mytinygl.h — context API of the GB300 back end.
 *
 * The first four functions replace MyTinyGL's context API one for one
 * (src/mytinygl.h:228-233): one current context per OS thread, created headless.
 * The mtgl_* functions replace direct access to ctx->framebuffer
 * (framebuffer_get_color_buffer, src/framebuffer.h:137, as used by
 * include/mytinygl/sdl.h:76-80): the framebuffer lives in device memory, so reading
 * it is an explicit, synchronising call.
 */
#ifndef MYTINYGL_GB300_CONTEXT_H
#define MYTINYGL_GB300_CONTEXT_H

#include <stdint.h>
#include "GL/gl.h"
#include "mytinygl/mtgl_dev.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct GLState GLState;

/* gl_create_context (gl_api.c:81): width/height in 1..16384; NULL on failure. */
GLState *gl_create_context(int32_t width, int32_t height);
void gl_destroy_context(GLState *ctx);
void gl_make_current(GLState *ctx);
GLState *gl_get_current_context(void);

/* Wait for all queued rendering of ctx. Returns 0 or an mtgl_status code. */
int mtgl_finish(GLState *ctx);
/* Synchronise and return a host copy of the colour buffer (row 0 = top, packed
 * a<<24|b<<16|g<<8|r). Valid until the next GL call on ctx. */
const uint32_t *mtgl_color_buffer(GLState *ctx);
/* Synchronise and copy whole buffers to caller memory; any pointer may be NULL. */
int mtgl_read_framebuffer(GLState *ctx, uint32_t *color, float *depth, uint8_t *stencil);
int mtgl_framebuffer_size(GLState *ctx, int32_t *width, int32_t *height);
/* Name of the back end that renders this library's contexts. */
const char *mtgl_backend_name(void);
/* Pipeline counters (draws, triangles, fragments, passes, kernel launches) of ctx. */
int mtgl_get_stats(GLState *ctx, mtgl_stats *out);
int mtgl_reset_stats(GLState *ctx);
/* Per-phase device timing of ctx's passes (vertex / setup / bin / tile). */
int mtgl_set_profiling(GLState *ctx, int enable);
int mtgl_get_timings(GLState *ctx, mtgl_timings *out);
/* cudaStream_t of ctx, for callers that order their own GPU work with the renderer's. */
void *mtgl_cuda_stream(GLState *ctx);
/* Back-end option of ctx (MTGL_OPT_* in mtgl_dev.h). */
int mtgl_set_option(GLState *ctx, int option, int value);

/* Submit ctx's queued rendering without allocating any memory. No counterpart in the
 * reference, which renders synchronously and allocates only host memory.
 *
 * For callers that cannot let the renderer call cudaMalloc/cudaFree while they render:
 * real-time threads that cannot take the implied device-wide synchronisation, serving
 * processes that keep all device memory under their own budget, hosts whose CUDA
 * allocator belongs to another runtime. The queued pass runs exactly as on the normal
 * path, but its scratch (vertices, triangle records, tile lists, sort and scan temporaries)
 * comes from one static 64 MiB device array that every GPU loading the library holds.
 * Returns 0, or MTGL_ERR_OVERFLOW when the pass needs more scratch than that or more
 * staging than ctx already holds; the pass then stays queued and renders at the next
 * mtgl_finish. All calls share the array, so calls whose GPU work overlapped would race:
 * every context renders on its own stream, so that holds even for two contexts flushed
 * one after the other from one thread. The library therefore orders them: each call's
 * GPU work waits for the previous call's on the same device (one event per device,
 * under a lock), so they run in the order the host made them, whatever the context or
 * thread. Work the caller enqueues on mtgl_cuda_stream outside these calls is not
 * ordered against them. The first call on a device looks up the array's address and
 * creates that event; make it before any stream capture. */
int mtgl_flush_noalloc(GLState *ctx);

/* Render the pending frame (clears, then draws) of each of ctxs[0..n) in one batch; see
 * mtgl_dev_batch_submit in mtgl_dev.h. No counterpart in the reference, which renders
 * each context synchronously. Frames may differ in size and state; every framebuffer ends
 * up exactly as mtgl_finish on each context alone would leave it. Returns without
 * waiting; reading a context (glReadPixels, glFinish, mtgl_color_buffer) waits for it. */
int mtgl_batch_render(mtgl_batch *b, GLState *const *ctxs, int32_t n);
/* mtgl_batch_render, then after the run a copy of each context's colour buffer (width*height
 * packed RGBA8, row 0 = top) into colors[i]; NULL entries (or a NULL colors) copy nothing.
 * The copies have landed when mtgl_dev_batch_wait returns; page-locked destinations keep
 * them asynchronous. Each colors[i] must hold the frame's width * height pixels: those in
 * page-locked memory the device maps are written by a read-back kernel (one launch per 128
 * frames) unless mtgl_batch_config.readback_kernel is 0, the others are copied. */
int mtgl_batch_render_read(mtgl_batch *b, GLState *const *ctxs, uint32_t *const *colors, int32_t n);

/* Replay a GL command stream onto ctx (made current). No counterpart in the reference.
 * The stream is a sequence of records: u32 function id (the entry point's index among the
 * gl* functions of GL/gl.h in sorted name order), u32 argument count, then one 8-byte slot
 * per argument: int64 for integers, enums and pointers, IEEE double for GLfloat and
 * GLdouble. Each record calls the public entry point, exactly as the application would;
 * pointers must stay valid for as long as GL may read them. Returns MTGL_ERR_INVALID at
 * the first malformed record (the calls before it have run). */
int mtgl_play(GLState *ctx, const void *stream, size_t bytes);
/* mtgl_play for each (ctxs[i], streams[i]). When the contexts are distinct and in no
 * unfinished batch, the streams play concurrently on a pool of host threads
 * (MTGL_PLAY_THREADS, default: the online cores), each context on one thread, the longest
 * streams claimed first; otherwise in order on the calling thread. Every stream is played;
 * returns the status of the first failing stream by index. The calling thread's current
 * context is restored. */
int mtgl_play_many(GLState *const *ctxs, const void *const *streams, const size_t *bytes, int32_t n);
/* number of entry points a stream can call (the function-id range) */
int mtgl_play_function_count(void);

#ifdef __cplusplus
}
#endif

#endif /* MYTINYGL_GB300_CONTEXT_H */
