/*
 * mtgl_serve.h — a serving loop over the batched renderer. No counterpart in MyTinyGL,
 * which renders one context synchronously inside glEnd.
 *
 * Scenes stay resident: each is a GL context holding its buffer objects and textures plus
 * a command stream (mtgl_play format) with the GL calls of one frame. A request names a
 * scene, a framebuffer size and a modelview. One worker thread runs the loop: it admits
 * queued requests against a memory budget (framebuffer plus pipeline scratch of every
 * admitted request), records each admitted request's frame on its scene's context
 * (glViewport(0, 0, w, h); glMatrixMode(GL_MODELVIEW); glLoadMatrixf(modelview); the
 * scene's stream), directs that pass into a pooled framebuffer of the request's size, and
 * launches what it has collected as one batch (mtgl_dev_batch_*) as soon as an executor is
 * free. Several executors, each with its own stream, keep batches in flight at once, so
 * requests that arrive while others render are batched and run beside them. When a batch
 * finishes its requests complete (colour read back if asked for), and their framebuffers
 * and budget return to the pool.
 *
 * A scene's stream must render one pass (one glClear, then draws; no glReadPixels,
 * glDrawPixels, glFinish or resource changes), and must not reset the modelview matrix
 * before its draws: the request's modelview is what positions the scene. While the
 * server runs, its scene contexts belong to its worker thread.
 */
#ifndef MYTINYGL_GB300_MTGL_SERVE_H
#define MYTINYGL_GB300_MTGL_SERVE_H

#include <stddef.h>
#include <stdint.h>

#include "GL/gl.h"
#include "mytinygl/mtgl_dev.h"
#include "mytinygl/mytinygl.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mtgl_server mtgl_server;

typedef struct {
    uint64_t memory_budget;    /* bytes admitted at once: framebuffers + pipeline scratch (0: 40 GiB) */
    int32_t max_batch;         /* requests per batch (0: 64)                                        */
    int32_t executors;         /* batches in flight at once (0: 2)                                  */
    mtgl_batch_config batch;   /* executor settings; zero fields take the tuned defaults            */
} mtgl_server_config;

typedef struct {
    /* set by the caller */
    int32_t scene;             /* index from mtgl_server_add_scene                                  */
    int32_t width, height;     /* framebuffer of this request                                       */
    float modelview[16];       /* column-major, loaded before the scene's stream                    */
    uint32_t *color;           /* optional: receives width*height packed RGBA8, row 0 = top          */
    double arrival;            /* mtgl_server_run_trace: submit time on the server clock (seconds)  */
    /* set by the server */
    double admitted, finished; /* server clock                                                       */
    int32_t status;            /* MTGL_OK, or an mtgl_status                                         */
    int32_t batch_size;        /* requests in the batch that rendered it                             */
} mtgl_request;

typedef struct {
    uint64_t submitted, completed, failed, batches, deferred_for_budget;
    uint64_t peak_bytes_admitted, framebuffers_allocated;
    double busy_seconds;       /* time with at least one batch in flight                             */
    uint64_t kernel_launches;  /* device kernels the completed batches launched                      */
} mtgl_server_stats;

int mtgl_server_create(const mtgl_server_config *cfg, mtgl_server **out);
/* Stops the worker (after finishing what was submitted) and frees the framebuffer pool;
 * the scene contexts stay the caller's. */
int mtgl_server_destroy(mtgl_server *s);
/* Registers a scene, before any request is submitted; returns its index, or a negative
 * mtgl_status. triangles: input triangles of the stream (pipeline-scratch estimate for
 * admission). The stream is copied; the arrays it points to must outlive the server. */
int mtgl_server_add_scene(mtgl_server *s, GLState *ctx, const void *stream, size_t bytes, uint64_t triangles);
/* Seconds since the server was created (CLOCK_MONOTONIC). */
double mtgl_server_now(mtgl_server *s);
/* Queues a request (thread-safe); the request must stay valid until it has finished. */
int mtgl_server_submit(mtgl_server *s, mtgl_request *req);
/* Waits until every submitted request has finished. */
int mtgl_server_drain(mtgl_server *s);
/* Replays a trace: submits reqs[i] when the server clock reaches reqs[i].arrival (from a
 * feeder thread), then drains. Arrival times must be non-decreasing. */
int mtgl_server_run_trace(mtgl_server *s, mtgl_request *reqs, int32_t n);
int mtgl_server_get_stats(mtgl_server *s, mtgl_server_stats *out);

#ifdef __cplusplus
}
#endif

#endif /* MYTINYGL_GB300_MTGL_SERVE_H */
