/*
 * serve.c — the serving loop (include/mytinygl/mtgl_serve.h). No counterpart in the reference.
 *
 * One worker thread owns the scene contexts and the GPU work. Each turn it:
 *   1. completes finished batches (mtgl_dev_batch_query, then _wait to verify), stamping
 *      their requests and returning framebuffers and budget to the pool;
 *   2. on a free executor, admits queued requests in arrival order while the memory budget
 *      (framebuffer bytes + pipeline-scratch estimate of every admitted request) allows,
 *      records each one's frame on its scene context, directs the pass into a pooled
 *      framebuffer of the request's size and launches the batch at once;
 *   3. otherwise sleeps briefly (a submission wakes it).
 * With several executors, batches launched while others still run overlap on the device;
 * a request that does not fit the budget waits at the head of the queue (requests are
 * admitted in arrival order), one that could never fit fails with MTGL_ERR_OVERFLOW.
 */
#define _POSIX_C_SOURCE 200809L
#include <errno.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mytinygl/mtgl_serve.h"

/* internal to the library (dev_runtime.cu, fe_context.c) */
extern int dev_device_index(const mtgl_dev *d);
extern int dev_bind_thread(int device);
extern int dev_current_device(void);
extern mtgl_dev *fe_context_device(GLState *ctx);

#define POST_VERTEX_BYTES 48u
#define RECORD_BYTES 244u  /* triangle record + its per-record tile count */
#define PAIR_BYTES 16u     /* key, value and their sort copies */

typedef struct {
    GLState *ctx;
    mtgl_dev *dev;
    void *stream;
    size_t bytes;
    uint64_t triangles;
    uint64_t scratch_bytes;
} scene_t;

typedef struct {
    mtgl_dev *dev;
    int32_t w, h;
    int busy;
} slot_t;

typedef struct {
    mtgl_batch *b;
    uint64_t launches_seen; /* the batch's kernel_launches counter at its last completion */
    int pending;
    int n;
    mtgl_request **reqs;
    slot_t **slots;
    uint64_t *costs;
} exec_t;

struct mtgl_server {
    mtgl_server_config cfg;
    int device;
    struct timespec t0;
    pthread_t worker;
    int worker_started;
    pthread_mutex_t mu;
    pthread_cond_t wake, idle;
    /* queue of submitted requests (FIFO ring) */
    mtgl_request **q;
    size_t q_cap, q_head, q_len;
    uint64_t outstanding; /* submitted and not finished */
    int stopping;
    /* worker-owned */
    scene_t *scenes;
    int32_t nscenes, scene_cap;
    slot_t *slots;
    int32_t nslots, slot_cap;
    exec_t *ex;
    uint64_t admitted_bytes;
    double busy_since;
    mtgl_server_stats st;
};

static double elapsed(const struct timespec *t0)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)(t.tv_sec - t0->tv_sec) + 1e-9 * (double)(t.tv_nsec - t0->tv_nsec);
}

double mtgl_server_now(mtgl_server *s) { return s ? elapsed(&s->t0) : 0.0; }

static void sleep_seconds(double sec)
{
    struct timespec ts;
    if (sec <= 0) return;
    ts.tv_sec = (time_t)sec;
    ts.tv_nsec = (long)((sec - (double)ts.tv_sec) * 1e9);
    nanosleep(&ts, NULL);
}

static uint64_t request_cost(const mtgl_server *s, const mtgl_request *r)
{
    const scene_t *sc = &s->scenes[r->scene];
    return (uint64_t)r->width * (uint64_t)r->height * 9u + sc->scratch_bytes;
}

/* a free framebuffer of w x h, creating one when the pool has none */
static slot_t *take_slot(mtgl_server *s, int32_t w, int32_t h)
{
    int32_t i;
    for (i = 0; i < s->nslots; i++)
        if (!s->slots[i].busy && s->slots[i].w == w && s->slots[i].h == h) {
            s->slots[i].busy = 1;
            return &s->slots[i];
        }
    if (s->nslots == s->slot_cap) {
        /* slots are referenced by pointer from in-flight batches: grow into a new array only
         * when none is in use would move them, so allocate generously up front instead */
        return NULL;
    }
    slot_t *sl = &s->slots[s->nslots];
    if (mtgl_dev_create(w, h, &sl->dev) != MTGL_OK) return NULL;
    sl->w = w;
    sl->h = h;
    sl->busy = 1;
    s->nslots++;
    s->st.framebuffers_allocated++;
    return sl;
}

static void finish_request(mtgl_server *s, mtgl_request *r, int status, int batch_size)
{
    r->status = status;
    r->batch_size = batch_size;
    r->finished = elapsed(&s->t0);
    pthread_mutex_lock(&s->mu);
    if (status == MTGL_OK) s->st.completed++;
    else s->st.failed++;
    s->outstanding--;
    if (s->outstanding == 0) pthread_cond_broadcast(&s->idle);
    pthread_mutex_unlock(&s->mu);
}

static int any_pending(const mtgl_server *s)
{
    int i;
    for (i = 0; i < s->cfg.executors; i++)
        if (s->ex[i].pending) return 1;
    return 0;
}

static int complete_batches(mtgl_server *s)
{
    int i, j, done = 0;
    for (i = 0; i < s->cfg.executors; i++) {
        exec_t *e = &s->ex[i];
        if (!e->pending) continue;
        int q = mtgl_dev_batch_query(e->b);
        if (q == 0) continue;
        int st = q < 0 ? -q : mtgl_dev_batch_wait(e->b);
        mtgl_batch_stats bs;
        if (mtgl_dev_batch_stats(e->b, &bs) == MTGL_OK) {
            pthread_mutex_lock(&s->mu);
            s->st.kernel_launches += bs.kernel_launches - e->launches_seen;
            pthread_mutex_unlock(&s->mu);
            e->launches_seen = bs.kernel_launches;
        }
        e->pending = 0;
        for (j = 0; j < e->n; j++) {
            e->slots[j]->busy = 0;
            s->admitted_bytes -= e->costs[j];
            finish_request(s, e->reqs[j], st, e->n);
        }
        e->n = 0;
        done = 1;
    }
    if (done && !any_pending(s)) {
        const double t = elapsed(&s->t0);
        pthread_mutex_lock(&s->mu);
        s->st.busy_seconds += t - s->busy_since;
        pthread_mutex_unlock(&s->mu);
    }
    return done;
}

/* pops up to `max` admissible requests; fails those that can never be served */
static int admit(mtgl_server *s, mtgl_request **out, uint64_t *costs, int max)
{
    int n = 0;
    uint64_t bytes = s->admitted_bytes;
    pthread_mutex_lock(&s->mu);
    while (s->q_len > 0 && n < max) {
        mtgl_request *r = s->q[s->q_head];
        int bad = r->scene < 0 || r->scene >= s->nscenes || r->width <= 0 || r->height <= 0;
        uint64_t cost = bad ? 0 : request_cost(s, r);
        if (!bad && cost > s->cfg.memory_budget) bad = MTGL_ERR_OVERFLOW;
        if (bad) {
            s->q_head = (s->q_head + 1) % s->q_cap;
            s->q_len--;
            pthread_mutex_unlock(&s->mu);
            finish_request(s, r, bad == MTGL_ERR_OVERFLOW ? MTGL_ERR_OVERFLOW : MTGL_ERR_INVALID, 0);
            pthread_mutex_lock(&s->mu);
            continue;
        }
        if (bytes + cost > s->cfg.memory_budget) {
            s->st.deferred_for_budget++;
            break;  /* the head waits for memory; later requests keep their order behind it */
        }
        bytes += cost;
        costs[n] = cost;
        out[n++] = r;
        s->q_head = (s->q_head + 1) % s->q_cap;
        s->q_len--;
    }
    pthread_mutex_unlock(&s->mu);
    return n;
}

static void launch_on(mtgl_server *s, exec_t *e)
{
    int i, n, st;
    mtgl_request **reqs = e->reqs;
    n = admit(s, reqs, e->costs, s->cfg.max_batch);
    if (n == 0) return;
    st = mtgl_dev_batch_begin(e->b);
    int kept = 0;
    for (i = 0; i < n; i++) {
        mtgl_request *r = reqs[i];
        scene_t *sc = &s->scenes[r->scene];
        slot_t *sl = st == MTGL_OK ? take_slot(s, r->width, r->height) : NULL;
        int rs = st != MTGL_OK ? st : (sl ? MTGL_OK : MTGL_ERR_OOM);
        if (rs == MTGL_OK) {
            gl_make_current(sc->ctx);
            glViewport(0, 0, r->width, r->height);
            glMatrixMode(GL_MODELVIEW);
            glLoadMatrixf(r->modelview);
            rs = mtgl_play(sc->ctx, sc->stream, sc->bytes);
        }
        if (rs == MTGL_OK) rs = mtgl_dev_batch_add(e->b, sc->dev, sl->dev);
        if (rs == MTGL_OK && r->color) rs = mtgl_dev_batch_readback(e->b, sl->dev, r->color);
        if (rs != MTGL_OK) {
            if (sl) sl->busy = 0;
            finish_request(s, r, rs, 0);
            continue;
        }
        r->admitted = elapsed(&s->t0);
        e->reqs[kept] = r;
        e->slots[kept] = sl;
        e->costs[kept] = e->costs[i];
        s->admitted_bytes += e->costs[i];
        kept++;
    }
    e->n = kept;
    if (st != MTGL_OK) return;
    st = mtgl_dev_batch_launch(e->b);
    if (kept == 0) return;
    if (st != MTGL_OK) {
        for (i = 0; i < kept; i++) {
            e->slots[i]->busy = 0;
            s->admitted_bytes -= e->costs[i];
            finish_request(s, e->reqs[i], st, 0);
        }
        e->n = 0;
        return;
    }
    if (!any_pending(s)) s->busy_since = elapsed(&s->t0);
    e->pending = 1;
    s->st.batches++;
    if (s->admitted_bytes > s->st.peak_bytes_admitted) s->st.peak_bytes_admitted = s->admitted_bytes;
}

static void *worker_main(void *arg)
{
    mtgl_server *s = (mtgl_server *)arg;
    dev_bind_thread(s->device);
    for (;;) {
        int progressed = complete_batches(s);
        exec_t *free_e = NULL;
        int i;
        for (i = 0; i < s->cfg.executors && !free_e; i++)
            if (!s->ex[i].pending) free_e = &s->ex[i];
        pthread_mutex_lock(&s->mu);
        const size_t queued = s->q_len;
        const int stop = s->stopping && queued == 0 && !any_pending(s);
        pthread_mutex_unlock(&s->mu);
        if (stop) break;
        if (free_e && queued) {
            const uint64_t before = s->st.batches;
            launch_on(s, free_e);
            progressed = progressed || s->st.batches != before;
        }
        if (progressed) continue;
        if (any_pending(s)) {
            sleep_seconds(20e-6);  /* poll the device */
        } else {
            struct timespec ts;
            pthread_mutex_lock(&s->mu);
            if (s->q_len == 0 && !s->stopping) {
                clock_gettime(CLOCK_REALTIME, &ts);
                ts.tv_nsec += 1000000;
                if (ts.tv_nsec >= 1000000000) {
                    ts.tv_sec++;
                    ts.tv_nsec -= 1000000000;
                }
                pthread_cond_timedwait(&s->wake, &s->mu, &ts);
            }
            pthread_mutex_unlock(&s->mu);
        }
    }
    return NULL;
}

int mtgl_server_create(const mtgl_server_config *cfg, mtgl_server **out)
{
    int i;
    if (!out) return MTGL_ERR_INVALID;
    mtgl_server *s = (mtgl_server *)calloc(1, sizeof(*s));
    if (!s) return MTGL_ERR_OOM;
    if (cfg) s->cfg = *cfg;
    if (!s->cfg.memory_budget) s->cfg.memory_budget = 40ull << 30;
    if (s->cfg.max_batch <= 0) s->cfg.max_batch = 64;
    if (s->cfg.executors <= 0) s->cfg.executors = 2;
    {
        mtgl_batch_config d;
        mtgl_dev_batch_defaults(&d);
        if (!s->cfg.batch.tile_size) s->cfg.batch.tile_size = d.tile_size;
        if (!s->cfg.batch.ctas_per_sm) s->cfg.batch.ctas_per_sm = d.ctas_per_sm;
        if (s->cfg.batch.record_factor <= 0) s->cfg.batch.record_factor = d.record_factor;
        if (s->cfg.batch.pair_factor <= 0) s->cfg.batch.pair_factor = d.pair_factor;
        if (!cfg) {
            s->cfg.batch.use_graph = d.use_graph;
            s->cfg.batch.order_by_cost = d.order_by_cost;
            s->cfg.batch.readback_kernel = d.readback_kernel;
        }
    }
    s->device = dev_current_device();
    clock_gettime(CLOCK_MONOTONIC, &s->t0);
    pthread_mutex_init(&s->mu, NULL);
    pthread_cond_init(&s->wake, NULL);
    pthread_cond_init(&s->idle, NULL);
    s->q_cap = 1024;
    s->q = (mtgl_request **)malloc(s->q_cap * sizeof(*s->q));
    s->slot_cap = 4096;
    s->slots = (slot_t *)calloc((size_t)s->slot_cap, sizeof(slot_t));
    s->ex = (exec_t *)calloc((size_t)s->cfg.executors, sizeof(exec_t));
    if (!s->q || !s->slots || !s->ex) {
        mtgl_server_destroy(s);
        return MTGL_ERR_OOM;
    }
    for (i = 0; i < s->cfg.executors; i++) {
        exec_t *e = &s->ex[i];
        e->reqs = (mtgl_request **)malloc((size_t)s->cfg.max_batch * sizeof(*e->reqs));
        e->slots = (slot_t **)malloc((size_t)s->cfg.max_batch * sizeof(*e->slots));
        e->costs = (uint64_t *)malloc((size_t)s->cfg.max_batch * sizeof(*e->costs));
        int st = mtgl_dev_batch_create(&s->cfg.batch, &e->b);
        if (!e->reqs || !e->slots || !e->costs || st != MTGL_OK) {
            mtgl_server_destroy(s);
            return st != MTGL_OK ? st : MTGL_ERR_OOM;
        }
    }
    if (pthread_create(&s->worker, NULL, worker_main, s) != 0) {
        mtgl_server_destroy(s);
        return MTGL_ERR_OOM;
    }
    s->worker_started = 1;
    *out = s;
    return MTGL_OK;
}

int mtgl_server_destroy(mtgl_server *s)
{
    int32_t i;
    if (!s) return MTGL_OK;
    if (s->worker_started) {
        pthread_mutex_lock(&s->mu);
        s->stopping = 1;
        pthread_cond_broadcast(&s->wake);
        pthread_mutex_unlock(&s->mu);
        pthread_join(s->worker, NULL);
    }
    if (s->ex) {
        for (i = 0; i < s->cfg.executors; i++) {
            if (s->ex[i].b) mtgl_dev_batch_destroy(s->ex[i].b);
            free(s->ex[i].reqs);
            free(s->ex[i].slots);
            free(s->ex[i].costs);
        }
    }
    for (i = 0; i < s->nslots; i++) mtgl_dev_destroy(s->slots[i].dev);
    for (i = 0; i < s->nscenes; i++) free(s->scenes[i].stream);
    free(s->scenes);
    free(s->slots);
    free(s->ex);
    free(s->q);
    pthread_mutex_destroy(&s->mu);
    pthread_cond_destroy(&s->wake);
    pthread_cond_destroy(&s->idle);
    free(s);
    return MTGL_OK;
}

int mtgl_server_add_scene(mtgl_server *s, GLState *ctx, const void *stream, size_t bytes, uint64_t triangles)
{
    if (!s || !ctx || (bytes && !stream)) return -MTGL_ERR_INVALID;
    mtgl_dev *dev = fe_context_device(ctx);
    if (!dev || dev_device_index(dev) != s->device) return -MTGL_ERR_INVALID;
    pthread_mutex_lock(&s->mu);
    if (s->nscenes == s->scene_cap) {
        int32_t cap = s->scene_cap ? 2 * s->scene_cap : 16;
        scene_t *n = (scene_t *)realloc(s->scenes, (size_t)cap * sizeof(scene_t));
        if (!n) {
            pthread_mutex_unlock(&s->mu);
            return -MTGL_ERR_OOM;
        }
        s->scenes = n;
        s->scene_cap = cap;
    }
    scene_t *sc = &s->scenes[s->nscenes];
    sc->stream = malloc(bytes ? bytes : 1);
    if (!sc->stream) {
        pthread_mutex_unlock(&s->mu);
        return -MTGL_ERR_OOM;
    }
    if (bytes) memcpy(sc->stream, stream, bytes);
    sc->bytes = bytes;
    sc->ctx = ctx;
    sc->dev = dev;
    sc->triangles = triangles;
    {
        const double per_tri = 3.0 * POST_VERTEX_BYTES + 8.0 +
                               s->cfg.batch.record_factor * (RECORD_BYTES + s->cfg.batch.pair_factor * PAIR_BYTES);
        sc->scratch_bytes = (uint64_t)(per_tri * (double)triangles);
    }
    int id = s->nscenes++;
    pthread_mutex_unlock(&s->mu);
    return id;
}

int mtgl_server_submit(mtgl_server *s, mtgl_request *req)
{
    if (!s || !req) return MTGL_ERR_INVALID;
    req->status = -1;
    req->admitted = req->finished = 0.0;
    req->batch_size = 0;
    pthread_mutex_lock(&s->mu);
    if (s->q_len == s->q_cap) {
        size_t cap = s->q_cap * 2, i;
        mtgl_request **n = (mtgl_request **)malloc(cap * sizeof(*n));
        if (!n) {
            pthread_mutex_unlock(&s->mu);
            return MTGL_ERR_OOM;
        }
        for (i = 0; i < s->q_len; i++) n[i] = s->q[(s->q_head + i) % s->q_cap];
        free(s->q);
        s->q = n;
        s->q_cap = cap;
        s->q_head = 0;
    }
    s->q[(s->q_head + s->q_len) % s->q_cap] = req;
    s->q_len++;
    s->outstanding++;
    s->st.submitted++;
    pthread_cond_signal(&s->wake);
    pthread_mutex_unlock(&s->mu);
    return MTGL_OK;
}

int mtgl_server_drain(mtgl_server *s)
{
    if (!s) return MTGL_ERR_INVALID;
    pthread_mutex_lock(&s->mu);
    while (s->outstanding > 0) pthread_cond_wait(&s->idle, &s->mu);
    pthread_mutex_unlock(&s->mu);
    return MTGL_OK;
}

typedef struct {
    mtgl_server *s;
    mtgl_request *reqs;
    int32_t n;
    int status;
} feeder_t;

static void *feeder_main(void *arg)
{
    feeder_t *f = (feeder_t *)arg;
    int32_t i;
    for (i = 0; i < f->n; i++) {
        for (;;) {
            const double wait = f->reqs[i].arrival - elapsed(&f->s->t0);
            if (wait <= 0) break;
            if (wait > 300e-6) sleep_seconds(wait - 200e-6);
        }
        if (mtgl_server_submit(f->s, &f->reqs[i]) != MTGL_OK) f->status = MTGL_ERR_OOM;
    }
    return NULL;
}

int mtgl_server_run_trace(mtgl_server *s, mtgl_request *reqs, int32_t n)
{
    pthread_t th;
    feeder_t f;
    if (!s || n < 0 || (n > 0 && !reqs)) return MTGL_ERR_INVALID;
    f.s = s;
    f.reqs = reqs;
    f.n = n;
    f.status = MTGL_OK;
    if (pthread_create(&th, NULL, feeder_main, &f) != 0) return MTGL_ERR_OOM;
    pthread_join(th, NULL);
    mtgl_server_drain(s);
    return f.status;
}

int mtgl_server_get_stats(mtgl_server *s, mtgl_server_stats *out)
{
    if (!s || !out) return MTGL_ERR_INVALID;
    pthread_mutex_lock(&s->mu);
    *out = s->st;
    pthread_mutex_unlock(&s->mu);
    return MTGL_OK;
}
