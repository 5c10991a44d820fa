/*
 * fe_play_many.c — mtgl_play_many: the command streams of many contexts played at once.
 *
 * No counterpart in the reference, where one thread drives one current context
 * (gl_api.c:14-23). Contexts share no front-end state and, outside an unfinished batch (one
 * writing their framebuffer or reading their resources), no back-end state either, so
 * distinct contexts play on a pool of threads: each thread claims the next unplayed stream
 * (longest first), makes its context current and plays it. Staging copies, index scans and state snapshots of
 * different frames then run on all host cores instead of one.
 */
#include <pthread.h>
#include <unistd.h>

#include "fe_internal.h"

typedef struct {
    GLState *const *ctxs;
    const void *const *streams;
    const size_t *bytes;
    int32_t n;
    int *status;
    const int32_t *order; /* claim order (null: stream order) */
    int32_t next;         /* next unclaimed position of the order */
} play_job;

static void *play_worker(void *arg)
{
    play_job *j = (play_job *)arg;
    for (;;) {
        int32_t k = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
        if (k >= j->n) break;
        const int32_t i = j->order ? j->order[k] : k;
        j->status[i] = mtgl_play(j->ctxs[i], j->streams[i], j->bytes[i]);
    }
    return NULL;
}

/* longest streams first (a stream's bytes stand for its work), so that the last streams
 * claimed are short and the threads finish together */
static const size_t *g_sort_bytes;
static int cmp_longer(const void *a, const void *b)
{
    const size_t x = g_sort_bytes[*(const int32_t *)a], y = g_sort_bytes[*(const int32_t *)b];
    if (x != y) return x > y ? -1 : 1;
    return *(const int32_t *)a - *(const int32_t *)b;
}

static int cmp_ptr(const void *a, const void *b)
{
    uintptr_t x = (uintptr_t) * (GLState *const *)a, y = (uintptr_t) * (GLState *const *)b;
    return x < y ? -1 : (x > y);
}

/* threads to use: MTGL_PLAY_THREADS, else the online cores; at most one per stream */
static int32_t play_threads(int32_t n)
{
    const char *e = getenv("MTGL_PLAY_THREADS");
    long t = (e && *e) ? strtol(e, NULL, 10) : sysconf(_SC_NPROCESSORS_ONLN);
    if (t < 1) t = 1;
    if (t > 64) t = 64;
    return t > n ? n : (int32_t)t;
}

/* 1 when every context is non-null, distinct and in no unfinished batch. (A context in one
 * plays on the calling thread, where its first device operation waits for the batch, as a
 * single mtgl_play would.) */
static int can_share(GLState *const *ctxs, int32_t n)
{
    GLState **sorted = (GLState **)malloc((size_t)n * sizeof(GLState *));
    int ok = sorted != NULL;
    for (int32_t i = 0; ok && i < n; i++) {
        ok = ctxs[i] != NULL && !mtgl_dev_in_batch(ctxs[i]->dev);
        if (ok) sorted[i] = ctxs[i];
    }
    if (ok) {
        qsort(sorted, (size_t)n, sizeof(GLState *), cmp_ptr);
        for (int32_t i = 1; ok && i < n; i++) ok = sorted[i] != sorted[i - 1];
    }
    free(sorted);
    return ok;
}

int mtgl_play_many(GLState *const *ctxs, const void *const *streams, const size_t *bytes, int32_t n)
{
    if (n < 0 || (n > 0 && (!ctxs || !streams || !bytes))) return MTGL_ERR_INVALID;
    if (n == 0) return MTGL_OK;
    GLState *prev = gl_get_current_context();
    int *status = (int *)calloc((size_t)n, sizeof(int));
    if (!status) return MTGL_ERR_OOM;
    int32_t threads = play_threads(n);
    if (threads > 1 && !can_share(ctxs, n)) threads = 1;
    int32_t *order = NULL;
    if (threads > 1 && (order = (int32_t *)malloc((size_t)n * sizeof(int32_t))) != NULL) {
        for (int32_t i = 0; i < n; i++) order[i] = i;
        static pthread_mutex_t sort_lock = PTHREAD_MUTEX_INITIALIZER;  /* qsort has no context argument */
        pthread_mutex_lock(&sort_lock);
        g_sort_bytes = bytes;
        qsort(order, (size_t)n, sizeof(int32_t), cmp_longer);
        pthread_mutex_unlock(&sort_lock);
    }
    play_job job = {ctxs, streams, bytes, n, status, order, 0};
    pthread_t tid[64];
    int32_t started = 0;
    for (int32_t k = 1; k < threads; k++) {
        if (pthread_create(&tid[started], NULL, play_worker, &job) != 0) break;
        started++;
    }
    play_worker(&job); /* this thread plays too; with no helper it plays every stream in order */
    for (int32_t k = 0; k < started; k++) pthread_join(tid[k], NULL);
    gl_make_current(prev);
    free(order);
    int st = MTGL_OK;
    for (int32_t i = 0; i < n && st == MTGL_OK; i++) st = status[i];
    free(status);
    return st;
}
