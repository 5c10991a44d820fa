// dev_batch.cu — batches: the pending passes of many contexts rendered by one pipeline run.
//
// No counterpart in the reference (one context renders at a time, inside glEnd). A batch
// turns n contexts' pending passes into one frame table (dev_pipeline.cu: every frame has
// its own framebuffer, size, tile range and clears; every draw keeps its own state
// blocks) and runs the pipeline once: K1 over all vertices, K2 over all triangles, K3 over
// the tiles of all frames, and a persistent K4 whose CTAs drain a device queue of
// (frame, tile) items (in frame order by default, or costliest first: the batch config's
// order_by_cost). The run has no host waits (record and pair
// buffers have fixed capacities, checked on the device), so it is captured once as a CUDA
// graph and replayed for as long as the batch's shape (tables, capacities, buffers) stays
// the same; only the staged bytes change between replays.
#include <algorithm>
#include <new>

#include "dev_internal.h"
#include "tuned.h"

using namespace mtgl;

namespace {

// launch shape the graph was captured with: a replay is valid while every field matches
struct Signature {
    const void *dstage, *hstage;
    size_t staged;
    Tables t;
    uint32_t rec_cap, pair_cap;
    int32_t ctas;
    int32_t order;
    void *scratch[kScratchSlots];
};

bool same(const Signature &a, const Signature &b) { return memcmp(&a, &b, sizeof(a)) == 0; }

// capacities are rounded up to 1/8 of their power-of-two size (at least 256 entries), so
// small changes between submissions keep the same capacity and the same graph
uint32_t round_capacity(uint64_t v)
{
    uint64_t p = 1;
    while (p < v) p <<= 1;
    const uint64_t q = std::max<uint64_t>(256, p / 8);
    const uint64_t r = (v + q - 1) / q * q;
    return (uint32_t)std::min<uint64_t>(r, 0xFFFFFF00ull);
}

}  // namespace

struct mtgl_batch {
    Exec x;
    HostStage stage;
    mtgl_batch_config cfg{};
    int tile_shift = 4;
    uint32_t rec_cap = 0, pair_cap = 0;  // capacities learned from the totals seen so far
    cudaEvent_t done = nullptr;
    // the submission being built (open) or in flight (pending)
    bool open = false;
    bool pending = false;
    std::vector<mtgl_dev *> devs;     // contexts whose framebuffer the run writes, once each
    std::vector<mtgl_dev *> sources;  // contexts whose resources it only reads, once each
    std::vector<Pass> passes;
    std::vector<FrameSrc> frames;     // frame f renders passes[f] into frames[f].dev
    std::vector<std::pair<mtgl_dev *, uint32_t *>> readbacks;
    std::vector<ReadbackItem> readback_items;  // scratch of record_after
    std::vector<mtgl_dev *> uploaded;  // contexts whose staging areas this run's copies read
    // client bytes of the first passes go to the device copy at add time, straight from
    // their context's pinned staging area; the rest are copied into this batch's area
    size_t direct_end = 0;
    bool direct_ok = true;
    uint64_t open_tris = 0;
    bool ran = false;                 // the pending submission ran the pipeline (not readbacks only)
    Tables t;
    PipeConfig run{};
    // graph of the last capacity-mode run
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    Signature sig{};
    bool have_sig = false;
    int graph_launches_ = 0;  // kernels one replay launches
    mtgl_batch_stats stats{};
};

namespace {

// The device address of [p, p + bytes) when both ends lie in page-locked host memory mapped
// into the device's address space, else null.
uint32_t *mapped_host(uint32_t *p, size_t bytes)
{
    cudaPointerAttributes a, z;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeHost || !a.devicePointer ||
        cudaPointerGetAttributes(&z, reinterpret_cast<char *>(p) + bytes - 1) != cudaSuccess ||
        z.type != cudaMemoryTypeHost ||
        z.devicePointer != static_cast<void *>(static_cast<char *>(a.devicePointer) + bytes - 1)) {
        cudaGetLastError();
        return nullptr;
    }
    return static_cast<uint32_t *>(a.devicePointer);
}

// Colour read-backs, then the run's completion events. Destinations in mapped page-locked
// memory are written by read-back kernels (one launch per group of frames instead of a copy
// call per frame); the others are copied.
int record_after(mtgl_batch *b)
{
    std::vector<ReadbackItem> &items = b->readback_items;
    items.clear();
    for (const auto &rb : b->readbacks) {
        const size_t n = (size_t)rb.first->width * (size_t)rb.first->height;
        uint32_t *dst = (b->cfg.readback_kernel && n > 0 && n <= UINT32_MAX) ? mapped_host(rb.second, n * 4) : nullptr;
        if (dst) items.push_back(ReadbackItem{rb.first->color, dst, (uint32_t)n, 0u});
        else CK(cudaMemcpyAsync(rb.second, rb.first->color, n * 4, cudaMemcpyDeviceToHost, b->x.stream));
    }
    if (!items.empty()) {
        const int k = launch_readback(items.data(), (int)items.size(), b->x.sms, b->x.stream);
        CK(cudaGetLastError());
        b->stats.kernel_launches += (uint64_t)k;
    }
    if (!b->devs.empty()) {  // one mark for every target's "written by this run"
        RunMark *m = mark_new(b->x.device);
        if (!m) return MTGL_ERR_CUDA;
        const cudaError_t e = cudaEventRecord(m->ev, b->x.stream);
        if (e != cudaSuccess) {
            mark_drop(m);
            return fail_cuda("cudaEventRecord", e);
        }
        for (mtgl_dev *d : b->devs) {
            if (d->after_batch) mark_drop(d->after_batch);
            mark_hold(m);
            d->after_batch = m;
            d->after_stream = b->x.stream;
        }
        mark_drop(m);
    }
    CK(cudaEventRecord(b->done, b->x.stream));
    return MTGL_OK;
}

// One mark after the copies queued from contexts' staging areas so far: each area may be
// rewritten once it has passed.
int mark_uploads(mtgl_batch *b)
{
    if (b->uploaded.empty()) return MTGL_OK;
    RunMark *m = mark_new(b->x.device);
    if (!m) return MTGL_ERR_CUDA;
    const cudaError_t e = cudaEventRecord(m->ev, b->x.stream);
    if (e != cudaSuccess) {
        mark_drop(m);
        return fail_cuda("cudaEventRecord", e);
    }
    for (mtgl_dev *d : b->uploaded) d->stage.hold_upload(m);
    mark_drop(m);
    b->uploaded.clear();
    return MTGL_OK;
}

int launch_run(mtgl_batch *b)
{
    const bool was_profiling = b->x.profile;
    if (b->cfg.use_graph) b->x.profile = false;  // phase events would be baked into the graph
    int st = run_pipeline(b->x, b->x.pool, b->stage, b->t, b->run, nullptr, true);  // scratch first
    if (st) return st;
    Signature s;
    memset(&s, 0, sizeof(s));
    s.dstage = b->x.dstage;
    s.hstage = b->stage.p;
    s.staged = b->stage.used;
    s.t = b->t;
    s.rec_cap = b->run.rec_cap;
    s.pair_cap = b->run.pair_cap;
    s.ctas = b->run.ctas;
    s.order = b->run.order ? 1 : 0;
    for (int i = 0; i < kScratchSlots; i++) s.scratch[i] = b->x.pool.p[i];
    if (!b->cfg.use_graph) {
        PipeOut o;
        st = run_pipeline(b->x, b->x.pool, b->stage, b->t, b->run, &o);
        b->stats.kernel_launches += (uint64_t)o.launches;
        b->x.profile = was_profiling;
        return st;
    }
    if (!(b->exec && b->have_sig && same(s, b->sig))) {
        CK(cudaStreamBeginCapture(b->x.stream, cudaStreamCaptureModeThreadLocal));
        PipeOut o;
        st = run_pipeline(b->x, b->x.pool, b->stage, b->t, b->run, &o);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->x.stream, &g);
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return fail_cuda("cudaStreamEndCapture", e);
        bool updated = false;
        if (b->exec) {
            cudaGraphExecUpdateResultInfo info;
            updated = cudaGraphExecUpdate(b->exec, g, &info) == cudaSuccess;
            if (!updated) {
                cudaGetLastError();
                cudaGraphExecDestroy(b->exec);
                b->exec = nullptr;
            }
        }
        if (!updated) CK(cudaGraphInstantiate(&b->exec, g, 0));
        if (b->graph) cudaGraphDestroy(b->graph);
        b->graph = g;
        b->sig = s;
        b->have_sig = true;
        b->stats.graph_captures++;
        b->stats.kernel_launches += (uint64_t)o.launches;
        b->graph_launches_ = o.launches;
    } else {
        b->stats.graph_replays++;
        b->stats.kernel_launches += (uint64_t)b->graph_launches_;
    }
    CK(cudaGraphLaunch(b->exec, b->x.stream));
    b->x.profile = was_profiling;
    return MTGL_OK;
}

}  // namespace

extern "C" {

void mtgl_dev_batch_defaults(mtgl_batch_config *cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->tile_size = MTGL_TUNED_TILE_SIZE;
    cfg->ctas_per_sm = MTGL_TUNED_CTAS_PER_SM;
    cfg->record_factor = MTGL_TUNED_RECORD_FACTOR;
    cfg->pair_factor = MTGL_TUNED_PAIR_FACTOR;
    cfg->use_graph = 1;
    cfg->order_by_cost = MTGL_TUNED_ORDER_BY_COST;
    cfg->readback_kernel = 1;
}

int mtgl_dev_batch_create(const mtgl_batch_config *cfg, mtgl_batch **out)
{
    if (!out) return MTGL_ERR_INVALID;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        snprintf(g_err, sizeof(g_err), "no CUDA device (%s)", e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
        return MTGL_ERR_NO_DEVICE;
    }
    mtgl_batch_config c;
    mtgl_dev_batch_defaults(&c);
    if (cfg) {
        if (cfg->tile_size) c.tile_size = cfg->tile_size;
        if (cfg->ctas_per_sm) c.ctas_per_sm = cfg->ctas_per_sm;
        if (cfg->record_factor > 0) c.record_factor = cfg->record_factor;
        if (cfg->pair_factor > 0) c.pair_factor = cfg->pair_factor;
        c.use_graph = cfg->use_graph;
        c.order_by_cost = cfg->order_by_cost;
        c.readback_kernel = cfg->readback_kernel;
    }
    int shift = 0;
    while (shift <= kTileShiftMax && (1 << shift) != c.tile_size) shift++;
    if (shift < kTileShiftMin || shift > kTileShiftMax || c.ctas_per_sm < 0) return MTGL_ERR_INVALID;
    mtgl_batch *b = new (std::nothrow) mtgl_batch();
    if (!b) return MTGL_ERR_OOM;
    b->cfg = c;
    b->tile_shift = shift;
    int st = b->x.init(nullptr);
    if (st) {
        delete b;
        return st;
    }
    CK(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    b->stats.tile_size = c.tile_size;
    *out = b;
    return MTGL_OK;
}

int mtgl_dev_batch_destroy(mtgl_batch *b)
{
    if (!b) return MTGL_OK;
    cudaSetDevice(b->x.device);
    mtgl_dev_batch_wait(b);
    mark_uploads(b);  // copies of an open run that never launched: their areas wait on a mark
    cudaStreamSynchronize(b->x.stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->stage.release();
    b->x.destroy();
    cudaEventDestroy(b->done);
    delete b;
    return MTGL_OK;
}

int mtgl_dev_batch_begin(mtgl_batch *b)
{
    if (!b) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(b->x.device));
    int st = mtgl_dev_batch_wait(b);
    if (st || (st = mark_uploads(b)) || (st = b->stage.wait())) return st;
    b->stage.used = 0;
    b->devs.clear();
    b->sources.clear();
    b->passes.clear();
    b->frames.clear();
    b->readbacks.clear();
    b->uploaded.clear();
    b->direct_end = 0;
    b->direct_ok = true;
    b->open_tris = 0;
    b->open = true;
    return MTGL_OK;
}

namespace {

// Puts d in the run's context sets once, ordering the batch stream after d's queued work.
// A written context (a target framebuffer) is also ordered after any batch of another
// executor that wrote it; a context whose resources are only read needs no order against
// other batches that only read them, so batches sharing a scene still run side by side.
int involve(mtgl_batch *b, mtgl_dev *d, bool write)
{
    if (d->device != b->x.device) return MTGL_ERR_INVALID;
    bool known = false;
    for (mtgl_dev *e : b->devs) known = known || e == d;
    for (mtgl_dev *e : b->sources) known = known || e == d;
    if (!known && d->dirty) {
        CK(cudaEventRecord(d->tail, d->x.stream));
        CK(cudaStreamWaitEvent(b->x.stream, d->tail, 0));
        d->dirty = false;
    }
    if (!write) {
        if (!known) b->sources.push_back(d);
        return MTGL_OK;
    }
    for (mtgl_dev *e : b->devs)
        if (e == d) return MTGL_OK;
    if (d->batch && d->batch != b) {
        int st = mtgl_dev_batch_wait(d->batch);
        if (st) return st;
    }
    // (a batch that last wrote d on this same stream is ordered before this run already)
    if (d->after_batch && d->after_stream != b->x.stream)
        CK(cudaStreamWaitEvent(b->x.stream, d->after_batch->ev, 0));
    b->devs.push_back(d);
    return MTGL_OK;
}

// marks the run's contexts: targets wait for it through their stream, sources list it as a
// reader their next device operation waits for
void attach(mtgl_batch *b)
{
    for (mtgl_dev *d : b->devs) d->batch = b;
    for (mtgl_dev *d : b->sources) {
        bool written = false;
        for (mtgl_dev *e : b->devs) written = written || e == d;
        if (!written) d->readers.push_back(b);
    }
}

void detach(mtgl_batch *b)
{
    for (mtgl_dev *d : b->devs)
        if (d->batch == b) d->batch = nullptr;
    for (mtgl_dev *d : b->sources)
        for (size_t i = 0; i < d->readers.size(); i++)
            if (d->readers[i] == b) {
                d->readers.erase(d->readers.begin() + (long)i);
                break;
            }
}

}  // namespace

int mtgl_dev_batch_add(mtgl_batch *b, mtgl_dev *src, mtgl_dev *target)
{
    if (!b || !src || !target || !b->open) return MTGL_ERR_INVALID;
    for (const FrameSrc &f : b->frames)
        if (f.dev == target) return MTGL_ERR_INVALID;  // two frames of one batch cannot share a framebuffer
    if (src->pass.empty()) return MTGL_OK;
    int st;
    if ((st = involve(b, src, src == target)) || (st = involve(b, target, true))) return st;
    int64_t off = 0;
    const size_t bytes = src->stage.used;
    if ((st = b->stage.reserve(bytes, &off))) return st;
    if (bytes && b->direct_ok && (size_t)off + bytes <= b->x.dcap) {
        // The batch stream runs this copy after the batch's previous run and before this
        // one; the context's next staging write waits for it.
        CK(cudaMemcpyAsync(b->x.dstage + off, src->stage.p, bytes, cudaMemcpyHostToDevice, b->x.stream));
        src->stage.upload_stream = b->x.stream;  // marked at launch (mark_uploads)
        b->uploaded.push_back(src);
        b->direct_end = (size_t)off + bytes;
    } else if (bytes) {
        b->direct_ok = false;  // offsets only grow: later passes do not fit either
        memcpy(b->stage.p + off, src->stage.p, bytes);
    }
    b->passes.push_back(std::move(src->pass));
    src->pass.reset();
    src->stage.used = 0;
    b->frames.push_back(FrameSrc{target, nullptr, off});
    b->open_tris += b->passes.back().tris;
    src->stats.passes++;
    src->stats.input_triangles += b->passes.back().tris;
    src->stats.vertices += b->passes.back().slots;
    src->stats.vertex_bytes += b->passes.back().vbytes;
    return MTGL_OK;
}

int mtgl_dev_batch_readback(mtgl_batch *b, mtgl_dev *target, uint32_t *host_color)
{
    if (!b || !target || !host_color || !b->open) return MTGL_ERR_INVALID;
    int st = involve(b, target, true);
    if (st) return st;
    b->readbacks.emplace_back(target, host_color);
    return MTGL_OK;
}

int mtgl_dev_batch_launch(mtgl_batch *b)
{
    if (!b || !b->open) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(b->x.device));
    b->open = false;
    int st;
    if ((st = mark_uploads(b))) return st;
    if (b->frames.empty()) {
        if (b->readbacks.empty()) return MTGL_OK;
        if ((st = record_after(b))) return st;  // readbacks only
        attach(b);
        b->pending = true;
        b->ran = false;
        return MTGL_OK;
    }
    for (size_t i = 0; i < b->frames.size(); i++) b->frames[i].pass = &b->passes[i];
    if ((st = build_tables(b->x, b->stage, b->frames.data(), (uint32_t)b->frames.size(), b->tile_shift, true, b->t,
                           b->direct_end)))
        return st;
    const uint64_t tris = b->open_tris;
    // capacities: the larger of the learned totals and the configured factors
    const uint64_t rec_want = std::max<uint64_t>((uint64_t)b->rec_cap, (uint64_t)(tris * b->cfg.record_factor) + 1);
    const uint32_t rec_cap = tris ? round_capacity(rec_want) : 0;
    const uint64_t pair_want = std::max<uint64_t>((uint64_t)b->pair_cap, (uint64_t)(rec_cap * b->cfg.pair_factor) + 1);
    const uint32_t pair_cap = tris ? round_capacity(pair_want) : 0;
    b->run = PipeConfig();
    b->run.exact = false;
    b->run.rec_cap = rec_cap;
    b->run.pair_cap = pair_cap;
    b->run.ctas = persistent_ctas(b->x, b->t, b->cfg.ctas_per_sm);
    b->run.order = b->cfg.order_by_cost != 0;
    if ((st = launch_run(b))) return st;
    if ((st = b->stage.mark_uploaded(b->x.stream))) return st;
    if ((st = record_after(b))) return st;
    attach(b);
    b->pending = true;
    b->ran = true;
    b->stats.batches++;
    b->stats.frames += b->frames.size();
    b->stats.input_triangles += tris;
    for (const Pass &p : b->passes) {
        b->stats.vertices += p.slots;
        b->stats.vertex_bytes += p.vbytes;
    }
    b->stats.ctas = b->run.ctas;
    return MTGL_OK;
}

// every context renders its own pending pass; colors[i] (when given and non-null) receives
// devs[i]'s colour buffer after the run
static int submit_read(mtgl_batch *b, mtgl_dev *const *devs, uint32_t *const *colors, int32_t n)
{
    if (!b || n < 0 || (n > 0 && !devs)) return MTGL_ERR_INVALID;
    for (int32_t i = 0; i < n; i++) {
        if (!devs[i]) return MTGL_ERR_INVALID;
        for (int32_t j = 0; j < i; j++)
            if (devs[j] == devs[i]) return MTGL_ERR_INVALID;  // a context renders one pass per batch
    }
    int st = mtgl_dev_batch_begin(b);
    if (st) return st;
    for (int32_t i = 0; i < n; i++) {
        if ((st = mtgl_dev_batch_add(b, devs[i], devs[i]))) {
            b->open = false;
            return st;
        }
    }
    for (int32_t i = 0; colors && i < n; i++) {
        if (colors[i] && (st = mtgl_dev_batch_readback(b, devs[i], colors[i]))) {
            b->open = false;
            return st;
        }
    }
    return mtgl_dev_batch_launch(b);
}

int mtgl_dev_batch_submit(mtgl_batch *b, mtgl_dev *const *devs, int32_t n) { return submit_read(b, devs, nullptr, n); }

int mtgl_dev_batch_query(mtgl_batch *b)
{
    if (!b) return MTGL_ERR_INVALID;
    if (!b->pending) return 1;
    cudaError_t e = cudaEventQuery(b->done);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return -fail_cuda("cudaEventQuery", e);
}

int mtgl_dev_batch_wait(mtgl_batch *b)
{
    if (!b) return MTGL_ERR_INVALID;
    if (!b->pending) return MTGL_OK;
    CK(cudaSetDevice(b->x.device));
    b->pending = false;  // a failure below leaves nothing to retry
    detach(b);
    CK(cudaEventSynchronize(b->done));
    if (!b->ran) {
        b->devs.clear();
        b->sources.clear();
        b->readbacks.clear();
        return MTGL_OK;
    }
    uint32_t nrec = b->x.h_totals[0], npairs = b->x.h_totals[1];
    if (nrec > b->run.rec_cap || npairs > b->run.pair_cap) {
        // The tile launch left every framebuffer untouched: render again with exact sizing
        // from the same staged tables, and remember the totals for the next submission.
        PipeConfig c = b->run;
        c.exact = true;
        PipeOut o;
        int st = run_pipeline(b->x, b->x.pool, b->stage, b->t, c, &o);
        if (st) return st;
        if ((st = b->stage.mark_uploaded(b->x.stream))) return st;
        if ((st = record_after(b))) return st;
        CK(cudaEventSynchronize(b->done));
        nrec = o.nrec;
        npairs = o.npairs;
        b->stats.overflow_reruns++;
        b->stats.kernel_launches += (uint64_t)o.launches;
    }
    b->rec_cap = std::max(b->rec_cap, nrec);
    b->pair_cap = std::max(b->pair_cap, npairs);
    b->stats.setup_triangles += nrec;
    b->stats.bin_entries += npairs;
    b->stats.record_capacity = b->run.rec_cap;
    b->stats.pair_capacity = b->run.pair_cap;
    b->devs.clear();
    b->sources.clear();
    b->passes.clear();
    b->frames.clear();
    b->readbacks.clear();
    return MTGL_OK;
}

int mtgl_dev_batch_stats(mtgl_batch *b, mtgl_batch_stats *out)
{
    if (!b || !out) return MTGL_ERR_INVALID;
    int st = mtgl_dev_batch_wait(b);
    if (st) return st;
    unsigned long long f = 0;
    CK(cudaMemcpyAsync(&f, b->x.d_frags, sizeof(f), cudaMemcpyDeviceToHost, b->x.stream));
    CK(cudaStreamSynchronize(b->x.stream));
    *out = b->stats;
    out->fragments = f;
    uint32_t dbg = 0;
    CK(cudaMemcpy(&dbg, b->x.d_totals + kDebugStatusWord, sizeof(dbg), cudaMemcpyDeviceToHost));
    out->debug_status = dbg;
    return MTGL_OK;
}

int mtgl_dev_batch_reset_stats(mtgl_batch *b)
{
    if (!b) return MTGL_ERR_INVALID;
    int st = mtgl_dev_batch_wait(b);
    if (st) return st;
    const int32_t ts = b->stats.tile_size, ctas = b->stats.ctas;
    memset(&b->stats, 0, sizeof(b->stats));
    b->stats.tile_size = ts;
    b->stats.ctas = ctas;
    CK(cudaMemsetAsync(b->x.d_frags, 0, sizeof(unsigned long long), b->x.stream));
    CK(cudaMemsetAsync(b->x.d_totals + kDebugStatusWord, 0, sizeof(uint32_t), b->x.stream));
    CK(cudaStreamSynchronize(b->x.stream));
    return MTGL_OK;
}

void *mtgl_dev_batch_stream(mtgl_batch *b) { return b ? (void *)b->x.stream : nullptr; }

int mtgl_dev_batch_profile(mtgl_batch *b, int enable)
{
    if (!b) return MTGL_ERR_INVALID;
    int st = mtgl_dev_batch_wait(b);
    if (st) return st;
    CK(cudaStreamSynchronize(b->x.stream));
    if ((st = b->x.prof_collect())) return st;
    b->x.profile = enable != 0;
    memset(&b->x.timings, 0, sizeof(b->x.timings));
    return MTGL_OK;
}

int mtgl_dev_batch_timings(mtgl_batch *b, mtgl_timings *out)
{
    if (!b || !out) return MTGL_ERR_INVALID;
    int st = mtgl_dev_batch_wait(b);
    if (st) return st;
    CK(cudaStreamSynchronize(b->x.stream));
    if ((st = b->x.prof_collect())) return st;
    *out = b->x.timings;
    return MTGL_OK;
}

}  // extern "C"

// ---- GL-level entry: the contexts' pending frames as one batch

extern "C" mtgl_dev *fe_context_device(GLState *ctx);

extern "C" int mtgl_batch_render_read(mtgl_batch *b, GLState *const *ctxs, uint32_t *const *colors, int32_t n)
{
    if (!b || n < 0 || (n > 0 && !ctxs)) return MTGL_ERR_INVALID;
    std::vector<mtgl_dev *> devs((size_t)n);
    for (int32_t i = 0; i < n; i++) {
        devs[i] = ctxs[i] ? fe_context_device(ctxs[i]) : nullptr;
        if (!devs[i]) return MTGL_ERR_INVALID;
    }
    return submit_read(b, devs.data(), colors, n);
}

extern "C" int mtgl_batch_render(mtgl_batch *b, GLState *const *ctxs, int32_t n)
{
    return mtgl_batch_render_read(b, ctxs, nullptr, n);
}
