// dev_pipeline.cu — the pass pipeline shared by single-context flushes and batches:
// staging helpers, scratch, table assembly and the K1 -> K2 -> K3 -> K4 launch sequence.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>

#include "dev_internal.h"

namespace mtgl {

thread_local char g_err[512] = "";

int fail_cuda(const char *what, cudaError_t e)
{
    snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
    return MTGL_ERR_CUDA;
}

// ------------------------------------------------------------------ host staging

// ------------------------------------------------------------------ run marks

namespace {
std::mutex g_mark_mu;
std::vector<RunMark *> g_mark_pool;  // marks no one holds
}  // namespace

RunMark *mark_new(int device)
{
    {
        std::lock_guard<std::mutex> lk(g_mark_mu);
        for (size_t i = 0; i < g_mark_pool.size(); i++) {
            RunMark *m = g_mark_pool[i];
            if (m->device != device) continue;
            g_mark_pool[i] = g_mark_pool.back();
            g_mark_pool.pop_back();
            m->refs.store(1);
            return m;
        }
    }
    RunMark *m = new (std::nothrow) RunMark();
    if (!m) {
        snprintf(g_err, sizeof(g_err), "out of host memory");
        return nullptr;
    }
    m->device = device;
    cudaError_t e = cudaEventCreateWithFlags(&m->ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        fail_cuda("cudaEventCreateWithFlags", e);
        delete m;
        return nullptr;
    }
    m->refs.store(1);
    return m;
}

void mark_hold(RunMark *m) { m->refs.fetch_add(1); }

void mark_drop(RunMark *m)
{
    if (m->refs.fetch_sub(1) != 1) return;
    std::lock_guard<std::mutex> lk(g_mark_mu);
    g_mark_pool.push_back(m);
}

int HostStage::wait()
{
    if (inflight) {
        CK(cudaEventSynchronize(done));
        inflight = false;
    }
    if (upload_stream) {  // a batch upload not marked yet: everything queued on its stream
        CK(cudaStreamSynchronize(upload_stream));
        upload_stream = nullptr;
    }
    if (upload_mark) {
        CK(cudaEventSynchronize(upload_mark->ev));
        mark_drop(upload_mark);
        upload_mark = nullptr;
    }
    return MTGL_OK;
}

void HostStage::hold_upload(RunMark *m)
{
    if (upload_mark) mark_drop(upload_mark);
    mark_hold(m);
    upload_mark = m;
    upload_stream = nullptr;
}

int HostStage::reserve(size_t bytes, int64_t *off)
{
    int st = wait();
    if (st) return st;
    const size_t at = align16(used);
    if (at + bytes > cap) {
        if (fixed) {
            snprintf(g_err, sizeof(g_err), "staging area full (%zu of %zu bytes)", at + bytes, cap);
            return MTGL_ERR_OVERFLOW;
        }
        size_t ncap = std::max(at + bytes, cap * 2);
        ncap = std::max(ncap, (size_t)1 << 20);
        uint8_t *n = nullptr;
        CK(cudaMallocHost((void **)&n, ncap));
        allocs++;
        if (used) memcpy(n, p, used);
        if (p) cudaFreeHost(p);
        p = n;
        cap = ncap;
    }
    used = at + bytes;
    *off = (int64_t)at;
    return MTGL_OK;
}

// One core copies into pinned memory at a fraction of what host memory and the link to the
// GPU sustain, so a large client array is copied by several threads at once. One such copy
// runs at a time; a copy that finds another running (contexts on several threads) copies
// alone.
static std::atomic<bool> g_par_copy_busy{false};

static void par_copy(uint8_t *dst, const uint8_t *src, size_t bytes)
{
    const size_t kMin = (size_t)8 << 20, kPiece = (size_t)2 << 20;
    const unsigned hc = std::thread::hardware_concurrency();
    bool idle = false;
    if (bytes < kMin || hc < 2 || !g_par_copy_busy.compare_exchange_strong(idle, true)) {
        memcpy(dst, src, bytes);
        return;
    }
    const size_t n = std::min<size_t>(std::min<size_t>(hc, 8), bytes / kPiece);
    const size_t per = (bytes / n + 63) & ~(size_t)63;
    std::vector<std::thread> helpers;
    size_t done = std::min(per, bytes);  // this thread's piece
    try {
        for (size_t a = per; a < bytes; a += per) {
            const size_t len = std::min(per, bytes - a);
            helpers.emplace_back([=] { memcpy(dst + a, src + a, len); });
            done = a + len;
        }
    } catch (...) {  // no thread to be had: copy the rest here
    }
    memcpy(dst, src, std::min(per, bytes));
    if (done < bytes) memcpy(dst + done, src + done, bytes - done);
    for (std::thread &t : helpers) t.join();
    g_par_copy_busy.store(false);
}

int HostStage::copy(const void *src, size_t bytes, int64_t *off)
{
    int st = reserve(bytes, off);
    if (st) return st;
    if (bytes) par_copy(p + *off, static_cast<const uint8_t *>(src), bytes);
    return MTGL_OK;
}

int HostStage::mark_uploaded(cudaStream_t s)
{
    if (!done) CK(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    CK(cudaEventRecord(done, s));
    inflight = true;
    return MTGL_OK;
}

void HostStage::release()
{
    wait();
    if (p) cudaFreeHost(p);
    if (done) cudaEventDestroy(done);
    p = nullptr;
    done = nullptr;
    cap = used = 0;
    inflight = false;
}

void Pass::reset()
{
    clears.clear();
    draws.clear();
    vstates.clear();
    rasters.clear();
    raster_src.clear();
    needs_eye = false;
    slots = tris = vbytes = 0;
}

// ------------------------------------------------------------------ scratch

int PoolScratch::get(int slot, size_t bytes, void **out)
{
    if (bytes > cap[slot]) {
        const size_t ncap = std::max(bytes, cap[slot] + cap[slot] / 2);
        if (p[slot]) CK(cudaFreeAsync(p[slot], stream));
        p[slot] = nullptr;
        cap[slot] = 0;
        CK(cudaMallocAsync(&p[slot], ncap, stream));
        allocs++;
        cap[slot] = ncap;
    }
    *out = p[slot];
    return MTGL_OK;
}

void PoolScratch::release()
{
    for (int i = 0; i < kScratchSlots; i++) {
        if (p[i]) cudaFreeAsync(p[i], stream);
        p[i] = nullptr;
        cap[i] = 0;
    }
}

// ------------------------------------------------------------------ exec

int Exec::init(cudaStream_t s)
{
    CK(cudaGetDevice(&device));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    if (sms <= 0) sms = 1;
    if (s) {
        stream = s;
        own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
    }
    pool.stream = stream;
    CK(cudaMallocAsync((void **)&d_totals, 16 * sizeof(uint32_t), stream));
    CK(cudaMemsetAsync(d_totals, 0, 16 * sizeof(uint32_t), stream));
    CK(cudaMallocAsync((void **)&d_frags, sizeof(unsigned long long), stream));
    CK(cudaMemsetAsync(d_frags, 0, sizeof(unsigned long long), stream));
    CK(cudaMallocHost((void **)&h_totals, 16 * sizeof(uint32_t)));
    memset(h_totals, 0, 16 * sizeof(uint32_t));
    return MTGL_OK;
}

void Exec::destroy()
{
    if (!stream) return;
    cudaStreamSynchronize(stream);
    pool.release();
    if (dstage) cudaFreeAsync(dstage, stream);
    if (d_totals) cudaFreeAsync(d_totals, stream);
    if (d_frags) cudaFreeAsync(d_frags, stream);
    cudaStreamSynchronize(stream);
    if (h_totals) cudaFreeHost(h_totals);
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : ev_pending) cudaEventDestroy(e);
    ev_pool.clear();
    ev_pending.clear();
    if (own_stream) cudaStreamDestroy(stream);
    stream = nullptr;
    dstage = nullptr;
    d_totals = nullptr;
    d_frags = nullptr;
    h_totals = nullptr;
}

int Exec::ensure_dstage(size_t bytes, bool may_grow, size_t keep)
{
    if (bytes <= dcap) return MTGL_OK;
    if (!may_grow) {
        snprintf(g_err, sizeof(g_err), "device staging area full (%zu of %zu bytes)", bytes, dcap);
        return MTGL_ERR_OVERFLOW;
    }
    const size_t cap = std::max(bytes, dcap * 2);
    uint8_t *n = nullptr;
    CK(cudaMallocAsync((void **)&n, cap, stream));
    allocs++;
    if (dstage && keep) CK(cudaMemcpyAsync(n, dstage, std::min(keep, dcap), cudaMemcpyDeviceToDevice, stream));
    if (dstage) CK(cudaFreeAsync(dstage, stream));
    dstage = n;
    dcap = cap;
    return MTGL_OK;
}

void Exec::prof_mark()
{
    if (!profile) return;
    cudaEvent_t e = nullptr;
    if (!ev_pool.empty()) {
        e = ev_pool.back();
        ev_pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
        return;
    }
    cudaEventRecord(e, stream);
    ev_pending.push_back(e);
}

int Exec::prof_collect()
{
    const size_t n = ev_pending.size() / 5 * 5;
    for (size_t i = 0; i < n; i += 5) {
        float t[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; k++) CK(cudaEventElapsedTime(&t[k], ev_pending[i + k], ev_pending[i + k + 1]));
        timings.vertex_ms += t[0];
        timings.setup_ms += t[1];
        timings.bin_ms += t[2];
        timings.tile_ms += t[3];
        timings.passes++;
    }
    for (cudaEvent_t e : ev_pending) ev_pool.push_back(e);
    ev_pending.clear();
    return MTGL_OK;
}

// ------------------------------------------------------------------ tables

int build_tables(Exec &x, HostStage &st, const FrameSrc *frames, uint32_t nframes, int tile_shift, bool may_grow,
                 Tables &t, size_t direct)
{
    t = Tables();
    t.off_upload = (int64_t)direct;
    t.tile_shift = tile_shift;
    t.nframes = nframes;
    size_t ndraws = 0, nvs = 0, nrs = 0, ncl = 0;
    uint64_t slots = 0, tris = 0, ntiles = 0;
    const int ts = 1 << tile_shift;
    for (uint32_t f = 0; f < nframes; f++) {
        const Pass &p = *frames[f].pass;
        ndraws += p.draws.size();
        nvs += p.vstates.size();
        nrs += p.rasters.size();
        ncl += p.clears.size();
        slots += p.slots;
        tris += p.tris;
        t.eye = t.eye || p.needs_eye;
        const mtgl_dev *d = frames[f].dev;
        ntiles += (uint64_t)((d->width + ts - 1) / ts) * (uint64_t)((d->height + ts - 1) / ts);
    }
    if (slots > 0x7FFFFFFFull || tris > 0x7FFFFFFFull || ntiles > 0x3FFFFFFFull || nrs > 0xFFFFFFFFull) {
        snprintf(g_err, sizeof(g_err), "pass too large (%llu vertices, %llu triangles, %llu tiles)",
                 (unsigned long long)slots, (unsigned long long)tris, (unsigned long long)ntiles);
        return MTGL_ERR_INVALID;
    }
    const size_t used0 = st.used;
    int s;
    if ((s = st.reserve(std::max<size_t>(1, ndraws) * sizeof(DevDraw), &t.off_draws)) ||
        (s = st.reserve(std::max<size_t>(1, ndraws) * sizeof(uint32_t), &t.off_vbase)) ||
        (s = st.reserve(std::max<size_t>(1, ndraws) * sizeof(uint32_t), &t.off_tbase)) ||
        (s = st.reserve(std::max<size_t>(1, nvs) * sizeof(mtgl_vertex_state), &t.off_vs)) ||
        (s = st.reserve(std::max<size_t>(1, nrs) * sizeof(DevRaster), &t.off_rs)) ||
        (s = st.reserve(std::max<size_t>(1, ncl) * sizeof(ClearOp), &t.off_clears)) ||
        (s = st.reserve(std::max<uint32_t>(1, nframes) * sizeof(DevFrame), &t.off_frames)) ||
        (s = x.ensure_dstage(st.used, may_grow, direct))) {
        st.used = used0;
        return s;
    }
    uint8_t *ds = x.dstage;
    DevDraw *hd = reinterpret_cast<DevDraw *>(st.p + t.off_draws);
    uint32_t *hvb = reinterpret_cast<uint32_t *>(st.p + t.off_vbase);
    uint32_t *htb = reinterpret_cast<uint32_t *>(st.p + t.off_tbase);
    mtgl_vertex_state *hvs = reinterpret_cast<mtgl_vertex_state *>(st.p + t.off_vs);
    DevRaster *hrs = reinterpret_cast<DevRaster *>(st.p + t.off_rs);
    ClearOp *hcl = reinterpret_cast<ClearOp *>(st.p + t.off_clears);
    DevFrame *hfr = reinterpret_cast<DevFrame *>(st.p + t.off_frames);
    uint32_t di = 0, vsb = 0, rsb = 0, clb = 0, slot_base = 0, tri_base = 0, tile_base = 0;
    bool defer = true;
    for (uint32_t f = 0; f < nframes; f++) {
        const Pass &p = *frames[f].pass;
        const mtgl_dev *d = frames[f].dev;
        uint8_t *data = ds + frames[f].data_off;
        for (const PendingDraw &pd : p.draws) {
            DevDraw dd = pd.d;
            if (dd.mode < GL_TRIANGLES || dd.mode > GL_POLYGON || dd.raster >= p.rasters.size() ||
                p.rasters[dd.raster].rs.polygon_mode_front != GL_FILL ||
                p.rasters[dd.raster].rs.polygon_mode_back != GL_FILL)
                defer = false;  // points and lines read the stored colour
            if (pd.off_pos >= 0) dd.pos.ptr = data + pd.off_pos;
            if (pd.off_color >= 0) dd.color.ptr = data + pd.off_color;
            if (pd.off_tex >= 0) dd.tex.ptr = data + pd.off_tex;
            if (pd.off_normal >= 0) dd.normal.ptr = data + pd.off_normal;
            if (pd.off_idx >= 0) dd.indices = data + pd.off_idx;
            if (pd.off_vsid >= 0) dd.vs_ids = reinterpret_cast<const uint32_t *>(data + pd.off_vsid);
            dd.vs_base += vsb;
            dd.raster += rsb;
            dd.vslot_base += slot_base;
            dd.tri_base += tri_base;
            hd[di] = dd;
            hvb[di] = dd.vslot_base;
            htb[di] = dd.tri_base;
            di++;
        }
        if (!p.vstates.empty()) memcpy(hvs + vsb, p.vstates.data(), p.vstates.size() * sizeof(mtgl_vertex_state));
        for (size_t i = 0; i < p.rasters.size(); i++) {
            DevRaster R = p.rasters[i];
            R.frame = f;
            t.any_texture = t.any_texture || R.tex != nullptr;
            const uint32_t c = R.fs.ctl;
            if ((c & FC_BLEND) || ((c & FC_ALPHA) && (c & FC_TEXTURE)) || !(c & (FC_MASK_ALL | FC_MASK_NONE)))
                defer = false;  // a fragment reads the stored colour, or may be discarded after its depth test
            hrs[rsb + i] = R;
        }
        if (!p.clears.empty()) memcpy(hcl + clb, p.clears.data(), p.clears.size() * sizeof(ClearOp));
        DevFrame F;
        memset(&F, 0, sizeof(F));
        F.color = d->color;
        F.depth = d->depth;
        F.stencil = d->stencil;
        F.dims.width = d->width;
        F.dims.height = d->height;
        F.dims.tiles_x = (d->width + ts - 1) / ts;
        F.dims.tiles_y = (d->height + ts - 1) / ts;
        F.tile_base = tile_base;
        F.clear_base = clb;
        F.nclears = (uint32_t)p.clears.size();
        hfr[f] = F;
        vsb += (uint32_t)p.vstates.size();
        rsb += (uint32_t)p.rasters.size();
        clb += (uint32_t)p.clears.size();
        slot_base += (uint32_t)p.slots;
        tri_base += (uint32_t)p.tris;
        tile_base += (uint32_t)(F.dims.tiles_x * F.dims.tiles_y);
    }
    t.ndraws = (uint32_t)ndraws;
    t.nrasters = (uint32_t)nrs;
    t.defer = defer && ndraws > 0;
    t.nclears = (uint32_t)ncl;
    t.slots = (uint32_t)slots;
    t.tris = (uint32_t)tris;
    t.ntiles = (uint32_t)ntiles;
    return MTGL_OK;
}

int persistent_ctas(const Exec &x, const Tables &t, int per_sm)
{
    TileArgs probe;
    memset(&probe, 0, sizeof(probe));
    probe.tile_shift = t.tile_shift;
    probe.any_texture = t.any_texture ? 1 : 0;
    probe.defer = t.defer ? 1 : 0;
    probe.eye_records = t.eye ? reinterpret_cast<const float *>(1) : nullptr;
    const int occ = tile_occupancy(probe);
    const int n = per_sm > 0 ? std::min(per_sm, occ) : occ;
    return std::max(1, n) * x.sms;
}

// ------------------------------------------------------------------ the pipeline

int run_pipeline(Exec &x, ScratchSource &sc, const HostStage &st, const Tables &t, const PipeConfig &c,
                 PipeOut *out, bool alloc_only)
{
    cudaStream_t s = x.stream;
    uint8_t *ds = x.dstage;
    const uint32_t slots = t.slots, tris = t.tris, ntiles = t.ntiles;
    const bool eye = t.eye;
    int rc;
    PipeOut o;

    // scratch known before any count: vertices, triangle counts, tiles
    float4 *verts = nullptr;  // the three vertex streams, one after another
    PostEye *eyes = nullptr;
    uint32_t *tri_counts = nullptr, *tri_offsets = nullptr, *tile_count = nullptr, *tile_start = nullptr;
    uint32_t *scan_temp = nullptr, *order = nullptr, *order_aux = nullptr;
    float *records = nullptr, *eye_records = nullptr;
    uint32_t *rec_tiles = nullptr, *keys = nullptr, *vals = nullptr, *keys_alt = nullptr, *vals_alt = nullptr;
    uint32_t *radix_hist = nullptr;
    if ((rc = sc.take(S_VERTS, 3 * (size_t)slots, &verts))) return rc;
    if (eye && (rc = sc.take(S_EYES, slots, &eyes))) return rc;
    if ((rc = sc.take(S_TRI_COUNTS, tris, &tri_counts))) return rc;
    if ((rc = sc.take(S_TRI_OFFSETS, tris, &tri_offsets))) return rc;
    // clip list, its class words, the class-sorted list, the class counters and the emit list
    uint32_t *clip_list = nullptr;
    if ((rc = sc.take(S_CLIP_LIST, 4 * (size_t)tris + kClipBuckets, &clip_list))) return rc;
    // tile counts, then (persistent ordered launches) the per-tile record-box coverage
    if ((rc = sc.take(S_TILE_COUNT, 2 * ((size_t)ntiles + 1), &tile_count))) return rc;
    // record-box coverage per tile, for the split between tiles run by rounds and per record;
    // deferred-colour passes run every tile per record (their fragments are cheap: tests only)
    uint32_t *tile_area = (c.ctas && (c.order || c.classify) && !t.defer) ? tile_count + ntiles + 1 : nullptr;
    if ((rc = sc.take(S_TILE_START, (size_t)ntiles + 1, &tile_start))) return rc;
    uint32_t *tile_frame = nullptr;  // batches: each tile's frame, found once by the range pass
    if (t.nframes > 1 && (rc = sc.take(S_TILE_FRAME, ntiles, &tile_frame))) return rc;
    if (c.ctas && c.order && (rc = sc.take(S_ORDER, ntiles, &order))) return rc;
    if (c.ctas && (rc = sc.take(S_ORDER_AUX, kOrderAuxWords, &order_aux))) return rc;
    uint32_t scan_n = std::max<uint32_t>(std::max(tris, ntiles), 1);
    if (!c.exact) {
        scan_n = std::max<uint32_t>(scan_n, c.rec_cap);
        scan_n = std::max<uint32_t>(scan_n, (uint32_t)radix_hist_words(c.pair_cap));
        if ((rc = sc.take(S_RECORDS, (size_t)c.rec_cap * kRecWords, &records))) return rc;
        if (eye && (rc = sc.take(S_EYE_RECORDS, (size_t)c.rec_cap * kEyeWords, &eye_records))) return rc;
        if ((rc = sc.take(S_REC_TILES, c.rec_cap, &rec_tiles))) return rc;
        if ((rc = sc.take(S_KEYS, c.pair_cap, &keys))) return rc;
        if ((rc = sc.take(S_VALS, c.pair_cap, &vals))) return rc;
        if ((rc = sc.take(S_KEYS_ALT, c.pair_cap, &keys_alt))) return rc;
        if ((rc = sc.take(S_VALS_ALT, c.pair_cap, &vals_alt))) return rc;
        if ((rc = sc.take(S_RADIX_HIST, radix_hist_words(c.pair_cap), &radix_hist))) return rc;
    }
    if ((rc = sc.take(S_SCAN_TEMP, scan_temp_words(scan_n), &scan_temp))) return rc;
    if (alloc_only) return MTGL_OK;

    CK(cudaMemcpyAsync(ds + t.off_upload, st.p + t.off_upload, st.used - (size_t)t.off_upload, cudaMemcpyHostToDevice,
                       s));
    x.prof_mark();

    GeomArgs ga;
    memset(&ga, 0, sizeof(ga));
    ga.draws = reinterpret_cast<const DevDraw *>(ds + t.off_draws);
    ga.draw_vslot_base = reinterpret_cast<const uint32_t *>(ds + t.off_vbase);
    ga.draw_tri_base = reinterpret_cast<const uint32_t *>(ds + t.off_tbase);
    ga.ndraws = (int32_t)t.ndraws;
    ga.vstates = reinterpret_cast<const mtgl_vertex_state *>(ds + t.off_vs);
    ga.rasters = reinterpret_cast<const DevRaster *>(ds + t.off_rs);
    ga.frames = reinterpret_cast<const DevFrame *>(ds + t.off_frames);
    ga.nframes = t.nframes;
    ga.verts = PostVertices{verts, verts + slots, verts + 2 * (size_t)slots};
    ga.eyes = eyes;
    ga.total_slots = slots;
    ga.total_tris = tris;
    ga.tri_counts = tri_counts;
    ga.tri_offsets = tri_offsets;
    ga.clip_list = clip_list;
    ga.clip_class = clip_list + tris;
    // sort by class below 2^24 triangles: a bucket then holds under 2^20 entries (its blocks
    // are every kClipSlots-th of 128 triangles), so a rank fits the class word's 20 bits
    ga.clip_sorted = tris < (1u << 24) ? clip_list + 2 * (size_t)tris : nullptr;
    ga.class_count = clip_list + 3 * (size_t)tris;
    ga.emit_list = clip_list + 3 * (size_t)tris + kClipBuckets;
    ga.list_counts = x.d_totals + 4;
    ga.debug = x.d_totals + kDebugStatusWord;
    ga.sms = x.sms;
    int launches = 0;
    launches += launch_vertex(ga, s);
    x.prof_mark();
    launches += launch_setup_count(ga, s);
    launches += launch_scan(tri_counts, tri_offsets, tris, scan_temp, x.d_totals + 0, x.d_totals + kDebugStatusWord, s);
    CK(cudaGetLastError());

    uint32_t rec_cap = c.rec_cap;
    if (c.exact) {
        CK(cudaMemcpyAsync(x.h_totals, x.d_totals, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        rec_cap = o.nrec = x.h_totals[0];
        if ((rc = sc.take(S_RECORDS, (size_t)rec_cap * kRecWords, &records))) return rc;
        if (eye && (rc = sc.take(S_EYE_RECORDS, (size_t)rec_cap * kEyeWords, &eye_records))) return rc;
        if ((rc = sc.take(S_REC_TILES, rec_cap, &rec_tiles))) return rc;
        if (rec_cap > scan_n) {
            scan_n = rec_cap;
            if ((rc = sc.take(S_SCAN_TEMP, scan_temp_words(scan_n), &scan_temp))) return rc;
        }
    }
    ga.records = records;
    ga.eye_records = eye_records;
    ga.records_cap = rec_cap;
    launches += launch_setup_emit(ga, s);
    x.prof_mark();

    // ---- binning
    CK(cudaMemsetAsync(tile_count, 0, (tile_area ? 2 : 1) * ((size_t)ntiles + 1) * sizeof(uint32_t), s));
    CK(cudaMemsetAsync(tile_start, 0, ((size_t)ntiles + 1) * sizeof(uint32_t), s));
    BinArgs ba;
    memset(&ba, 0, sizeof(ba));
    ba.records = records;
    ba.nrec = rec_cap;
    ba.nrec_dev = x.d_totals + 0;
    ba.frames = ga.frames;
    ba.nframes = t.nframes;
    ba.tile_shift = t.tile_shift;
    ba.ntiles = ntiles;
    ba.rec_tiles = rec_tiles;
    ba.tile_count = tile_count;
    ba.tile_area = tile_area;
    ba.tile_start = tile_start;
    ba.tile_frame = tile_frame;
    ba.total_dev = x.d_totals + 1;
    ba.sort_total_dev = x.d_totals + 3;
    ba.debug = x.d_totals + kDebugStatusWord;
    ba.scan_temp = scan_temp;
    ba.sms = x.sms;
    uint32_t pair_cap = c.pair_cap;
    if (rec_cap) {
        launches += launch_bin_count(ba, s);
        launches += launch_scan(rec_tiles, rec_tiles, rec_cap, scan_temp, x.d_totals + 1, x.d_totals + kDebugStatusWord, s);
        CK(cudaGetLastError());
        if (c.exact) {
            CK(cudaMemcpyAsync(x.h_totals + 1, x.d_totals + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            pair_cap = o.npairs = x.h_totals[1];
            const size_t hist = radix_hist_words(pair_cap);
            if ((rc = sc.take(S_KEYS, pair_cap, &keys)) || (rc = sc.take(S_VALS, pair_cap, &vals)) ||
                (rc = sc.take(S_KEYS_ALT, pair_cap, &keys_alt)) || (rc = sc.take(S_VALS_ALT, pair_cap, &vals_alt)) ||
                (rc = sc.take(S_RADIX_HIST, hist, &radix_hist)))
                return rc;
            const uint32_t need = std::max<uint32_t>(std::max<uint32_t>((uint32_t)hist, rec_cap), scan_n);
            if ((rc = sc.take(S_SCAN_TEMP, scan_temp_words(need), &scan_temp))) return rc;
            ba.scan_temp = scan_temp;
        }
        ba.keys = keys;
        ba.vals = vals;
        ba.keys_alt = keys_alt;
        ba.vals_alt = vals_alt;
        ba.radix_hist = radix_hist;
        ba.npairs = pair_cap;
        launches += launch_bin_expand(ba, s);
        launches += launch_bin_sort(ba, s);
        launches += launch_tile_ranges(ba, s);
    } else {
        CK(cudaMemsetAsync(x.d_totals + 1, 0, sizeof(uint32_t), s));
    }
    x.prof_mark();

    TileArgs ta;
    memset(&ta, 0, sizeof(ta));
    ta.records = records;
    ta.eye_records = eye_records;
    ta.tile_vals = rec_cap ? ba.vals : nullptr;
    ta.pair_mask = rec_cap ? ba.keys : nullptr;
    ta.debug = x.d_totals + kDebugStatusWord;
    ta.records_cap = rec_cap;
    ta.entries_cap = rec_cap ? pair_cap : 0u;
    ta.tile_start = tile_start;
    ta.tile_count = tile_count;
    ta.tile_frame = rec_cap ? tile_frame : nullptr;  // written by the range pass, which runs with records
    ta.rasters = ga.rasters;
    ta.nrasters = std::max<uint32_t>(1, t.nrasters);
    ta.clears = reinterpret_cast<const ClearOp *>(ds + t.off_clears);
    ta.frames = ga.frames;
    ta.nframes = t.nframes;
    ta.ntiles = ntiles;
    ta.tile_shift = t.tile_shift;
    ta.any_texture = t.any_texture ? 1 : 0;
    ta.defer = t.defer ? 1 : 0;
    ta.fragments = x.d_frags;
    if (c.ctas) {
        ta.queue = order_aux + kOrderQueues;
        if (order) {  // clears the queue heads too
            launches += launch_tile_order(tile_count, tile_area, ntiles, t.tile_shift, order_aux, order, x.sms, s);
            ta.order = order;
            ta.split = order_aux + kOrderSplit;
        } else {
            CK(cudaMemsetAsync(ta.queue, 0, 2 * sizeof(uint32_t), s));
            ta.tile_area = tile_area;  // classes, tile order
        }
        ta.ctas = c.ctas;
    }
    if (!c.exact) {
        ta.guard = x.d_totals;
        ta.pairs_cap = pair_cap;
    }
    launches += launch_tile(ta, s);
    x.prof_mark();
    CK(cudaGetLastError());
    if (!c.exact) CK(cudaMemcpyAsync(x.h_totals, x.d_totals, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    o.launches = launches;
    if (out) *out = o;
    return MTGL_OK;
}

}  // namespace mtgl
