// dev_runtime.cu — the mtgl_dev C ABI of the GB300 back end (include/mytinygl/mtgl_dev.h).
//
// One mtgl_dev per GL context: the framebuffer in device memory (row-major, row 0 = top,
// colour u32 a<<24|b<<16|g<<8|r, depth f32, stencil u8, as src/framebuffer.h:19-25), one
// CUDA stream, resource storage (buffer objects, textures with their mip level 1) and the
// pending pass. A pass is a run of clears followed by draws. Draws are queued with their
// state blocks; client memory they borrow is copied into pinned staging at enqueue time.
// A flush uploads the staging area with one copy and runs K1 vertex -> K2 setup count ->
// scan -> K2 emit -> K3 bin -> K4 tile over the whole pass. Anything that must observe the
// framebuffer or change a resource a queued draw reads flushes first, and every device
// operation of a context runs on its one stream, so GL submission order is preserved.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "dev_kernels.h"
#include "mytinygl/mytinygl.h"

using namespace mtgl;

namespace {

thread_local char g_err[512] = "";

int fail_cuda(const char *what, cudaError_t e)
{
    snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
    return MTGL_ERR_CUDA;
}

#define CK(call)                                             \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return fail_cuda(#call, e_);  \
    } while (0)

struct DevBufferObj {
    uint8_t *ptr = nullptr;
    uint64_t size = 0;
};

struct DevTextureObj {
    uint32_t *base = nullptr;
    uint32_t *mip1 = nullptr;
    int32_t w = 0, h = 0, mw = 0, mh = 0;
};

template <class T>
struct Scratch {
    T *p = nullptr;
    size_t cap = 0;  // elements
};

// Pending draw: a DevDraw whose pointers are patched at flush for staged sources.
struct PendingDraw {
    DevDraw d;
    int64_t off_pos = -1, off_color = -1, off_tex = -1, off_normal = -1, off_idx = -1, off_vsid = -1;
};

size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

}  // namespace

struct mtgl_dev {
    int device = 0;
    cudaStream_t stream = nullptr;
    FrameDims dims{};
    uint32_t *color = nullptr;
    float *depth = nullptr;
    uint8_t *stencil = nullptr;

    std::vector<ClearOp> clears;
    std::vector<PendingDraw> draws;
    std::vector<mtgl_vertex_state> vstates;
    std::vector<DevRaster> rasters;
    std::vector<mtgl_raster_state> raster_src;  // for de-duplication
    bool pass_needs_eye = false;
    uint64_t slots = 0, tris = 0;

    uint8_t *hstage = nullptr;  // pinned
    size_t hcap = 0, hused = 0;
    uint8_t *dstage = nullptr;
    size_t dcap = 0;
    cudaEvent_t stage_done = nullptr;
    bool stage_inflight = false;

    Scratch<PostVertex> verts;
    Scratch<PostEye> eyes;
    Scratch<uint32_t> tri_counts, tri_offsets, rec_tiles, keys, vals, keys_alt, vals_alt, tile_count, tile_start,
        radix_hist, scan_temp;
    Scratch<float> records, eye_records;
    uint32_t *d_totals = nullptr;  // device: [0] records, [1] pairs, [2..] scratch
    uint32_t *h_totals = nullptr;  // pinned
    unsigned long long *d_frags = nullptr;
    mtgl_stats stats{};

    // per-phase profiling: 5 events per pass (before K1, after K1, after K2, after K3, after K4)
    bool profile = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<cudaEvent_t> ev_pending;
    mtgl_timings timings{};
    bool depth_rejection = true;
};

namespace {

template <class T>
int ensure(mtgl_dev *d, Scratch<T> &s, size_t n)
{
    if (n <= s.cap) return MTGL_OK;
    size_t cap = std::max(n, s.cap + s.cap / 2);
    if (s.p) CK(cudaFreeAsync(s.p, d->stream));
    s.p = nullptr;
    s.cap = 0;
    CK(cudaMallocAsync((void **)&s.p, cap * sizeof(T), d->stream));
    s.cap = cap;
    return MTGL_OK;
}

template <class T>
void release(mtgl_dev *d, Scratch<T> &s)
{
    if (s.p) cudaFreeAsync(s.p, d->stream);
    s.p = nullptr;
    s.cap = 0;
}

// Host staging must not be rewritten while the previous pass's upload is in flight.
int stage_begin(mtgl_dev *d)
{
    if (d->stage_inflight) {
        CK(cudaEventSynchronize(d->stage_done));
        d->stage_inflight = false;
    }
    return MTGL_OK;
}

int stage_reserve(mtgl_dev *d, size_t bytes, int64_t *off)
{
    int st = stage_begin(d);
    if (st) return st;
    size_t at = align16(d->hused);
    if (at + bytes > d->hcap) {
        size_t cap = std::max(at + bytes, d->hcap * 2);
        cap = std::max(cap, (size_t)1 << 20);
        uint8_t *n = nullptr;
        CK(cudaMallocHost((void **)&n, cap));
        if (d->hused) memcpy(n, d->hstage, d->hused);
        if (d->hstage) cudaFreeHost(d->hstage);
        d->hstage = n;
        d->hcap = cap;
    }
    d->hused = at + bytes;
    *off = (int64_t)at;
    return MTGL_OK;
}

int stage_copy(mtgl_dev *d, const void *src, size_t bytes, int64_t *off)
{
    int st = stage_reserve(d, bytes, off);
    if (st) return st;
    if (bytes) memcpy(d->hstage + *off, src, bytes);
    return MTGL_OK;
}

uint64_t triangles_of(uint32_t mode, int64_t n)
{
    switch (mode) {
    case GL_TRIANGLES: return (uint64_t)(n / 3);
    case GL_TRIANGLE_STRIP:
    case GL_TRIANGLE_FAN:
    case GL_POLYGON: return n >= 3 ? (uint64_t)(n - 2) : 0;
    case GL_QUADS: return 2 * (uint64_t)(n / 4);
    case GL_QUAD_STRIP: return n >= 4 ? 2 * (uint64_t)((n - 2) / 2) : 0;
    default: return 0;
    }
}

int index_size(uint32_t type)
{
    return type == GL_UNSIGNED_INT ? 4 : (type == GL_UNSIGNED_SHORT ? 2 : 1);
}

uint32_t push_raster(mtgl_dev *d, const mtgl_raster_state *rs)
{
    if (!d->raster_src.empty() && memcmp(&d->raster_src.back(), rs, sizeof(*rs)) == 0)
        return (uint32_t)(d->rasters.size() - 1);
    DevRaster R;
    memset(&R, 0, sizeof(R));
    R.rs = *rs;
    const DevTextureObj *t = reinterpret_cast<const DevTextureObj *>(rs->texture);
    if (t && t->base) {
        R.tex = t->base;
        R.tex_w = t->w;
        R.tex_h = t->h;
        R.mip1 = t->mip1;
        R.mip_w = t->mw;
        R.mip_h = t->mh;
    }
    R.default_depth_range = (rs->depth_near == 0.0 && rs->depth_far == 1.0) ? 1 : 0;
    R.needs_eye = (rs->lighting && (rs->shade_model == GL_PHONG || rs->lit.two_side)) ? 1 : 0;
    R.depth_rejection = d->depth_rejection ? 1 : 0;
    if (R.needs_eye) d->pass_needs_eye = true;
    d->raster_src.push_back(*rs);
    d->rasters.push_back(R);
    return (uint32_t)(d->rasters.size() - 1);
}

uint32_t push_vstates(mtgl_dev *d, const mtgl_vertex_state *vs, uint32_t n)
{
    if (n == 1 && !d->vstates.empty() && memcmp(&d->vstates.back(), vs, sizeof(*vs)) == 0)
        return (uint32_t)(d->vstates.size() - 1);
    uint32_t base = (uint32_t)d->vstates.size();
    d->vstates.insert(d->vstates.end(), vs, vs + n);
    return base;
}

// Resolve one attribute stream. Client memory is copied for element range [lo, hi].
int resolve_attr(mtgl_dev *d, const mtgl_attrib &a, int64_t lo, int64_t hi, DevAttrib &out, int64_t &off)
{
    memset(&out, 0, sizeof(out));
    off = -1;
    if (!a.enabled) return MTGL_OK;
    out.enabled = 1;
    out.size = a.size;
    out.type = a.type;
    out.stride = a.stride;
    const int comp = a.type == GL_FLOAT ? 4 : 1;
    if (a.buffer) {
        const DevBufferObj *b = reinterpret_cast<const DevBufferObj *>(a.buffer);
        if (b->ptr && a.offset < b->size) {
            out.ptr = b->ptr + a.offset;
            out.bytes = std::min<uint64_t>(a.bytes, b->size - a.offset);
        }
        out.base_index = 0;
        return MTGL_OK;
    }
    if (!a.host || hi < lo || a.stride <= 0) return MTGL_OK;
    const size_t bytes = (size_t)(hi - lo) * (size_t)a.stride + (size_t)a.size * comp;
    int st = stage_copy(d, (const uint8_t *)a.host + (size_t)lo * (size_t)a.stride, bytes, &off);
    if (st) return st;
    out.base_index = lo;
    out.bytes = bytes;
    return MTGL_OK;
}

int flush_pass(mtgl_dev *d);

cudaEvent_t prof_event(mtgl_dev *d)
{
    cudaEvent_t e = nullptr;
    if (!d->ev_pool.empty()) {
        e = d->ev_pool.back();
        d->ev_pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
        return nullptr;
    }
    return e;
}

void prof_mark(mtgl_dev *d)
{
    if (!d->profile) return;
    cudaEvent_t e = prof_event(d);
    if (!e) return;
    cudaEventRecord(e, d->stream);
    d->ev_pending.push_back(e);
}

// fold completed passes' events into the sums (the caller has synchronised the stream)
int prof_collect(mtgl_dev *d)
{
    const size_t n = d->ev_pending.size() / 5 * 5;
    for (size_t i = 0; i < n; i += 5) {
        float t[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; k++) CK(cudaEventElapsedTime(&t[k], d->ev_pending[i + k], d->ev_pending[i + k + 1]));
        d->timings.vertex_ms += t[0];
        d->timings.setup_ms += t[1];
        d->timings.bin_ms += t[2];
        d->timings.tile_ms += t[3];
        d->timings.passes++;
    }
    for (size_t i = 0; i < d->ev_pending.size(); i++) d->ev_pool.push_back(d->ev_pending[i]);
    d->ev_pending.clear();
    return MTGL_OK;
}

int flush_if_drawing(mtgl_dev *d)
{
    if (!d->draws.empty()) return flush_pass(d);
    return MTGL_OK;
}

int run_clears_only(mtgl_dev *d)
{
    if (d->clears.empty()) return MTGL_OK;
    launch_clear(d->clears.data(), (int)d->clears.size(), d->dims, d->color, d->depth, d->stencil, d->stream);
    d->stats.kernel_launches += (d->clears.size() + 15) / 16;
    d->stats.passes++;
    d->clears.clear();
    CK(cudaGetLastError());
    return MTGL_OK;
}

int flush_pass(mtgl_dev *d)
{
    if (d->draws.empty()) return run_clears_only(d);
    const size_t ndraws = d->draws.size();
    int st;

    // ---- tables go to the end of the staging area; patch device pointers first
    int64_t off_draws, off_vbase, off_tbase, off_vs, off_rs, off_clears;
    if ((st = stage_reserve(d, ndraws * sizeof(DevDraw), &off_draws))) return st;
    if ((st = stage_reserve(d, ndraws * sizeof(uint32_t), &off_vbase))) return st;
    if ((st = stage_reserve(d, ndraws * sizeof(uint32_t), &off_tbase))) return st;
    if ((st = stage_reserve(d, d->vstates.size() * sizeof(mtgl_vertex_state), &off_vs))) return st;
    if ((st = stage_reserve(d, d->rasters.size() * sizeof(DevRaster), &off_rs))) return st;
    if ((st = stage_reserve(d, std::max<size_t>(1, d->clears.size()) * sizeof(ClearOp), &off_clears))) return st;
    if (d->hused > d->dcap) {
        if (d->dstage) CK(cudaFreeAsync(d->dstage, d->stream));
        d->dstage = nullptr;
        size_t cap = std::max(d->hused, d->dcap * 2);
        CK(cudaMallocAsync((void **)&d->dstage, cap, d->stream));
        d->dcap = cap;
    }
    uint8_t *ds = d->dstage;
    DevDraw *hd = reinterpret_cast<DevDraw *>(d->hstage + off_draws);
    uint32_t *hvb = reinterpret_cast<uint32_t *>(d->hstage + off_vbase);
    uint32_t *htb = reinterpret_cast<uint32_t *>(d->hstage + off_tbase);
    for (size_t i = 0; i < ndraws; i++) {
        PendingDraw &p = d->draws[i];
        DevDraw dd = p.d;
        if (p.off_pos >= 0) dd.pos.ptr = ds + p.off_pos;
        if (p.off_color >= 0) dd.color.ptr = ds + p.off_color;
        if (p.off_tex >= 0) dd.tex.ptr = ds + p.off_tex;
        if (p.off_normal >= 0) dd.normal.ptr = ds + p.off_normal;
        if (p.off_idx >= 0) dd.indices = ds + p.off_idx;
        if (p.off_vsid >= 0) dd.vs_ids = reinterpret_cast<const uint32_t *>(ds + p.off_vsid);
        hd[i] = dd;
        hvb[i] = dd.vslot_base;
        htb[i] = dd.tri_base;
    }
    if (!d->vstates.empty())
        memcpy(d->hstage + off_vs, d->vstates.data(), d->vstates.size() * sizeof(mtgl_vertex_state));
    memcpy(d->hstage + off_rs, d->rasters.data(), d->rasters.size() * sizeof(DevRaster));
    if (!d->clears.empty()) memcpy(d->hstage + off_clears, d->clears.data(), d->clears.size() * sizeof(ClearOp));
    CK(cudaMemcpyAsync(d->dstage, d->hstage, d->hused, cudaMemcpyHostToDevice, d->stream));
    CK(cudaEventRecord(d->stage_done, d->stream));
    d->stage_inflight = true;

    const uint32_t slots = (uint32_t)d->slots, tris = (uint32_t)d->tris;
    const bool eye = d->pass_needs_eye;
    if ((st = ensure(d, d->verts, std::max<size_t>(1, slots)))) return st;
    if (eye && (st = ensure(d, d->eyes, std::max<size_t>(1, slots)))) return st;
    if ((st = ensure(d, d->tri_counts, std::max<size_t>(1, tris)))) return st;
    if ((st = ensure(d, d->tri_offsets, std::max<size_t>(1, tris)))) return st;
    const uint32_t ntiles = (uint32_t)(d->dims.tiles_x * d->dims.tiles_y);
    if ((st = ensure(d, d->scan_temp, scan_temp_words(std::max<uint32_t>(std::max(tris, ntiles), 1))))) return st;

    GeomArgs ga;
    memset(&ga, 0, sizeof(ga));
    ga.draws = reinterpret_cast<const DevDraw *>(ds + off_draws);
    ga.draw_vslot_base = reinterpret_cast<const uint32_t *>(ds + off_vbase);
    ga.draw_tri_base = reinterpret_cast<const uint32_t *>(ds + off_tbase);
    ga.ndraws = (int32_t)ndraws;
    ga.vstates = reinterpret_cast<const mtgl_vertex_state *>(ds + off_vs);
    ga.rasters = reinterpret_cast<const DevRaster *>(ds + off_rs);
    ga.verts = d->verts.p;
    ga.eyes = eye ? d->eyes.p : nullptr;
    ga.total_slots = slots;
    ga.total_tris = tris;
    ga.dims = d->dims;
    ga.tri_counts = d->tri_counts.p;
    ga.tri_offsets = d->tri_offsets.p;

    int launches = 0;
    prof_mark(d);
    launches += launch_vertex(ga, d->stream);
    prof_mark(d);
    launches += launch_setup_count(ga, d->stream);
    launches += launch_scan(d->tri_counts.p, d->tri_offsets.p, tris, d->scan_temp.p, d->d_totals + 0, d->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(d->h_totals, d->d_totals, sizeof(uint32_t), cudaMemcpyDeviceToHost, d->stream));
    CK(cudaStreamSynchronize(d->stream));
    const uint32_t nrec = d->h_totals[0];

    if ((st = ensure(d, d->records, std::max<size_t>(1, (size_t)nrec * kRecWords)))) return st;
    if (eye && (st = ensure(d, d->eye_records, std::max<size_t>(1, (size_t)nrec * kEyeWords)))) return st;
    ga.records = d->records.p;
    ga.eye_records = eye ? d->eye_records.p : nullptr;
    ga.records_cap = nrec;
    launches += launch_setup_emit(ga, d->stream);
    prof_mark(d);

    // ---- binning
    if ((st = ensure(d, d->tile_count, ntiles + 1))) return st;
    if ((st = ensure(d, d->tile_start, ntiles + 1))) return st;
    CK(cudaMemsetAsync(d->tile_count.p, 0, (ntiles + 1) * sizeof(uint32_t), d->stream));
    BinArgs ba;
    memset(&ba, 0, sizeof(ba));
    ba.records = d->records.p;
    ba.nrec = nrec;
    ba.dims = d->dims;
    ba.tile_count = d->tile_count.p;
    ba.tile_start = d->tile_start.p;
    ba.total_dev = d->d_totals + 1;
    uint32_t npairs = 0;
    if (nrec) {
        if ((st = ensure(d, d->rec_tiles, nrec))) return st;
        if ((st = ensure(d, d->scan_temp, scan_temp_words(std::max(nrec, ntiles))))) return st;
        ba.rec_tiles = d->rec_tiles.p;
        ba.scan_temp = d->scan_temp.p;
        launches += launch_bin_count(ba, d->stream);
        launches += launch_scan(d->rec_tiles.p, d->rec_tiles.p, nrec, d->scan_temp.p, d->d_totals + 1, d->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(d->h_totals + 1, d->d_totals + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, d->stream));
        CK(cudaStreamSynchronize(d->stream));
        npairs = d->h_totals[1];
        if ((st = ensure(d, d->keys, std::max<uint32_t>(1, npairs)))) return st;
        if ((st = ensure(d, d->vals, std::max<uint32_t>(1, npairs)))) return st;
        if ((st = ensure(d, d->keys_alt, std::max<uint32_t>(1, npairs)))) return st;
        if ((st = ensure(d, d->vals_alt, std::max<uint32_t>(1, npairs)))) return st;
        if ((st = ensure(d, d->radix_hist, radix_hist_words(npairs)))) return st;
        if ((st = ensure(d, d->scan_temp, scan_temp_words(std::max<uint32_t>(
                                              std::max<uint32_t>((uint32_t)radix_hist_words(npairs), nrec), ntiles)))))
            return st;
        ba.scan_temp = d->scan_temp.p;
        ba.keys = d->keys.p;
        ba.vals = d->vals.p;
        ba.keys_alt = d->keys_alt.p;
        ba.vals_alt = d->vals_alt.p;
        ba.radix_hist = d->radix_hist.p;
        ba.npairs = npairs;
        ba.pairs_cap = npairs;
        launches += launch_bin_expand(ba, d->stream);
        launches += launch_bin_sort(ba, d->stream);
    }
    launches += launch_scan(d->tile_count.p, d->tile_start.p, ntiles, d->scan_temp.p, d->d_totals + 2, d->stream);
    prof_mark(d);

    TileArgs ta;
    memset(&ta, 0, sizeof(ta));
    ta.records = d->records.p;
    ta.eye_records = eye ? d->eye_records.p : nullptr;
    ta.tile_vals = nrec ? ba.vals : nullptr;
    ta.tile_start = d->tile_start.p;
    ta.tile_count = d->tile_count.p;
    ta.rasters = ga.rasters;
    ta.nrasters = (uint32_t)d->rasters.size();
    ta.clears = reinterpret_cast<const ClearOp *>(ds + off_clears);
    ta.nclears = (int32_t)d->clears.size();
    ta.any_texture = 0;
    for (const DevRaster &R : d->rasters) ta.any_texture |= R.tex != nullptr;
    ta.dims = d->dims;
    ta.color = d->color;
    ta.depth = d->depth;
    ta.stencil = d->stencil;
    ta.fragments = d->d_frags;
    launches += launch_tile(ta, d->stream);
    prof_mark(d);
    CK(cudaGetLastError());

    d->stats.passes++;
    d->stats.input_triangles += tris;
    d->stats.setup_triangles += nrec;
    d->stats.bin_entries += npairs;
    d->stats.kernel_launches += (uint64_t)launches;

    d->draws.clear();
    d->clears.clear();
    d->vstates.clear();
    d->rasters.clear();
    d->raster_src.clear();
    d->pass_needs_eye = false;
    d->slots = d->tris = 0;
    d->hused = 0;
    return MTGL_OK;
}

}  // namespace

extern "C" {

const char *mtgl_dev_last_error(void) { return g_err; }
const char *mtgl_dev_backend_name(void) { return "cuda-sm_103a"; }

int mtgl_dev_create(int32_t width, int32_t height, mtgl_dev **out)
{
    if (!out || width <= 0 || height <= 0) return MTGL_ERR_INVALID;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        snprintf(g_err, sizeof(g_err), "no CUDA device (%s)", e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
        return MTGL_ERR_NO_DEVICE;
    }
    mtgl_dev *d = new (std::nothrow) mtgl_dev();
    if (!d) return MTGL_ERR_OOM;
    CK(cudaGetDevice(&d->device));
    d->dims.width = width;
    d->dims.height = height;
    d->dims.tiles_x = (width + kTile - 1) / kTile;
    d->dims.tiles_y = (height + kTile - 1) / kTile;
    const size_t np = (size_t)width * (size_t)height;
    CK(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&d->stage_done, cudaEventDisableTiming));
    CK(cudaMallocAsync((void **)&d->color, np * 4, d->stream));
    CK(cudaMallocAsync((void **)&d->depth, np * 4, d->stream));
    CK(cudaMallocAsync((void **)&d->stencil, np, d->stream));
    CK(cudaMemsetAsync(d->color, 0, np * 4, d->stream));
    CK(cudaMemsetAsync(d->depth, 0, np * 4, d->stream));
    CK(cudaMemsetAsync(d->stencil, 0, np, d->stream));
    CK(cudaMallocAsync((void **)&d->d_totals, 16 * sizeof(uint32_t), d->stream));
    CK(cudaMallocAsync((void **)&d->d_frags, sizeof(unsigned long long), d->stream));
    CK(cudaMemsetAsync(d->d_frags, 0, sizeof(unsigned long long), d->stream));
    CK(cudaMallocHost((void **)&d->h_totals, 16 * sizeof(uint32_t)));
    CK(cudaStreamSynchronize(d->stream));
    *out = d;
    return MTGL_OK;
}

int mtgl_dev_destroy(mtgl_dev *d)
{
    if (!d) return MTGL_OK;
    cudaSetDevice(d->device);
    cudaStreamSynchronize(d->stream);
    release(d, d->verts);
    release(d, d->eyes);
    release(d, d->tri_counts);
    release(d, d->tri_offsets);
    release(d, d->rec_tiles);
    release(d, d->keys);
    release(d, d->vals);
    release(d, d->keys_alt);
    release(d, d->vals_alt);
    release(d, d->tile_count);
    release(d, d->tile_start);
    release(d, d->radix_hist);
    release(d, d->scan_temp);
    release(d, d->records);
    release(d, d->eye_records);
    if (d->dstage) cudaFreeAsync(d->dstage, d->stream);
    cudaFreeAsync(d->color, d->stream);
    cudaFreeAsync(d->depth, d->stream);
    cudaFreeAsync(d->stencil, d->stream);
    cudaFreeAsync(d->d_totals, d->stream);
    cudaFreeAsync(d->d_frags, d->stream);
    cudaStreamSynchronize(d->stream);
    if (d->hstage) cudaFreeHost(d->hstage);
    if (d->h_totals) cudaFreeHost(d->h_totals);
    cudaEventDestroy(d->stage_done);
    for (cudaEvent_t e : d->ev_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : d->ev_pending) cudaEventDestroy(e);
    cudaStreamDestroy(d->stream);
    delete d;
    return MTGL_OK;
}

// ---- resources: a change flushes queued draws first, so they read the old contents

int mtgl_dev_buffer_create(mtgl_dev *d, mtgl_handle *out)
{
    if (!d || !out) return MTGL_ERR_INVALID;
    DevBufferObj *b = new (std::nothrow) DevBufferObj();
    if (!b) return MTGL_ERR_OOM;
    *out = (mtgl_handle)(uintptr_t)b;
    return MTGL_OK;
}

int mtgl_dev_buffer_data(mtgl_dev *d, mtgl_handle h, const void *data, uint64_t bytes)
{
    DevBufferObj *b = reinterpret_cast<DevBufferObj *>(h);
    if (!d || !b) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);
    if (st) return st;
    if (b->ptr && b->size != bytes) {
        CK(cudaFreeAsync(b->ptr, d->stream));
        b->ptr = nullptr;
        b->size = 0;
    }
    if (bytes && !b->ptr) CK(cudaMallocAsync((void **)&b->ptr, bytes, d->stream));
    b->size = bytes;
    if (bytes) {
        if (data) CK(cudaMemcpyAsync(b->ptr, data, bytes, cudaMemcpyHostToDevice, d->stream));
        else CK(cudaMemsetAsync(b->ptr, 0, bytes, d->stream));
    }
    return MTGL_OK;
}

int mtgl_dev_buffer_sub_data(mtgl_dev *d, mtgl_handle h, uint64_t offset, const void *data, uint64_t bytes)
{
    DevBufferObj *b = reinterpret_cast<DevBufferObj *>(h);
    if (!d || !b || offset + bytes > b->size) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);
    if (st) return st;
    if (bytes) CK(cudaMemcpyAsync(b->ptr + offset, data, bytes, cudaMemcpyHostToDevice, d->stream));
    return MTGL_OK;
}

int mtgl_dev_buffer_destroy(mtgl_dev *d, mtgl_handle h)
{
    DevBufferObj *b = reinterpret_cast<DevBufferObj *>(h);
    if (!d || !b) return MTGL_OK;
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);
    if (st) return st;
    if (b->ptr) CK(cudaFreeAsync(b->ptr, d->stream));
    delete b;
    return MTGL_OK;
}

int mtgl_dev_texture_create(mtgl_dev *d, mtgl_handle *out)
{
    if (!d || !out) return MTGL_ERR_INVALID;
    DevTextureObj *t = new (std::nothrow) DevTextureObj();
    if (!t) return MTGL_ERR_OOM;
    *out = (mtgl_handle)(uintptr_t)t;
    return MTGL_OK;
}

int mtgl_dev_texture_image(mtgl_dev *d, mtgl_handle h, int32_t w, int32_t hgt, const uint32_t *rgba32)
{
    DevTextureObj *t = reinterpret_cast<DevTextureObj *>(h);
    if (!d || !t || w <= 0 || hgt <= 0 || !rgba32) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);
    if (st) return st;
    if (t->base) CK(cudaFreeAsync(t->base, d->stream));
    if (t->mip1) CK(cudaFreeAsync(t->mip1, d->stream));
    t->base = nullptr;
    t->mip1 = nullptr;
    const size_t n = (size_t)w * (size_t)hgt;
    CK(cudaMallocAsync((void **)&t->base, n * 4, d->stream));
    CK(cudaMemcpyAsync(t->base, rgba32, n * 4, cudaMemcpyHostToDevice, d->stream));
    t->w = w;
    t->h = hgt;
    t->mw = t->mh = 0;
    if (w >= 2 && hgt >= 2) {
        t->mw = w / 2;
        t->mh = hgt / 2;
        CK(cudaMallocAsync((void **)&t->mip1, (size_t)t->mw * t->mh * 4, d->stream));
        launch_mip1(t->base, w, hgt, t->mip1, d->stream);
        CK(cudaGetLastError());
        d->stats.kernel_launches++;
    }
    return MTGL_OK;
}

int mtgl_dev_texture_destroy(mtgl_dev *d, mtgl_handle h)
{
    DevTextureObj *t = reinterpret_cast<DevTextureObj *>(h);
    if (!d || !t) return MTGL_OK;
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);
    if (st) return st;
    if (t->base) CK(cudaFreeAsync(t->base, d->stream));
    if (t->mip1) CK(cudaFreeAsync(t->mip1, d->stream));
    delete t;
    return MTGL_OK;
}

// ---- commands

int mtgl_dev_clear(mtgl_dev *d, uint32_t mask, int32_t x0, int32_t y0, int32_t x1, int32_t y1, uint32_t color,
                   float depth, uint8_t stencil)
{
    if (!d) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);  // a clear after draws starts a new pass
    if (st) return st;
    ClearOp c;
    c.mask = mask;
    c.x0 = x0;
    c.y0 = y0;
    c.x1 = x1;
    c.y1 = y1;
    c.color = color;
    c.depth = depth;
    c.stencil = stencil;
    d->clears.push_back(c);
    return MTGL_OK;
}

int mtgl_dev_draw(mtgl_dev *d, const mtgl_draw *dr)
{
    if (!d || !dr || !dr->raster_state || !dr->vertex_states || dr->vertex_state_count == 0 || dr->count < 0)
        return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    const mtgl_raster_state *rs = dr->raster_state;
    if (dr->mode > GL_POLYGON) return MTGL_ERR_INVALID;
    if (dr->mode < GL_TRIANGLES) {
        snprintf(g_err, sizeof(g_err), "points and lines are not rendered by this back end");
        return MTGL_ERR_UNSUPPORTED;
    }
    if (rs->polygon_mode_front != GL_FILL || rs->polygon_mode_back != GL_FILL) {
        snprintf(g_err, sizeof(g_err), "glPolygonMode GL_POINT/GL_LINE is not rendered by this back end");
        return MTGL_ERR_UNSUPPORTED;
    }
    d->stats.draws++;
    const uint64_t ntri = triangles_of(dr->mode, dr->count);
    if (ntri == 0) return MTGL_OK;
    if (d->tris + ntri > 0x7FFFFFFFull) {
        int st = flush_if_drawing(d);
        if (st) return st;
        if (ntri > 0x7FFFFFFFull) return MTGL_ERR_INVALID;
    }
    int st = stage_begin(d);
    if (st) return st;

    PendingDraw p;
    memset(&p.d, 0, sizeof(p.d));
    DevDraw &D = p.d;
    D.mode = dr->mode;
    D.first = dr->first;
    D.count = dr->count;
    D.index_type = dr->index_type;
    D.pos2d = dr->position_2d;
    memcpy(D.cur_color, dr->current_color, sizeof(D.cur_color));
    memcpy(D.cur_tex, dr->current_texcoord, sizeof(D.cur_tex));
    memcpy(D.cur_normal, dr->current_normal, sizeof(D.cur_normal));

    int64_t lo, hi;
    if (dr->index_type) {
        lo = dr->index_min;
        hi = dr->index_max;
        const int64_t range_n = hi >= lo ? hi - lo + 1 : 0;
        D.index_min = lo;
        if (range_n <= 2 * (int64_t)dr->count + 1024) {
            D.range_mode = 1;
            D.range_n = (int32_t)range_n;
            D.vslot_count = (uint32_t)range_n + 1;  // + the default-attribute slot
        } else {
            D.range_mode = 0;
            D.vslot_count = (uint32_t)dr->count;
        }
        const size_t ib = (size_t)dr->count * index_size(dr->index_type);
        if (dr->index_buffer) {
            const DevBufferObj *b = reinterpret_cast<const DevBufferObj *>(dr->index_buffer);
            if (!b->ptr || dr->index_offset + ib > b->size) return MTGL_ERR_INVALID;
            D.indices = b->ptr + dr->index_offset;
        } else {
            if ((st = stage_copy(d, dr->index_host, ib, &p.off_idx))) return st;
        }
    } else {
        lo = dr->first < 0 ? 0 : dr->first;
        hi = (int64_t)dr->first + dr->count - 1;
        D.vslot_count = (uint32_t)dr->count;
    }
    const bool host_attr = (dr->position.enabled && !dr->position.buffer) || (dr->color.enabled && !dr->color.buffer) ||
                           (dr->texcoord.enabled && !dr->texcoord.buffer) || (dr->normal.enabled && !dr->normal.buffer);
    if (dr->index_type && !D.range_mode && host_attr) {
        snprintf(g_err, sizeof(g_err), "sparse client-memory index ranges are not supported");
        return MTGL_ERR_UNSUPPORTED;
    }
    if ((st = resolve_attr(d, dr->position, lo, hi, D.pos, p.off_pos))) return st;
    if ((st = resolve_attr(d, dr->color, lo, hi, D.color, p.off_color))) return st;
    if ((st = resolve_attr(d, dr->texcoord, lo, hi, D.tex, p.off_tex))) return st;
    if ((st = resolve_attr(d, dr->normal, lo, hi, D.normal, p.off_normal))) return st;
    if (dr->vertex_state_ids && !dr->index_type) {
        if ((st = stage_copy(d, dr->vertex_state_ids, (size_t)dr->count * sizeof(uint32_t), &p.off_vsid))) return st;
    }
    D.vs_base = push_vstates(d, dr->vertex_states, dr->vertex_state_count);
    D.raster = push_raster(d, rs);
    D.vslot_base = (uint32_t)d->slots;
    D.tri_base = (uint32_t)d->tris;
    D.tri_count = (uint32_t)ntri;
    d->slots += D.vslot_count;
    d->tris += ntri;
    d->draws.push_back(p);
    return MTGL_OK;
}

int mtgl_dev_draw_pixels(mtgl_dev *d, int32_t rx, int32_t ry, int32_t w, int32_t h, const uint32_t *rgba32,
                         const mtgl_raster_state *rs)
{
    if (!d || !rs) return MTGL_ERR_INVALID;
    if (w <= 0 || h <= 0 || !rgba32) return MTGL_OK;
    CK(cudaSetDevice(d->device));
    int st = flush_pass(d);
    if (st) return st;
    DevRaster R;
    memset(&R, 0, sizeof(R));
    R.rs = *rs;
    uint32_t *img = nullptr;
    DevRaster *dr = nullptr;
    const size_t n = (size_t)w * (size_t)h;
    CK(cudaMallocAsync((void **)&img, n * 4, d->stream));
    CK(cudaMallocAsync((void **)&dr, sizeof(DevRaster), d->stream));
    CK(cudaMemcpyAsync(img, rgba32, n * 4, cudaMemcpyHostToDevice, d->stream));
    CK(cudaMemcpyAsync(dr, &R, sizeof(R), cudaMemcpyHostToDevice, d->stream));
    launch_draw_pixels(img, rx, ry, w, h, dr, d->dims, d->color, d->depth, d->stream);
    CK(cudaGetLastError());
    CK(cudaFreeAsync(img, d->stream));
    CK(cudaFreeAsync(dr, d->stream));
    d->stats.kernel_launches++;
    return MTGL_OK;
}

int mtgl_dev_flush(mtgl_dev *d)
{
    if (!d) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    return flush_pass(d);
}

int mtgl_dev_finish(mtgl_dev *d)
{
    if (!d) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    int st = flush_pass(d);
    if (st) return st;
    CK(cudaStreamSynchronize(d->stream));
    return MTGL_OK;
}

int mtgl_dev_read(mtgl_dev *d, uint32_t *color, float *depth, uint8_t *stencil)
{
    if (!d) return MTGL_ERR_INVALID;
    int st = mtgl_dev_finish(d);
    if (st) return st;
    const size_t n = (size_t)d->dims.width * (size_t)d->dims.height;
    if (color) CK(cudaMemcpyAsync(color, d->color, n * 4, cudaMemcpyDeviceToHost, d->stream));
    if (depth) CK(cudaMemcpyAsync(depth, d->depth, n * 4, cudaMemcpyDeviceToHost, d->stream));
    if (stencil) CK(cudaMemcpyAsync(stencil, d->stencil, n, cudaMemcpyDeviceToHost, d->stream));
    CK(cudaStreamSynchronize(d->stream));
    return MTGL_OK;
}

int mtgl_dev_stats(mtgl_dev *d, mtgl_stats *out)
{
    if (!d || !out) return MTGL_ERR_INVALID;
    int st = mtgl_dev_finish(d);
    if (st) return st;
    unsigned long long f = 0;
    CK(cudaMemcpy(&f, d->d_frags, sizeof(f), cudaMemcpyDeviceToHost));
    *out = d->stats;
    out->fragments = f;
    return MTGL_OK;
}

int mtgl_dev_profile(mtgl_dev *d, int enable)
{
    if (!d) return MTGL_ERR_INVALID;
    int st = mtgl_dev_finish(d);
    if (st) return st;
    if ((st = prof_collect(d))) return st;
    d->profile = enable != 0;
    memset(&d->timings, 0, sizeof(d->timings));
    return MTGL_OK;
}

int mtgl_dev_timings(mtgl_dev *d, mtgl_timings *out)
{
    if (!d || !out) return MTGL_ERR_INVALID;
    int st = mtgl_dev_finish(d);
    if (st) return st;
    if ((st = prof_collect(d))) return st;
    *out = d->timings;
    return MTGL_OK;
}

void *mtgl_dev_stream(mtgl_dev *d) { return d ? (void *)d->stream : nullptr; }

int mtgl_dev_set_option(mtgl_dev *d, int option, int value)
{
    if (!d) return MTGL_ERR_INVALID;
    if (option != MTGL_OPT_DEPTH_REJECTION) return MTGL_ERR_INVALID;
    if (d->depth_rejection != (value != 0)) {
        d->raster_src.clear();  // the next draw pushes a raster state carrying the new value
        d->depth_rejection = value != 0;
    }
    return MTGL_OK;
}

int mtgl_dev_reset_stats(mtgl_dev *d)
{
    if (!d) return MTGL_ERR_INVALID;
    int st = mtgl_dev_finish(d);
    if (st) return st;
    memset(&d->stats, 0, sizeof(d->stats));
    CK(cudaMemsetAsync(d->d_frags, 0, sizeof(unsigned long long), d->stream));
    CK(cudaStreamSynchronize(d->stream));
    return MTGL_OK;
}

}  // extern "C"

// ============================================================================================
// Allocation-free flush.
//
// Some callers cannot let this library allocate device memory while they render: a
// real-time render thread cannot afford the device-wide synchronisation cudaMalloc and
// cudaFree imply; a serving process may keep every byte of device memory under its own
// budget; code that owns the CUDA allocator (another runtime's memory pool) may forbid
// foreign allocations. mtgl_flush_noalloc gives them the same pass pipeline as
// mtgl_dev_flush with every per-pass scratch buffer (post-transform vertices, triangle
// records, tile pairs, radix histograms, scan temporaries, tile counts) carved from one
// file-scope device array of kNoAllocScratchBytes instead of from cudaMallocAsync.
//
// Limits: a pass whose scratch does not fit is refused with MTGL_ERR_OVERFLOW before
// anything is drawn, and stays queued (mtgl_finish or mtgl_dev_flush can still render
// it). The pass's tables must fit the staging areas the context already holds. Every
// call, from every context on the device, shares the one array and overwrites what the
// previous call left; calls whose work overlaps on the GPU (two contexts on different
// streams) race, so callers serialise them. The array's device address is looked up
// once per device, on the first call with that device current; make that first call
// before any stream capture.
// ============================================================================================
#include <mutex>

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;  // 64 MiB held by every GPU that loads the library
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
uint8_t *g_noalloc_addr[kNoAllocMaxDevices] = {};

// set-up, once per device with that device current: host code needs the array's device address
int noalloc_scratch(int device, uint8_t **out)
{
    if (device < 0 || device >= kNoAllocMaxDevices) {
        snprintf(g_err, sizeof(g_err), "mtgl_flush_noalloc: device %d out of range", device);
        return MTGL_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return fail_cuda("cudaGetSymbolAddress(g_noalloc_scratch)", e);
        g_noalloc_addr[device] = static_cast<uint8_t *>(p);
    }
    *out = g_noalloc_addr[device];
    return MTGL_OK;
}

// bump allocator over the static array (256-byte aligned pieces)
struct Carve {
    uint8_t *base;
    size_t used, cap;
    template <class T>
    T *take(size_t n)
    {
        size_t at = (used + 255) & ~(size_t)255;
        size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        if (at + bytes > cap) return nullptr;
        used = at + bytes;
        return reinterpret_cast<T *>(base + at);
    }
};

int noalloc_overflow(const char *what, size_t need)
{
    snprintf(g_err, sizeof(g_err),
             "mtgl_flush_noalloc: the pass needs more than the %zu-byte static scratch (%s, %zu bytes); "
             "the pass stays queued",
             kNoAllocScratchBytes, what, need);
    return MTGL_ERR_OVERFLOW;
}

int flush_pass_noalloc(mtgl_dev *d)
{
    if (d->draws.empty()) return run_clears_only(d);  // clears launch kernels only
    uint8_t *scratch = nullptr;
    int st = noalloc_scratch(d->device, &scratch);
    if (st) return st;
    const size_t ndraws = d->draws.size();
    const size_t hused0 = d->hused;

    // tables into the existing staging area, without growing it
    size_t at = hused0;
    auto place = [&](size_t bytes) {
        size_t off = align16(at);
        at = off + bytes;
        return (int64_t)off;
    };
    const int64_t off_draws = place(ndraws * sizeof(DevDraw));
    const int64_t off_vbase = place(ndraws * sizeof(uint32_t));
    const int64_t off_tbase = place(ndraws * sizeof(uint32_t));
    const int64_t off_vs = place(d->vstates.size() * sizeof(mtgl_vertex_state));
    const int64_t off_rs = place(d->rasters.size() * sizeof(DevRaster));
    const int64_t off_clears = place(std::max<size_t>(1, d->clears.size()) * sizeof(ClearOp));
    if (at > d->hcap || at > d->dcap) {
        snprintf(g_err, sizeof(g_err),
                 "mtgl_flush_noalloc: the pass's tables (%zu bytes) exceed the context's staging areas; "
                 "the pass stays queued",
                 at);
        return MTGL_ERR_OVERFLOW;
    }
    if ((st = stage_begin(d))) return st;

    const uint32_t slots = (uint32_t)d->slots, tris = (uint32_t)d->tris;
    const bool eye = d->pass_needs_eye;
    const uint32_t ntiles = (uint32_t)(d->dims.tiles_x * d->dims.tiles_y);
    Carve cv{scratch, 0, kNoAllocScratchBytes};
    PostVertex *verts = cv.take<PostVertex>(slots);
    PostEye *eyes = eye ? cv.take<PostEye>(slots) : nullptr;
    uint32_t *tri_counts = cv.take<uint32_t>(tris);
    uint32_t *tri_offsets = cv.take<uint32_t>(tris);
    uint32_t *tile_count = cv.take<uint32_t>(ntiles + 1);
    uint32_t *tile_start = cv.take<uint32_t>(ntiles + 1);
    uint32_t *scan_temp = cv.take<uint32_t>(scan_temp_words(std::max<uint32_t>(std::max(tris, ntiles), 1)));
    if (!verts || (eye && !eyes) || !tri_counts || !tri_offsets || !tile_count || !tile_start || !scan_temp)
        return noalloc_overflow("vertices and triangle counts", cv.used);

    uint8_t *ds = d->dstage;
    DevDraw *hd = reinterpret_cast<DevDraw *>(d->hstage + off_draws);
    uint32_t *hvb = reinterpret_cast<uint32_t *>(d->hstage + off_vbase);
    uint32_t *htb = reinterpret_cast<uint32_t *>(d->hstage + off_tbase);
    for (size_t i = 0; i < ndraws; i++) {
        PendingDraw &p = d->draws[i];
        DevDraw dd = p.d;
        if (p.off_pos >= 0) dd.pos.ptr = ds + p.off_pos;
        if (p.off_color >= 0) dd.color.ptr = ds + p.off_color;
        if (p.off_tex >= 0) dd.tex.ptr = ds + p.off_tex;
        if (p.off_normal >= 0) dd.normal.ptr = ds + p.off_normal;
        if (p.off_idx >= 0) dd.indices = ds + p.off_idx;
        if (p.off_vsid >= 0) dd.vs_ids = reinterpret_cast<const uint32_t *>(ds + p.off_vsid);
        hd[i] = dd;
        hvb[i] = dd.vslot_base;
        htb[i] = dd.tri_base;
    }
    if (!d->vstates.empty())
        memcpy(d->hstage + off_vs, d->vstates.data(), d->vstates.size() * sizeof(mtgl_vertex_state));
    memcpy(d->hstage + off_rs, d->rasters.data(), d->rasters.size() * sizeof(DevRaster));
    if (!d->clears.empty()) memcpy(d->hstage + off_clears, d->clears.data(), d->clears.size() * sizeof(ClearOp));
    CK(cudaMemcpyAsync(d->dstage, d->hstage, at, cudaMemcpyHostToDevice, d->stream));

    GeomArgs ga;
    memset(&ga, 0, sizeof(ga));
    ga.draws = reinterpret_cast<const DevDraw *>(ds + off_draws);
    ga.draw_vslot_base = reinterpret_cast<const uint32_t *>(ds + off_vbase);
    ga.draw_tri_base = reinterpret_cast<const uint32_t *>(ds + off_tbase);
    ga.ndraws = (int32_t)ndraws;
    ga.vstates = reinterpret_cast<const mtgl_vertex_state *>(ds + off_vs);
    ga.rasters = reinterpret_cast<const DevRaster *>(ds + off_rs);
    ga.verts = verts;
    ga.eyes = eyes;
    ga.total_slots = slots;
    ga.total_tris = tris;
    ga.dims = d->dims;
    ga.tri_counts = tri_counts;
    ga.tri_offsets = tri_offsets;
    int launches = 0;
    launches += launch_vertex(ga, d->stream);
    launches += launch_setup_count(ga, d->stream);
    launches += launch_scan(tri_counts, tri_offsets, tris, scan_temp, d->d_totals + 0, d->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(d->h_totals, d->d_totals, sizeof(uint32_t), cudaMemcpyDeviceToHost, d->stream));
    CK(cudaStreamSynchronize(d->stream));
    const uint32_t nrec = d->h_totals[0];

    float *records = cv.take<float>((size_t)nrec * kRecWords);
    float *eye_records = eye ? cv.take<float>((size_t)nrec * kEyeWords) : nullptr;
    uint32_t *rec_tiles = cv.take<uint32_t>(nrec);
    if (!records || (eye && !eye_records) || !rec_tiles) {
        d->hused = hused0;
        return noalloc_overflow("triangle records", cv.used + (size_t)nrec * (kRecWords + kEyeWords + 1) * 4);
    }
    ga.records = records;
    ga.eye_records = eye_records;
    ga.records_cap = nrec;
    launches += launch_setup_emit(ga, d->stream);

    CK(cudaMemsetAsync(tile_count, 0, (ntiles + 1) * sizeof(uint32_t), d->stream));
    BinArgs ba;
    memset(&ba, 0, sizeof(ba));
    ba.records = records;
    ba.nrec = nrec;
    ba.dims = d->dims;
    ba.tile_count = tile_count;
    ba.tile_start = tile_start;
    ba.total_dev = d->d_totals + 1;
    uint32_t npairs = 0;
    if (nrec) {
        uint32_t *rec_scan_temp = cv.take<uint32_t>(scan_temp_words(std::max(nrec, ntiles)));
        if (!rec_scan_temp) {
            d->hused = hused0;
            return noalloc_overflow("record scan", cv.used);
        }
        ba.rec_tiles = rec_tiles;
        ba.scan_temp = rec_scan_temp;
        launches += launch_bin_count(ba, d->stream);
        launches += launch_scan(rec_tiles, rec_tiles, nrec, rec_scan_temp, d->d_totals + 1, d->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(d->h_totals + 1, d->d_totals + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, d->stream));
        CK(cudaStreamSynchronize(d->stream));
        npairs = d->h_totals[1];
        const size_t hist = radix_hist_words(npairs);
        uint32_t *keys = cv.take<uint32_t>(npairs), *vals = cv.take<uint32_t>(npairs);
        uint32_t *keys_alt = cv.take<uint32_t>(npairs), *vals_alt = cv.take<uint32_t>(npairs);
        uint32_t *radix_hist = cv.take<uint32_t>(hist);
        uint32_t *sort_scan_temp = cv.take<uint32_t>(
            scan_temp_words(std::max<uint32_t>(std::max<uint32_t>((uint32_t)hist, nrec), ntiles)));
        if (!keys || !vals || !keys_alt || !vals_alt || !radix_hist || !sort_scan_temp) {
            d->hused = hused0;
            return noalloc_overflow("tile pairs", cv.used + (size_t)npairs * 16);
        }
        ba.scan_temp = sort_scan_temp;
        ba.keys = keys;
        ba.vals = vals;
        ba.keys_alt = keys_alt;
        ba.vals_alt = vals_alt;
        ba.radix_hist = radix_hist;
        ba.npairs = npairs;
        ba.pairs_cap = npairs;
        launches += launch_bin_expand(ba, d->stream);
        launches += launch_bin_sort(ba, d->stream);
        scan_temp = sort_scan_temp;
    }
    launches += launch_scan(tile_count, tile_start, ntiles, scan_temp, d->d_totals + 2, d->stream);

    TileArgs ta;
    memset(&ta, 0, sizeof(ta));
    ta.records = records;
    ta.eye_records = eye_records;
    ta.tile_vals = nrec ? ba.vals : nullptr;
    ta.tile_start = tile_start;
    ta.tile_count = tile_count;
    ta.rasters = ga.rasters;
    ta.nrasters = (uint32_t)d->rasters.size();
    ta.clears = reinterpret_cast<const ClearOp *>(ds + off_clears);
    ta.nclears = (int32_t)d->clears.size();
    ta.any_texture = 0;
    for (const DevRaster &R : d->rasters) ta.any_texture |= R.tex != nullptr;
    ta.dims = d->dims;
    ta.color = d->color;
    ta.depth = d->depth;
    ta.stencil = d->stencil;
    ta.fragments = d->d_frags;
    launches += launch_tile(ta, d->stream);
    CK(cudaGetLastError());
    CK(cudaEventRecord(d->stage_done, d->stream));
    d->stage_inflight = true;

    d->stats.passes++;
    d->stats.input_triangles += tris;
    d->stats.setup_triangles += nrec;
    d->stats.bin_entries += npairs;
    d->stats.kernel_launches += (uint64_t)launches;
    d->draws.clear();
    d->clears.clear();
    d->vstates.clear();
    d->rasters.clear();
    d->raster_src.clear();
    d->pass_needs_eye = false;
    d->slots = d->tris = 0;
    d->hused = 0;
    return MTGL_OK;
}

}  // namespace

extern "C" mtgl_dev *fe_context_device(GLState *ctx);

extern "C" int mtgl_flush_noalloc(GLState *ctx)
{
    mtgl_dev *d = ctx ? fe_context_device(ctx) : nullptr;
    if (!d) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    return flush_pass_noalloc(d);
}
