// dev_runtime.cu — the mtgl_dev C ABI of the GB300 back end (include/mytinygl/mtgl_dev.h).
//
// One mtgl_dev per GL context: the framebuffer in device memory (row-major, row 0 = top,
// colour u32 a<<24|b<<16|g<<8|r, depth f32, stencil u8, as src/framebuffer.h:19-25), one
// CUDA stream, resource storage (buffer objects, textures with their mip level 1) and the
// pending pass. A pass is a run of clears followed by draws. Draws are queued with their
// state blocks; client memory they borrow is copied into pinned staging at enqueue time.
// A flush uploads the staging area with one copy and runs K1 vertex -> K2 setup count ->
// scan -> K2 emit -> K3 bin -> K4 tile over the whole pass (dev_pipeline.cu). Anything that
// must observe the framebuffer or change a resource a queued draw reads flushes first, and
// every device operation of a context runs on its one stream, so GL submission order is
// preserved. A context whose pass was rendered by a batch (dev_batch.cu) orders its stream
// after that batch before its next device operation.
#include <algorithm>
#include <new>

#include "dev_internal.h"

using namespace mtgl;

namespace {

// primitives of a draw: what K2 runs one thread for (points, line segments or triangles)
uint64_t triangles_of(uint32_t mode, int64_t n)
{
    switch (mode) {
    case GL_POINTS: return (uint64_t)(n > 0 ? n : 0);
    case GL_LINES: return (uint64_t)(n / 2);
    case GL_LINE_STRIP: return n >= 2 ? (uint64_t)(n - 1) : 0;
    case GL_LINE_LOOP: return n >= 2 ? (uint64_t)n : 0;
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

// the tile kernel's packed copy of the fragment stages' state (FragState)
void pack_frag_state(DevRaster &R)
{
    const mtgl_raster_state &rs = R.rs;
    FragState &f = R.fs;
    memset(&f, 0, sizeof(f));
    uint32_t c = 0;
    if (rs.stencil_test) c |= FC_STENCIL;
    if (rs.depth_test) c |= FC_DEPTH;
    if (rs.depth_test && rs.depth_mask) c |= FC_DEPTH_WRITE;
    if (rs.shade_model == GL_FLAT) c |= FC_FLAT;
    if (rs.alpha_test) c |= FC_ALPHA;
    if (rs.perspective_hint == GL_FASTEST) c |= FC_AFFINE_UV;
    if (rs.fog) c |= FC_FOG;
    if (rs.blend) c |= FC_BLEND;
    if (R.default_depth_range) c |= FC_DEFAULT_RANGE;
    uint32_t mask = 0;
    for (int i = 0; i < 4; i++)
        if (rs.color_mask[i]) mask |= 1u << i;
    if (mask == 15u) c |= FC_MASK_ALL;
    if (mask == 0u) c |= FC_MASK_NONE;
    if (R.tex) c |= FC_TEXTURE;
    f.ctl = c;
    f.depth_func = rs.depth_func;
    f.alpha_func = rs.alpha_func;
    f.tex_env_mode = rs.tex_env_mode;
    f.stencil_func = rs.stencil_func;
    f.stencil_ref = rs.stencil_ref;
    f.stencil_mask = rs.stencil_mask;
    f.stencil_writemask = rs.stencil_writemask;
    f.stencil_fail = rs.stencil_fail;
    f.stencil_zfail = rs.stencil_zfail;
    f.stencil_zpass = rs.stencil_zpass;
    f.alpha_ref = rs.alpha_ref;
    f.blend_src = rs.blend_src;
    f.blend_dst = rs.blend_dst;
    f.fog_mode = rs.fog_mode;
    f.fog_density = rs.fog_density;
    f.fog_start = rs.fog_start;
    f.fog_end = rs.fog_end;
    f.color_mask = mask;
    memcpy(f.fog_color, rs.fog_color, sizeof(f.fog_color));
    memcpy(f.tex_env_color, rs.tex_env_color, sizeof(f.tex_env_color));
    f.tex = R.tex;
    f.mip1 = R.mip1;
    f.tex_w = R.tex_w;
    f.tex_h = R.tex_h;
    f.mip_w = R.mip_w;
    f.mip_h = R.mip_h;
    f.wrap_s = rs.tex_wrap_s;
    f.wrap_t = rs.tex_wrap_t;
    f.min_filter = rs.tex_min_filter;
    f.mag_filter = rs.tex_mag_filter;
    f.chain = R.chain;
    f.chain_levels = R.chain_levels;
}

uint32_t push_raster(mtgl_dev *d, const mtgl_raster_state *rs)
{
    Pass &P = d->pass;
    if (!P.raster_src.empty() && memcmp(&P.raster_src.back(), rs, sizeof(*rs)) == 0)
        return (uint32_t)(P.rasters.size() - 1);
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
        R.chain = t->chain_tab;
        R.chain_levels = (int32_t)t->levels.size();
    }
    R.default_depth_range = (rs->depth_near == 0.0 && rs->depth_far == 1.0) ? 1 : 0;
    R.needs_eye = (rs->lighting && (rs->shade_model == GL_PHONG || rs->lit.two_side)) ? 1 : 0;
    R.depth_rejection = d->depth_rejection ? 1 : 0;
    pack_frag_state(R);
    if (R.needs_eye) P.needs_eye = true;
    P.raster_src.push_back(*rs);
    P.rasters.push_back(R);
    return (uint32_t)(P.rasters.size() - 1);
}

uint32_t push_vstates(mtgl_dev *d, const mtgl_vertex_state *vs, uint32_t n)
{
    Pass &P = d->pass;
    if (n == 1 && !P.vstates.empty() && memcmp(&P.vstates.back(), vs, sizeof(*vs)) == 0)
        return (uint32_t)(P.vstates.size() - 1);
    uint32_t base = (uint32_t)P.vstates.size();
    P.vstates.insert(P.vstates.end(), vs, vs + n);
    return base;
}

// Resolve one attribute stream. Client memory is copied for element range [lo, hi].
// bytes of one element of an enabled array (what the vertex stage reads per slot)
uint64_t attr_bytes(const mtgl_attrib &a) { return a.enabled ? (uint64_t)a.size * (a.type == GL_FLOAT ? 4u : 1u) : 0u; }

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
    int st = d->stage.copy((const uint8_t *)a.host + (size_t)lo * (size_t)a.stride, bytes, &off);
    if (st) return st;
    out.base_index = lo;
    out.bytes = bytes;
    return MTGL_OK;
}

int run_clears_only(mtgl_dev *d)
{
    Pass &P = d->pass;
    if (P.clears.empty()) return MTGL_OK;
    FrameDims dims;
    dims.width = d->width;
    dims.height = d->height;
    dims.tiles_x = dims.tiles_y = 0;
    launch_clear(P.clears.data(), (int)P.clears.size(), dims, d->color, d->depth, d->stencil, d->x.stream);
    d->stats.kernel_launches += (P.clears.size() + 15) / 16;
    d->stats.passes++;
    P.clears.clear();
    CK(cudaGetLastError());
    return MTGL_OK;
}

// Exact sizing. A large pass runs the tile kernel persistently in two launches, tiles of
// small records by rounds and the rest per record, each in tile order; a small one, where
// those extra launches would cost more than they save, with one CTA per tile.
PipeConfig plain_config(mtgl_dev *d, const Tables &t)
{
    PipeConfig c;
    if (t.tris >= 32768) {
        c.ctas = persistent_ctas(d->x, t, 0);
        c.classify = true;  // one frame: tile order keeps neighbouring tiles' records in cache together
    }
    return c;
}

int flush_pass(mtgl_dev *d)
{
    int st = mtgl_dev_enter(d);
    if (st) return st;
    Pass &P = d->pass;
    if (P.draws.empty()) return run_clears_only(d);
    FrameSrc fs{d, &P, 0};
    Tables t;
    if ((st = build_tables(d->x, d->stage, &fs, 1, kTileShiftPlain, true, t))) return st;
    PipeConfig c = plain_config(d, t);
    PipeOut o;
    if ((st = run_pipeline(d->x, d->x.pool, d->stage, t, c, &o))) return st;
    if ((st = d->stage.mark_uploaded(d->x.stream))) return st;
    d->stats.passes++;
    d->stats.input_triangles += P.tris;
    d->stats.vertices += P.slots;
    d->stats.vertex_bytes += P.vbytes;
    d->stats.setup_triangles += o.nrec;
    d->stats.bin_entries += o.npairs;
    d->stats.kernel_launches += (uint64_t)o.launches;
    P.reset();
    d->stage.used = 0;
    return MTGL_OK;
}

int flush_if_drawing(mtgl_dev *d)
{
    if (!d->pass.draws.empty()) return flush_pass(d);
    return MTGL_OK;
}

}  // namespace

// For the serving loop (csrc/serve): the device a context lives on, and binding a thread to
// it. Internal to the library (not exported).
extern "C" int dev_device_index(const mtgl_dev *d) { return d ? d->device : -1; }
extern "C" int dev_bind_thread(int device) { return cudaSetDevice(device) == cudaSuccess ? MTGL_OK : MTGL_ERR_CUDA; }
extern "C" int dev_current_device(void)
{
    int d = 0;
    return cudaGetDevice(&d) == cudaSuccess ? d : -1;
}

int mtgl_dev_enter(mtgl_dev *d)
{
    if (d->batch) {
        int st = mtgl_dev_batch_wait(d->batch);  // verifies (and if needed re-runs) the batch
        if (st) return st;
    }
    while (!d->readers.empty()) {  // batches still reading this context's resources
        int st = mtgl_dev_batch_wait(d->readers.back());
        if (st) return st;
    }
    if (d->after_batch) {
        CK(cudaStreamWaitEvent(d->x.stream, d->after_batch->ev, 0));
        mark_drop(d->after_batch);
        d->after_batch = nullptr;
    }
    d->dirty = true;
    return MTGL_OK;
}

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
    int st = d->x.init(nullptr);
    if (st) {
        delete d;
        return st;
    }
    d->device = d->x.device;
    d->width = width;
    d->height = height;
    const size_t np = (size_t)width * (size_t)height;
    cudaStream_t s = d->x.stream;
    CK(cudaEventCreateWithFlags(&d->stage.done, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&d->tail, cudaEventDisableTiming));
    CK(cudaMallocAsync((void **)&d->color, np * 4, s));
    CK(cudaMallocAsync((void **)&d->depth, np * 4, s));
    CK(cudaMallocAsync((void **)&d->stencil, np, s));
    CK(cudaMemsetAsync(d->color, 0, np * 4, s));
    CK(cudaMemsetAsync(d->depth, 0, np * 4, s));
    CK(cudaMemsetAsync(d->stencil, 0, np, s));
    CK(cudaStreamSynchronize(s));
    *out = d;
    return MTGL_OK;
}

int mtgl_dev_destroy(mtgl_dev *d)
{
    if (!d) return MTGL_OK;
    cudaSetDevice(d->device);
    mtgl_dev_enter(d);
    cudaStreamSynchronize(d->x.stream);
    cudaFreeAsync(d->color, d->x.stream);
    cudaFreeAsync(d->depth, d->x.stream);
    cudaFreeAsync(d->stencil, d->x.stream);
    d->stage.release();
    d->x.destroy();
    cudaEventDestroy(d->tail);
    if (d->after_batch) mark_drop(d->after_batch);
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
    if (st || (st = mtgl_dev_enter(d))) return st;
    cudaStream_t s = d->x.stream;
    if (b->ptr && b->size != bytes) {
        CK(cudaFreeAsync(b->ptr, s));
        b->ptr = nullptr;
        b->size = 0;
    }
    if (bytes && !b->ptr) CK(cudaMallocAsync((void **)&b->ptr, bytes, s));
    b->size = bytes;
    if (bytes) {
        if (data) CK(cudaMemcpyAsync(b->ptr, data, bytes, cudaMemcpyHostToDevice, s));
        else CK(cudaMemsetAsync(b->ptr, 0, bytes, s));
    }
    return MTGL_OK;
}

int mtgl_dev_buffer_sub_data(mtgl_dev *d, mtgl_handle h, uint64_t offset, const void *data, uint64_t bytes)
{
    DevBufferObj *b = reinterpret_cast<DevBufferObj *>(h);
    if (!d || !b || offset + bytes > b->size) return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);
    if (st || (st = mtgl_dev_enter(d))) return st;
    if (bytes) CK(cudaMemcpyAsync(b->ptr + offset, data, bytes, cudaMemcpyHostToDevice, d->x.stream));
    return MTGL_OK;
}

int mtgl_dev_buffer_destroy(mtgl_dev *d, mtgl_handle h)
{
    DevBufferObj *b = reinterpret_cast<DevBufferObj *>(h);
    if (!d || !b) return MTGL_OK;
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);
    if (st || (st = mtgl_dev_enter(d))) return st;
    if (b->ptr) CK(cudaFreeAsync(b->ptr, d->x.stream));
    delete b;
    return MTGL_OK;
}

// MTGL_OPT_MIPMAP_CHAIN: levels 2.. of t, each the 2x2 box filter of the one before (the
// kernel that builds level 1), while both sides of the previous level are at least 2.
static int build_chain(mtgl_dev *d, DevTextureObj *t)
{
    cudaStream_t s = d->x.stream;
    std::vector<DevMip> lv;
    size_t texels = 0;
    for (int32_t w = t->mw, h = t->mh; w >= 2 && h >= 2; w /= 2, h /= 2) {
        lv.push_back(DevMip{nullptr, w / 2, h / 2});
        texels += (size_t)(w / 2) * (size_t)(h / 2);
    }
    if (lv.empty()) return MTGL_OK;
    CK(cudaMallocAsync((void **)&t->chain, texels * 4, s));
    CK(cudaMallocAsync((void **)&t->chain_tab, lv.size() * sizeof(DevMip), s));
    size_t at = 0;
    const uint32_t *prev = t->mip1;
    int32_t pw = t->mw, ph = t->mh;
    for (DevMip &m : lv) {
        m.px = t->chain + at;
        at += (size_t)m.w * (size_t)m.h;
        launch_mip1(prev, pw, ph, const_cast<uint32_t *>(m.px), s);
        d->stats.kernel_launches++;
        prev = m.px;
        pw = m.w;
        ph = m.h;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(t->chain_tab, lv.data(), lv.size() * sizeof(DevMip), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // the table's source is this function's vector
    t->levels = std::move(lv);
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
    if (st || (st = mtgl_dev_enter(d))) return st;
    cudaStream_t s = d->x.stream;
    if (t->base) CK(cudaFreeAsync(t->base, s));
    if (t->mip1) CK(cudaFreeAsync(t->mip1, s));
    if (t->chain) CK(cudaFreeAsync(t->chain, s));
    if (t->chain_tab) CK(cudaFreeAsync(t->chain_tab, s));
    t->base = nullptr;
    t->mip1 = nullptr;
    t->chain = nullptr;
    t->chain_tab = nullptr;
    t->levels.clear();
    const size_t n = (size_t)w * (size_t)hgt;
    CK(cudaMallocAsync((void **)&t->base, n * 4, s));
    CK(cudaMemcpyAsync(t->base, rgba32, n * 4, cudaMemcpyHostToDevice, s));
    t->w = w;
    t->h = hgt;
    t->mw = t->mh = 0;
    if (w >= 2 && hgt >= 2) {
        t->mw = w / 2;
        t->mh = hgt / 2;
        CK(cudaMallocAsync((void **)&t->mip1, (size_t)t->mw * t->mh * 4, s));
        launch_mip1(t->base, w, hgt, t->mip1, s);
        CK(cudaGetLastError());
        d->stats.kernel_launches++;
    }
    if (d->mipmap_chain && t->mip1) return build_chain(d, t);
    return MTGL_OK;
}

int mtgl_dev_texture_level(mtgl_dev *d, mtgl_handle h, int32_t level, int32_t w, int32_t hgt, const uint32_t *rgba32)
{
    DevTextureObj *t = reinterpret_cast<DevTextureObj *>(h);
    if (!d || !t || !rgba32 || level < 1) return MTGL_ERR_INVALID;
    uint32_t *dst = nullptr;
    if (level == 1 && t->mip1 && w == t->mw && hgt == t->mh) dst = t->mip1;
    const size_t k = (size_t)level - 2;
    if (level >= 2 && k < t->levels.size() && w == t->levels[k].w && hgt == t->levels[k].h)
        dst = const_cast<uint32_t *>(t->levels[k].px);
    if (!dst || t->levels.empty()) {
        snprintf(g_err, sizeof(g_err), "texture level %d of %dx%d: no such level in the texture's chain", level, w, hgt);
        return MTGL_ERR_INVALID;
    }
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);
    if (st || (st = mtgl_dev_enter(d))) return st;
    CK(cudaMemcpyAsync(dst, rgba32, (size_t)w * (size_t)hgt * 4, cudaMemcpyHostToDevice, d->x.stream));
    return MTGL_OK;
}

int mtgl_dev_texture_destroy(mtgl_dev *d, mtgl_handle h)
{
    DevTextureObj *t = reinterpret_cast<DevTextureObj *>(h);
    if (!d || !t) return MTGL_OK;
    CK(cudaSetDevice(d->device));
    int st = flush_if_drawing(d);
    if (st || (st = mtgl_dev_enter(d))) return st;
    if (t->base) CK(cudaFreeAsync(t->base, d->x.stream));
    if (t->mip1) CK(cudaFreeAsync(t->mip1, d->x.stream));
    if (t->chain) CK(cudaFreeAsync(t->chain, d->x.stream));
    if (t->chain_tab) CK(cudaFreeAsync(t->chain_tab, d->x.stream));
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
    d->pass.clears.push_back(c);
    return MTGL_OK;
}

int mtgl_dev_draw(mtgl_dev *d, const mtgl_draw *dr)
{
    if (!d || !dr || !dr->raster_state || !dr->vertex_states || dr->vertex_state_count == 0 || dr->count < 0)
        return MTGL_ERR_INVALID;
    CK(cudaSetDevice(d->device));
    const mtgl_raster_state *rs = dr->raster_state;
    if (dr->mode > GL_POLYGON) return MTGL_ERR_INVALID;
    d->stats.draws++;
    const uint64_t ntri = triangles_of(dr->mode, dr->count);
    if (ntri == 0) return MTGL_OK;
    Pass &P = d->pass;
    if (P.tris + ntri > 0x7FFFFFFFull) {
        int st = flush_if_drawing(d);
        if (st) return st;
        if (ntri > 0x7FFFFFFFull) return MTGL_ERR_INVALID;
    }
    const size_t staged0 = d->stage.used;
    int st = d->stage.wait();
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
            if ((st = d->stage.copy(dr->index_host, ib, &p.off_idx))) return st;
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
        if ((st = d->stage.copy(dr->vertex_state_ids, (size_t)dr->count * sizeof(uint32_t), &p.off_vsid))) return st;
    }
    D.vs_base = push_vstates(d, dr->vertex_states, dr->vertex_state_count);
    D.raster = push_raster(d, rs);
    D.vslot_base = (uint32_t)P.slots;
    D.tri_base = (uint32_t)P.tris;
    D.tri_count = (uint32_t)ntri;
    P.slots += D.vslot_count;
    P.vbytes += (uint64_t)D.vslot_count * (attr_bytes(dr->position) + attr_bytes(dr->color) +
                                           attr_bytes(dr->texcoord) + attr_bytes(dr->normal));
    P.tris += ntri;
    P.draws.push_back(p);
    d->stats.staged_bytes += d->stage.used - staged0;
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
    cudaStream_t s = d->x.stream;
    CK(cudaMallocAsync((void **)&img, n * 4, s));
    CK(cudaMallocAsync((void **)&dr, sizeof(DevRaster), s));
    CK(cudaMemcpyAsync(img, rgba32, n * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dr, &R, sizeof(R), cudaMemcpyHostToDevice, s));
    FrameDims dims;
    dims.width = d->width;
    dims.height = d->height;
    dims.tiles_x = dims.tiles_y = 0;
    launch_draw_pixels(img, rx, ry, w, h, dr, dims, d->color, d->depth, s);
    CK(cudaGetLastError());
    CK(cudaFreeAsync(img, s));
    CK(cudaFreeAsync(dr, s));
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
    CK(cudaStreamSynchronize(d->x.stream));
    return MTGL_OK;
}

int mtgl_dev_in_batch(const mtgl_dev *d) { return d && (d->batch || !d->readers.empty()) ? 1 : 0; }

int mtgl_dev_read(mtgl_dev *d, uint32_t *color, float *depth, uint8_t *stencil)
{
    if (!d) return MTGL_ERR_INVALID;
    int st = mtgl_dev_finish(d);
    if (st) return st;
    const size_t n = (size_t)d->width * (size_t)d->height;
    cudaStream_t s = d->x.stream;
    if (color) CK(cudaMemcpyAsync(color, d->color, n * 4, cudaMemcpyDeviceToHost, s));
    if (depth) CK(cudaMemcpyAsync(depth, d->depth, n * 4, cudaMemcpyDeviceToHost, s));
    if (stencil) CK(cudaMemcpyAsync(stencil, d->stencil, n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return MTGL_OK;
}

int mtgl_dev_stats(mtgl_dev *d, mtgl_stats *out)
{
    if (!d || !out) return MTGL_ERR_INVALID;
    int st = mtgl_dev_finish(d);
    if (st) return st;
    unsigned long long f = 0;
    CK(cudaMemcpy(&f, d->x.d_frags, sizeof(f), cudaMemcpyDeviceToHost));
    *out = d->stats;
    out->fragments = f;
    out->allocations = d->x.pool.allocs + d->x.allocs + d->stage.allocs - d->alloc_base;
    uint32_t dbg = 0;
    CK(cudaMemcpy(&dbg, d->x.d_totals + kDebugStatusWord, sizeof(dbg), cudaMemcpyDeviceToHost));
    out->debug_status = dbg;
    return MTGL_OK;
}

int mtgl_dev_profile(mtgl_dev *d, int enable)
{
    if (!d) return MTGL_ERR_INVALID;
    int st = mtgl_dev_finish(d);
    if (st) return st;
    if ((st = d->x.prof_collect())) return st;
    d->x.profile = enable != 0;
    memset(&d->x.timings, 0, sizeof(d->x.timings));
    return MTGL_OK;
}

int mtgl_dev_timings(mtgl_dev *d, mtgl_timings *out)
{
    if (!d || !out) return MTGL_ERR_INVALID;
    int st = mtgl_dev_finish(d);
    if (st) return st;
    if ((st = d->x.prof_collect())) return st;
    *out = d->x.timings;
    return MTGL_OK;
}

void *mtgl_dev_stream(mtgl_dev *d) { return d ? (void *)d->x.stream : nullptr; }

int mtgl_dev_set_option(mtgl_dev *d, int option, int value)
{
    if (!d) return MTGL_ERR_INVALID;
    if (option == MTGL_OPT_MIPMAP_CHAIN) {
        d->mipmap_chain = value != 0;  // applies to texture images given afterwards
        return MTGL_OK;
    }
    if (option != MTGL_OPT_DEPTH_REJECTION) return MTGL_ERR_INVALID;
    if (d->depth_rejection != (value != 0)) {
        d->pass.raster_src.clear();  // the next draw pushes a raster state carrying the new value
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
    d->alloc_base = d->x.pool.allocs + d->x.allocs + d->stage.allocs;
    CK(cudaMemsetAsync(d->x.d_frags, 0, sizeof(unsigned long long), d->x.stream));
    CK(cudaMemsetAsync(d->x.d_totals + kDebugStatusWord, 0, sizeof(uint32_t), d->x.stream));
    CK(cudaStreamSynchronize(d->x.stream));
    return MTGL_OK;
}

int mtgl_dev_debug_bounds(void)
{
#ifdef MTGL_DEBUG_BOUNDS
    return 1;
#else
    return 0;
#endif
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
// previous call left. Two calls whose GPU work overlapped would race on it (each context
// has its own stream, so even two calls made one after the other from one thread would),
// so each call's work waits on the GPU for the previous call's: one event per device,
// recorded at the end of every call and waited on by the next, under a lock, so calls
// run on the GPU in the order the host made them. The array's device address and the
// event are set up once per device, on the first call with that device current; make
// that first call before any stream capture.
// ============================================================================================
#include <mutex>

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;  // 64 MiB held by every GPU that loads the library
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;  // held for a whole call: set-up, and the wait - launch - record sequence
struct NoAllocDevice {
    uint8_t *scratch = nullptr;  // device address of g_noalloc_scratch
    cudaEvent_t done = nullptr;  // end of the last call's GPU work on this device
    bool pending = false;        // `done` has been recorded
};
NoAllocDevice g_noalloc[kNoAllocMaxDevices];

// set-up, once per device with that device current: host code needs the array's device
// address, and the calls need their ordering event; the caller holds g_noalloc_mu
int noalloc_setup(int device, NoAllocDevice **out)
{
    if (device < 0 || device >= kNoAllocMaxDevices) {
        snprintf(g_err, sizeof(g_err), "mtgl_flush_noalloc: device %d out of range", device);
        return MTGL_ERR_INVALID;
    }
    NoAllocDevice &nd = g_noalloc[device];
    if (!nd.scratch) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return fail_cuda("cudaGetSymbolAddress(g_noalloc_scratch)", e);
        if (!nd.done && (e = cudaEventCreateWithFlags(&nd.done, cudaEventDisableTiming)) != cudaSuccess)
            return fail_cuda("cudaEventCreateWithFlags", e);
        nd.scratch = static_cast<uint8_t *>(p);
    }
    *out = &nd;
    return MTGL_OK;
}

// Bump allocator over the static array (256-byte aligned pieces). A slot taken again gets
// its previous piece back when the new size fits in it, so re-taking a slot (the scan
// temporaries are taken once per sort pass) costs no space.
struct Carve final : ScratchSource {
    uint8_t *base = nullptr;
    size_t used = 0, cap = 0;
    size_t at_of[kScratchSlots] = {}, len_of[kScratchSlots] = {};
    bool held[kScratchSlots] = {};
    int get(int slot, size_t bytes, void **out) override
    {
        if (slot >= 0 && slot < kScratchSlots && held[slot] && bytes <= len_of[slot]) {
            *out = base + at_of[slot];
            return MTGL_OK;
        }
        const size_t at = (used + 255) & ~(size_t)255;
        if (at + bytes > cap) {
            snprintf(g_err, sizeof(g_err),
                     "mtgl_flush_noalloc: the pass needs more than the %zu-byte static scratch (%zu bytes so far); "
                     "the pass stays queued",
                     cap, at + bytes);
            return MTGL_ERR_OVERFLOW;
        }
        used = at + bytes;
        if (slot >= 0 && slot < kScratchSlots) {
            held[slot] = true;
            at_of[slot] = at;
            len_of[slot] = bytes;
        }
        *out = base + at;
        return MTGL_OK;
    }
};

// A refused pass may have recorded some of its profiling events: drop them, so the next
// pass's five events are read as one group.
void drop_profile_marks(Exec &x, size_t keep)
{
    while (x.ev_pending.size() > keep) {
        x.ev_pool.push_back(x.ev_pending.back());
        x.ev_pending.pop_back();
    }
}

int flush_pass_noalloc(mtgl_dev *d)
{
    int st = mtgl_dev_enter(d);
    if (st) return st;
    Pass &P = d->pass;
    if (P.draws.empty()) return run_clears_only(d);  // clears launch kernels only
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice *nd = nullptr;
    if ((st = noalloc_setup(d->device, &nd))) return st;
    Carve cv;
    cv.base = nd->scratch;
    cv.cap = kNoAllocScratchBytes;
    const size_t used0 = d->stage.used;
    const size_t marks0 = d->x.ev_pending.size();
    FrameSrc fs{d, &P, 0};
    Tables t;
    d->stage.fixed = true;  // tables go into the staging areas the context already holds
    st = build_tables(d->x, d->stage, &fs, 1, kTileShiftPlain, false, t);
    d->stage.fixed = false;
    if (st) {
        if (st == MTGL_ERR_OVERFLOW)
            snprintf(g_err, sizeof(g_err),
                     "mtgl_flush_noalloc: the pass's tables exceed the context's staging areas; the pass stays queued");
        return st;
    }
    // the previous call's kernels (any context, any stream) are done with the array first
    if (nd->pending) CK(cudaStreamWaitEvent(d->x.stream, nd->done, 0));
    PipeConfig c = plain_config(d, t);
    PipeOut o;
    st = run_pipeline(d->x, cv, d->stage, t, c, &o);
    // whatever this call enqueued, the next call waits for it
    CK(cudaEventRecord(nd->done, d->x.stream));
    nd->pending = true;
    if (st) {
        d->stage.used = used0;  // drop the tables; the pass stays queued
        drop_profile_marks(d->x, marks0);
        return st;
    }
    if ((st = d->stage.mark_uploaded(d->x.stream))) return st;
    d->stats.passes++;
    d->stats.input_triangles += P.tris;
    d->stats.vertices += P.slots;
    d->stats.vertex_bytes += P.vbytes;
    d->stats.setup_triangles += o.nrec;
    d->stats.bin_entries += o.npairs;
    d->stats.kernel_launches += (uint64_t)o.launches;
    P.reset();
    d->stage.used = 0;
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
