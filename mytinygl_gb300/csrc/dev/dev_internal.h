// dev_internal.h — host-side structures shared by the context runtime (dev_runtime.cu),
// the pass pipeline (dev_pipeline.cu) and the batch executor (dev_batch.cu).
#pragma once

#include <atomic>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dev_kernels.h"
#include "mytinygl/mytinygl.h"

namespace mtgl {

extern thread_local char g_err[512];
int fail_cuda(const char *what, cudaError_t e);

#define CK(call)                                                  \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return ::mtgl::fail_cuda(#call, e_); \
    } while (0)

inline size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

struct DevBufferObj {
    uint8_t *ptr = nullptr;
    uint64_t size = 0;
};

struct DevTextureObj {
    uint32_t *base = nullptr;
    uint32_t *mip1 = nullptr;
    int32_t w = 0, h = 0, mw = 0, mh = 0;
    // MTGL_OPT_MIPMAP_CHAIN: levels 2.. in one allocation, and their device table
    uint32_t *chain = nullptr;
    DevMip *chain_tab = nullptr;
    std::vector<DevMip> levels;  // host copy of the table (device pointers)
};

// Pending draw: a DevDraw whose pointers are patched when its pass is staged; off_* are
// offsets of client data copied into the context's staging area (-1: not staged).
struct PendingDraw {
    DevDraw d;
    int64_t off_pos = -1, off_color = -1, off_tex = -1, off_normal = -1, off_idx = -1, off_vsid = -1;
};

// An event recorded once at a point of a batch run that many contexts order after (the
// end of the run's uploads from their staging areas, or the end of the run), held by each
// of them and returned to a pool when the last lets go: one record per run, not one per
// context. It is never recorded again while held.
struct RunMark {
    cudaEvent_t ev = nullptr;
    int device = 0;
    std::atomic<int> refs{0};
};
RunMark *mark_new(int device);  // held once, by the caller; null on failure (g_err set)
void mark_hold(RunMark *m);
void mark_drop(RunMark *m);

// Pinned host staging. Client data is copied in at enqueue; a flush appends the pass's
// tables and uploads the whole area with one copy. It is not rewritten while that copy
// is in flight.
struct HostStage {
    uint8_t *p = nullptr;
    size_t cap = 0, used = 0;
    cudaEvent_t done = nullptr;  // recorded after the upload that reads the area
    bool inflight = false;
    // a batch's upload of the area: queued on `upload_stream` and not yet marked (wait
    // synchronises that stream), then marked by `upload_mark`
    cudaStream_t upload_stream = nullptr;
    RunMark *upload_mark = nullptr;
    bool fixed = false;          // refuse to grow (allocation-free flush)
    uint64_t allocs = 0;         // page-locked allocations made by growth

    int wait();
    int reserve(size_t bytes, int64_t *off);
    int copy(const void *src, size_t bytes, int64_t *off);
    int mark_uploaded(cudaStream_t s);
    void hold_upload(RunMark *m);  // the batch upload queued from this area ends at m
    void release();
};

// The pending pass of one context: clears, then draws with their state blocks.
struct Pass {
    std::vector<ClearOp> clears;
    std::vector<PendingDraw> draws;
    std::vector<mtgl_vertex_state> vstates;
    std::vector<DevRaster> rasters;
    std::vector<mtgl_raster_state> raster_src;  // for de-duplication
    bool needs_eye = false;
    uint64_t slots = 0, tris = 0;
    uint64_t vbytes = 0;  // attribute bytes the vertex stage reads for the pass's slots

    bool empty() const { return clears.empty() && draws.empty(); }
    void reset();
};

// Where per-pass device scratch comes from.
enum ScratchSlot {
    S_VERTS, S_EYES, S_TRI_COUNTS, S_TRI_OFFSETS, S_RECORDS, S_EYE_RECORDS, S_REC_TILES, S_KEYS, S_VALS,
    S_KEYS_ALT, S_VALS_ALT, S_TILE_COUNT, S_TILE_START, S_RADIX_HIST, S_SCAN_TEMP, S_ORDER, S_ORDER_AUX,
    S_CLIP_LIST, S_TILE_FRAME, kScratchSlots
};

struct ScratchSource {
    virtual int get(int slot, size_t bytes, void **out) = 0;  // contents undefined
    virtual ~ScratchSource() {}
    template <class T>
    int take(int slot, size_t n, T **out)
    {
        void *p = nullptr;
        const size_t bytes = (n ? n : 1) * sizeof(T);
        int st = get(slot, bytes, &p);
        *out = static_cast<T *>(p);
        return st;
    }
};

// grow-only buffers from the stream-ordered allocator
struct PoolScratch final : ScratchSource {
    cudaStream_t stream = nullptr;
    void *p[kScratchSlots] = {};
    size_t cap[kScratchSlots] = {};
    uint64_t allocs = 0;  // device allocations made by growth
    int get(int slot, size_t bytes, void **out) override;
    void release();
};

// A stream with its scratch, device staging copy and small counters: what runs a pass.
struct Exec {
    int device = 0;
    int sms = 1;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    PoolScratch pool;
    uint8_t *dstage = nullptr;
    size_t dcap = 0;
    uint64_t allocs = 0;  // device allocations of the staging copy
    uint32_t *d_totals = nullptr;  // [0] records, [1] pairs, [2] tiles' records, [3] sort scratch, [4] clip list, [5] emit list (GeomArgs::list_counts),
                                   // [kDebugStatusWord] the debug bounds checks' status
    uint32_t *h_totals = nullptr;  // pinned copy of [0..1]
    unsigned long long *d_frags = nullptr;
    // per-phase profiling: 5 events per pass (before K1, after K1, after K2, after K3, after K4)
    bool profile = false;
    std::vector<cudaEvent_t> ev_pool, ev_pending;
    mtgl_timings timings{};

    int init(cudaStream_t s);  // s null: create a stream
    void destroy();
    int ensure_dstage(size_t bytes, bool may_grow, size_t keep = 0);  // keep: leading bytes that survive growth
    void prof_mark();
    int prof_collect();  // the caller has synchronised the stream
};

// One frame of a pass: a context's framebuffer and pending pass, whose staged client data
// lies at data_off in the staging area being built.
struct FrameSrc {
    mtgl_dev *dev;
    const Pass *pass;
    int64_t data_off;
};

// The tables of a pass inside the staging area (offsets are the same in the host copy and
// in the device copy).
struct Tables {
    int64_t off_upload = 0;  // staged bytes before this offset are already in the device copy
    int64_t off_draws = 0, off_vbase = 0, off_tbase = 0, off_vs = 0, off_rs = 0, off_clears = 0, off_frames = 0;
    uint32_t ndraws = 0, nrasters = 0, nclears = 0, nframes = 0;
    uint32_t slots = 0, tris = 0, ntiles = 0;
    int tile_shift = kTileShiftPlain;
    bool eye = false, any_texture = false;
    bool defer = false;  // every record a filled triangle whose colour can be deferred (k_tile.cuh)
};

// Appends the tables of `frames` to `st` and makes the device staging copy large enough.
// `direct`: the first bytes of the area were copied to the device copy already (the upload
// starts after them, and they survive a growth of the device copy).
int build_tables(Exec &x, HostStage &st, const FrameSrc *frames, uint32_t nframes, int tile_shift, bool may_grow,
                 Tables &t, size_t direct = 0);

// CTAs of a persistent tile launch for these tables: per_sm per SM (0: all that fit)
int persistent_ctas(const Exec &x, const Tables &t, int per_sm);

struct PipeConfig {
    bool exact = true;       // wait for the record and pair totals and size scratch from them
    uint32_t rec_cap = 0;    // capacity mode: records and tile pairs the scratch holds
    uint32_t pair_cap = 0;
    int32_t ctas = 0;        // persistent tile CTAs (0: one CTA per tile)
    bool order = false;      // hand out tiles costliest first (classified: small-record tiles first)
    bool classify = false;   // without an order: small-record tiles by rounds, the rest per record
};

struct PipeOut {
    uint32_t nrec = 0, npairs = 0;  // exact mode only (capacity mode: read h_totals after the stream)
    int launches = 0;
};

// Uploads st[t.off_upload, st.used) and runs K1..K4 on x.stream. Capacity mode enqueues only (no host
// waits and no allocation after its first step), so it can be captured into a CUDA graph;
// alloc_only makes it take its scratch and return without enqueueing anything.
int run_pipeline(Exec &x, ScratchSource &sc, const HostStage &st, const Tables &t, const PipeConfig &c,
                 PipeOut *out, bool alloc_only = false);

}  // namespace mtgl

// The context object behind the mtgl_dev ABI.
struct mtgl_dev {
    int device = 0;
    int32_t width = 0, height = 0;
    uint32_t *color = nullptr;
    float *depth = nullptr;
    uint8_t *stencil = nullptr;
    mtgl::Exec x;
    mtgl::HostStage stage;
    mtgl::Pass pass;
    mtgl_stats stats{};
    uint64_t alloc_base = 0;  // allocation count at the last reset of the counters
    bool depth_rejection = true;
    bool mipmap_chain = false;  // MTGL_OPT_MIPMAP_CHAIN
    // ordering against batches, which run on their own streams: work of this context's
    // stream that a batch must wait for, and a batch this context's stream must wait for
    cudaEvent_t tail = nullptr;
    bool dirty = false;
    mtgl::RunMark *after_batch = nullptr;  // end of the last batch run that wrote this context
    cudaStream_t after_stream = nullptr;   // the stream that run was on
    mtgl_batch *batch = nullptr;  // an unverified batch that writes this context's framebuffer
    std::vector<mtgl_batch *> readers;  // unfinished batches that read this context's resources
};

// Every entry that enqueues work on a context's stream goes through here first.
int mtgl_dev_enter(mtgl_dev *d);
