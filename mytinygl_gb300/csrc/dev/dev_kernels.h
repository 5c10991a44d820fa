// dev_kernels.h — host-side launchers of the sm_103a kernels (one translation unit each).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "mtgl_device.cuh"

namespace mtgl {

constexpr uint32_t kClipClasses = 96;  // one-plane candidates: first plane x in/out pattern; the rest
// Each class is counted in kClipSlots counters (a block of the count pass uses slot
// blockIdx % kClipSlots), so that the appends of many blocks do not all meet on a few words.
constexpr uint32_t kClipSlots = 32;
constexpr int kDebugStatusWord = 8;  // word of an Exec's counters that the debug bounds checks write
constexpr uint32_t kClipBuckets = kClipClasses * kClipSlots;  // class-major

struct GeomArgs {
    const DevDraw *draws;
    const uint32_t *draw_vslot_base;  // per draw, ascending
    const uint32_t *draw_tri_base;    // per draw, ascending
    int32_t ndraws;
    const mtgl_vertex_state *vstates;
    const DevRaster *rasters;
    PostVertices verts;
    PostEye *eyes;                    // null when no draw of the pass lights per fragment
    uint32_t total_slots;
    uint32_t total_tris;
    const DevFrame *frames;           // the raster state's `frame` indexes this table
    uint32_t nframes;
    uint32_t *tri_counts;             // count pass output
    const uint32_t *tri_offsets;      // emit pass input (exclusive scan of tri_counts)
    float *records;                   // emit pass output, kRecWords per record
    float *eye_records;               // emit pass output, kEyeWords per record (may be null)
    uint32_t records_cap;             // records the output buffers hold (writes beyond are dropped)
    uint32_t *clip_list;              // triangles that straddle a clip plane (total_tris entries)
    uint32_t *clip_class;             // per entry: bucket << 20 | rank within the bucket
    uint32_t *clip_sorted;            // the entries grouped by class (null: process clip_list as is)
    uint32_t *class_count;            // kClipBuckets counters (zeroed by the count launch)
    uint32_t *emit_list;              // primitives the set-up emit pass writes (count pass output; unordered)
    uint32_t *list_counts;            // entries of [0] the clip list, [1] the emit list (device; zeroed
                                      // by the count launch)
    int32_t sms;
    uint32_t *debug;                  // status word of the debug bounds checks
};

// K1: per-vertex stage (gl_api.c:263-348) for every vertex slot of the pass.
int launch_vertex(const GeomArgs &a, cudaStream_t s);
// K2: primitive assembly, clipping, perspective divide, culling and triangle setup
// (raster.c:451-529, 729-1017, 1199-1231); count pass then emit pass.
int launch_setup_count(const GeomArgs &a, cudaStream_t s);
int launch_setup_emit(const GeomArgs &a, cudaStream_t s);

// Every launcher returns the number of kernels it launched.

// Device-wide exclusive scan of n uint32 values (in place allowed; one launch); writes the
// total to *total_dev. in and out 16-byte aligned; temp must hold scan_temp_words(n) words,
// 8-byte aligned; debug is the
// status word its bounded waits report to (may be null).
size_t scan_temp_words(uint32_t n);
int launch_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *temp, uint32_t *total_dev, uint32_t *debug,
                cudaStream_t s);

// Element counts of the binning stage live on the device (written by the scans), so the
// stage runs without the host knowing them. `nrec` / `npairs` on the host are capacities:
// they size grids and buffers, and kernels read the real counts through nrec_dev / total_dev.
struct BinArgs {
    const float *records;
    uint32_t nrec;              // record capacity
    const uint32_t *nrec_dev;   // records written (may exceed nrec: the excess was dropped)
    const DevFrame *frames;
    uint32_t nframes;
    int32_t tile_shift;         // tile edge = 1 << tile_shift
    uint32_t ntiles;            // tiles of all frames
    uint32_t *rec_tiles;        // per record tile count, then its exclusive scan (in place)
    uint32_t *keys, *vals;      // pair buffers (capacity >= pairs)
    uint32_t *keys_alt, *vals_alt;
    uint32_t *tile_count;       // per tile (ntiles + 1 entries)
    uint32_t *tile_area;        // per tile: pixels of its records' boxes inside it, summed (may be null)
    uint32_t *tile_start;       // exclusive scan of tile_count
    uint32_t *tile_frame;       // per tile: the frame owning it (written by the range pass; may be null)
    uint32_t *radix_hist;       // radix histograms
    uint32_t *scan_temp;
    uint32_t *total_dev;        // where the pair scan writes its total: the pairs generated
    uint32_t *sort_total_dev;   // a word the sort's histogram scans may overwrite
    uint32_t npairs;            // pair capacity of keys/vals (writes beyond are dropped)
    int32_t sms;                // SMs of the device (grid sizes)
    uint32_t *debug;            // status word of the debug bounds checks
};

int launch_bin_count(const BinArgs &a, cudaStream_t s);
int launch_bin_expand(const BinArgs &a, cudaStream_t s);
// Stable sort of (tile, record) pairs by tile; result in keys/vals. Uses keys_alt/vals_alt
// as ping-pong storage.
int launch_bin_sort(BinArgs &a, cudaStream_t s);
size_t radix_hist_words(uint32_t npairs);
// Each tile's range of the sorted pairs: tile_start and tile_count (zero for a tile with no
// pairs), read off the sorted keys where the tile id changes. tile_start and tile_count must
// be zero for every tile on entry.
int launch_tile_ranges(const BinArgs &a, cudaStream_t s);

// Work order of the persistent tile launches. Tiles whose records are small (their boxes
// cover on average less than a quarter of the tile) come first, then the others; each group
// by descending record count (coarse log buckets), so the longest tiles start first. The
// split point is written to aux[kOrderSplit]. order holds ntiles words, aux kOrderAuxWords.
int launch_tile_order(const uint32_t *tile_count, const uint32_t *tile_area, uint32_t ntiles, int tile_shift,
                      uint32_t *aux, uint32_t *order, int sms, cudaStream_t s);
constexpr size_t kOrderSplit = 1024;      // aux word: number of small-record tiles
constexpr size_t kOrderQueues = 1028;     // aux words: work-queue heads of the tile launches
constexpr size_t kOrderAuxWords = 1040;

// A tile's class: 0 when its records are small (their boxes cover on average under a quarter
// of the tile), else 1. Empty tiles are class 1.
__device__ __forceinline__ uint32_t tile_class(const uint32_t *tile_count, const uint32_t *tile_area, uint32_t t,
                                               int tile_shift)
{
    const uint32_t c = tile_count[t];
    if (c == 0 || !tile_area) return 1u;
    return (uint64_t)tile_area[t] * 4u < ((uint64_t)c << (2 * tile_shift)) ? 0u : 1u;
}

struct TileArgs {
    const float *records;
    const float *eye_records;
    const uint32_t *tile_vals;   // record indices sorted by tile, submission order within a tile
    uint32_t *pair_mask;         // per entry of tile_vals: the warp blocks that walk it (written
                                 // by the tile's CTA; binning's sorted keys, no longer read)
    const uint32_t *tile_start;  // per tile
    const uint32_t *tile_count;
    const uint32_t *tile_frame;  // per tile: its frame (null: found by a search of the frame table)
    const DevRaster *rasters;
    uint32_t nrasters;
    const ClearOp *clears;       // all frames' clears; a frame holds its range
    const DevFrame *frames;
    uint32_t nframes;
    uint32_t ntiles;             // work items: global tile ids
    const uint32_t *order;       // item -> tile (null: item i is tile i)
    const uint32_t *split;       // items [0, *split) have small records (null: no split)
    const uint32_t *tile_area;   // without an order: per-tile record-box coverage; each launch
                                 // takes the tiles of its class in tile order (null: no classes)
    uint32_t *queue;             // work-queue heads (two), zero at launch
    int32_t ctas;                // persistent CTAs (0: one per tile)
    int32_t tile_shift;
    int32_t any_texture;         // some raster state of the pass samples a texture
    // capacity check: when guard[0] > records_cap or guard[1] > pairs_cap the binning
    // dropped entries, and the launch leaves every framebuffer untouched
    const uint32_t *guard;
    uint32_t records_cap, pairs_cap;
    unsigned long long *fragments;
    int32_t defer;               // every record is a filled triangle with deferrable colour (k_tile.cuh)
    uint32_t *debug;             // status word of the debug bounds checks
    uint32_t entries_cap;        // entries tile_vals holds (debug bounds checks)
};

// K4: CTAs take tiles from the work queue; for each: clears, then every triangle of the
// tile in order through the full fragment pipeline (raster.c:532-724), then one write-back.
int launch_tile(const TileArgs &a, cudaStream_t s);
// resident CTAs per SM of the K4 variant a launch with these arguments uses
int tile_occupancy(const TileArgs &a);

// glClear without draws (gl_api.c:409-457)
void launch_clear(const ClearOp *ops_host, int nops, FrameDims dims, uint32_t *color, float *depth, uint8_t *stencil,
                  cudaStream_t s);
// mip level 1 (textures.c:311-354)
void launch_mip1(const uint32_t *base, int32_t w, int32_t h, uint32_t *mip, cudaStream_t s);
// glDrawPixels blit (gl_api.c:1287-1376)
void launch_draw_pixels(const uint32_t *img, int32_t rx, int32_t ry, int32_t w, int32_t h, const DevRaster *raster,
                        FrameDims dims, uint32_t *color, float *depth, cudaStream_t s);

// Colour read-back by kernel into page-locked host memory mapped into the device's address
// space (dst is the device-side address): one launch per kReadbackMax items, the items in the
// launch's parameters. Returns the kernels launched.
struct ReadbackItem {
    const uint32_t *src;  // device colour buffer
    uint32_t *dst;        // device address of the host buffer
    uint32_t n;           // pixels
    uint32_t first_unit;  // set by the launcher
};
constexpr int kReadbackMax = 128;
constexpr uint32_t kReadbackUnit = 4096;  // pixels per work unit
struct ReadbackArgs {
    ReadbackItem item[kReadbackMax];
    int32_t count;
    uint32_t units;
};
int launch_readback(const ReadbackItem *items, int n, int sms, cudaStream_t s);

}  // namespace mtgl
