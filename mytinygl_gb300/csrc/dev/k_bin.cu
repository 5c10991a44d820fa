// k_bin.cu — K3 binning: triangle records -> per-tile lists in submission order.
//
// No counterpart in the reference, which scans every triangle's bounding box on one thread
// (raster.c:532-724). Here each record is expanded into one (tile, record) pair per tile
// (8, 16 or 32 pixels square) of its clamped bounding box in which it can cover a pixel (an
// exact edge test per tile for triangles); pairs are generated in submission order and a
// stable LSD radix sort on the tile id (warp match-any ranking plus prefix sums) groups
// them by tile while keeping that order inside every tile. The tile kernel then walks each
// list front to back, so blending and stencil updates happen in GL order.
#include <algorithm>

#include "dev_kernels.h"

namespace mtgl {

// ------------------------------------------------------------------ scan

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // 2048 values per block

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// exclusive block scan of one value per thread; returns the block total in *total
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total)
{
    __shared__ uint32_t warp_sums[kScanThreads / 32 + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = warp_incl_scan(v);
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
        uint32_t wi = warp_incl_scan(w);
        if (lane < kScanThreads / 32) warp_sums[lane] = wi - w;
        if (lane == kScanThreads / 32 - 1) warp_sums[kScanThreads / 32] = wi;
    }
    __syncthreads();
    uint32_t r = warp_sums[warp] + incl - v;
    *total = warp_sums[kScanThreads / 32];
    __syncthreads();
    return r;
}

// Single-pass exclusive scan with decoupled look-back (Merrill and Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", 2016). Blocks take their tile of kScanTile
// values in the order they start (a ticket), publish the tile's sum, then walk back over
// the tiles before theirs, 32 at a time, adding published sums until one publishes its
// inclusive prefix.
// A tile's status word: (flag << 32) | value, flag 0 = nothing yet, 1 = the tile's sum,
// 2 = the inclusive prefix through the tile; written whole, so a reader sees one or the other.
// A tile before a block's own was taken by a block that started earlier and publishes its sum
// without waiting, so every wait ends; each is still bounded (kScanWaitLimit reads) and a
// wait that runs out is recorded in the debug status word and counts the tile as empty.
constexpr uint32_t kScanWaitLimit = 1u << 24;
constexpr uint64_t kScanSum = 1ull << 32, kScanPrefix = 2ull << 32;

__device__ __forceinline__ uint64_t ld_status(const uint64_t *p) { return *(const volatile uint64_t *)p; }
__device__ __forceinline__ void st_status(uint64_t *p, uint64_t v) { *(volatile uint64_t *)p = v; }

__global__ void __launch_bounds__(kScanThreads) k_scan(const uint32_t *in, uint32_t *out, uint32_t n,
                                                      uint64_t *status, uint32_t *ticket, uint32_t *total_dev,
                                                      uint32_t *debug)
{
    __shared__ uint32_t s_tile, s_prefix;
    if (threadIdx.x == 0) s_tile = gridDim.x == 1 ? 0u : atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * (uint32_t)kScanTile + threadIdx.x * kScanItems;
    // each thread's 8 values as two 16-byte words (base is a multiple of 8 words)
    uint32_t v[kScanItems];
    if (base + kScanItems <= n) {
        const uint4 a = *reinterpret_cast<const uint4 *>(in + base), b = *reinterpret_cast<const uint4 *>(in + base + 4);
        v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; i++) v[i] = (base + i < n) ? in[base + i] : 0u;
    }
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) sum += v[i];
    uint32_t agg;
    uint32_t run = block_excl_scan(sum, &agg);
    if (threadIdx.x < 32) {
        // warp 0 looks back 32 tiles at a time: lane k reads the status of tile (window - k)
        const uint32_t lane = threadIdx.x;
        uint32_t prefix = 0;
        if (tile == 0) {
            if (lane == 0) st_status(status, kScanPrefix | agg);
        } else {
            if (lane == 0) st_status(status + tile, kScanSum | agg);
            for (int64_t win = (int64_t)tile - 1;; win -= 32) {
                const int64_t p = win - (int64_t)lane;
                uint64_t st = p >= 0 ? ld_status(status + p) : kScanPrefix;  // before tile 0: a zero prefix
                for (uint32_t w = 0; !__all_sync(0xffffffffu, (st >> 32) != 0);) {
                    if (++w < kScanWaitLimit) {
                        if ((st >> 32) == 0) st = ld_status(status + p);
                    } else if ((st >> 32) == 0) {
                        st = kScanSum;  // counted as empty
                        if (debug) atomicCAS(debug, 0u, (uint32_t)DBG_SCAN_WAIT);
                    }
                }
                // the nearest tile with its inclusive prefix ends the walk; the nearer ones add sums
                const uint32_t prefixed = __ballot_sync(0xffffffffu, (st >> 32) == 2);
                const uint32_t upto = prefixed ? (uint32_t)__ffs(prefixed) - 1u : 31u;
                prefix += __reduce_add_sync(0xffffffffu, lane <= upto ? (uint32_t)st : 0u);
                if (prefixed) break;
            }
            if (lane == 0) st_status(status + tile, kScanPrefix | (prefix + agg));
        }
        if (lane == 0) {
            s_prefix = prefix;
            if (tile + 1 == gridDim.x) *total_dev = prefix + agg;
        }
    }
    __syncthreads();
    run += s_prefix;
    uint32_t o[kScanItems];
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        o[i] = run;
        run += v[i];
    }
    if (base + kScanItems <= n) {
        *reinterpret_cast<uint4 *>(out + base) = make_uint4(o[0], o[1], o[2], o[3]);
        *reinterpret_cast<uint4 *>(out + base + 4) = make_uint4(o[4], o[5], o[6], o[7]);
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; i++)
            if (base + i < n) out[base + i] = o[i];
    }
}

size_t scan_temp_words(uint32_t n)
{
    // a 64-bit status word per tile, then the ticket
    return 2 * (((size_t)n + kScanTile - 1) / kScanTile) + 64;
}

int launch_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *temp, uint32_t *total_dev, uint32_t *debug,
                cudaStream_t s)
{
    if (n == 0) {
        cudaMemsetAsync(total_dev, 0, sizeof(uint32_t), s);
        return 0;
    }
    const uint32_t nb = (n + kScanTile - 1) / kScanTile;
    // temp is 8-byte aligned (scratch slices start on 256-byte boundaries); a single tile needs
    // neither tickets nor statuses (and so no clearing)
    uint64_t *status = reinterpret_cast<uint64_t *>(temp);
    uint32_t *ticket = temp + 2 * (size_t)nb;
    if (nb > 1) cudaMemsetAsync(temp, 0, (2 * (size_t)nb + 1) * sizeof(uint32_t), s);
    k_scan<<<nb, kScanThreads, 0, s>>>(in, out, n, status, ticket, total_dev, debug);
    return 1;
}

// ------------------------------------------------------------------ record -> tiles

// The setup kernel clamps every bbox to its framebuffer; the clamps here only keep tile
// indices inside the frame's tile grid whatever a record holds. Returns the frame.
__device__ __forceinline__ const DevFrame &rec_tile_box(const float *rec, const BinArgs &A, int &tx0, int &ty0,
                                                        int &tx1, int &ty1)
{
    const float4 b1 = __ldg(reinterpret_cast<const float4 *>(rec) + 1);
    const float4 b2 = __ldg(reinterpret_cast<const float4 *>(rec) + 2);
    const uint32_t f = min(__float_as_uint(__ldg(rec + R_FRAME)), A.nframes - 1);
    const DevFrame &F = A.frames[f];
    const int sh = A.tile_shift;
    tx0 = min(max(__float_as_int(b1.z), 0), F.dims.width - 1) >> sh;
    ty0 = min(max(__float_as_int(b1.w), 0), F.dims.height - 1) >> sh;
    tx1 = max(min(__float_as_int(b2.x), F.dims.width - 1) >> sh, tx0);
    ty1 = max(min(__float_as_int(b2.y), F.dims.height - 1) >> sh, ty0);
    return F;
}

__device__ __forceinline__ uint32_t records_in(const BinArgs &A) { return min(*A.nrec_dev, A.nrec); }

// The tiles of a record's box that get a pair: every tile for points and lines; for a
// triangle, the tiles in which its coverage test (edge functions at integer pixel positions,
// raster.c:299-302, 534-536) can pass. k_bin_count counts them and k_bin_expand writes them,
// with this one test.
//
// The record's positions and per-edge differences are integer-valued floats. When every
// product (px - ax) * A, (py - ay) * B that the per-pixel test forms over the box's tiles is
// below 2^24 in magnitude, those products are exact, so each edge function's sign per pixel
// is the sign of the exact integer. Then each edge's largest value over a tile (a corner:
// the function is affine) is an int32 stepped per tile column and row, and a tile whose
// largest value is negative for some edge has no pixel the test passes (for a negative
// area the signs flip). Otherwise every tile of the box gets a pair.
struct RecTiles {
    int tx0, ty0, w, cnt;  // the box in tiles, row-major, cnt tiles
    int mode;              // kAll, kNone or kTest
    int e00[3], sx[3], sy[3];  // per edge: value at the first tile's corner, steps per column / row
};
constexpr int kAll = 0, kNone = 1, kTest = 2;
constexpr int kTestMinTiles = 4;  // smaller boxes keep every tile: little to drop, and the set-up dominates

__device__ __forceinline__ const DevFrame &rec_tiles_of(const BinArgs &A, uint32_t r, RecTiles &t)
{
    const float *rec = A.records + (size_t)r * kRecWords;
    int tx1, ty1;
    const DevFrame &F = rec_tile_box(rec, A, t.tx0, t.ty0, tx1, ty1);
    t.w = tx1 - t.tx0 + 1;
    t.cnt = t.w * (ty1 - t.ty0 + 1);
    const float4 *q = reinterpret_cast<const float4 *>(rec);
    t.mode = kAll;
    if (t.cnt < kTestMinTiles) return F;
    const float4 q12 = __ldg(q + 12);
    if (((__float_as_uint(q12.x) >> kRecTypeShift) & 3u) != REC_TRI) return F;
    const float4 q0 = __ldg(q + 0), q1 = __ldg(q + 1), q2 = __ldg(q + 2), q13 = __ldg(q + 13);
    const float area = q2.z;
    if (!(area > 0.0f) && !(area < 0.0f)) {  // zero or NaN area: the test never passes
        t.mode = kNone;
        return F;
    }
    const int sh = A.tile_shift, ts = 1 << sh;
    const int xl = t.tx0 << sh, xh = (tx1 << sh) + ts - 1, yl = t.ty0 << sh, yh = (ty1 << sh) + ts - 1;
    const float ax[3] = {q0.z, q1.x, q0.x}, ay[3] = {q0.w, q1.y, q0.y};
    const float ea[3] = {q12.y, q12.w, q13.y}, eb[3] = {q12.z, q13.x, q13.z};
    const bool pos = area > 0.0f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        constexpr float kLim = 16777216.0f;  // 2^24
        if (!(fabsf(ax[k]) < kLim && fabsf(ay[k]) < kLim && fabsf(ea[k]) < kLim && fabsf(eb[k]) < kLim)) return F;
        const int iax = (int)ax[k], iay = (int)ay[k];
        const int a = pos ? (int)ea[k] : -(int)ea[k], b = pos ? (int)eb[k] : -(int)eb[k];
        const long long mx = max(llabs((long long)xl - iax), llabs((long long)xh - iax)) * llabs((long long)a);
        const long long my = max(llabs((long long)yl - iay), llabs((long long)yh - iay)) * llabs((long long)b);
        if (mx >= (1ll << 24) || my >= (1ll << 24)) return F;
        // (x - ax) * a - (y - ay) * b is largest over a tile at x = right edge when a >= 0,
        // y = top row when b >= 0
        const int cx = xl + (a >= 0 ? ts - 1 : 0), cy = yl + (b >= 0 ? 0 : ts - 1);
        t.e00[k] = (cx - iax) * a - (cy - iay) * b;
        t.sx[k] = a * ts;
        t.sy[k] = b * ts;
    }
    t.mode = kTest;
    return F;
}

// the i-th tile of the box (row-major) gets a pair
__device__ __forceinline__ bool tile_gets_pair(const RecTiles &t, int i)
{
    if (t.mode != kTest) return t.mode == kAll;
    const int col = i % t.w, row = i / t.w;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 3; k++) ok = ok && t.e00[k] + col * t.sx[k] - row * t.sy[k] >= 0;
    return ok;
}

constexpr uint32_t kCountLanes = 2;  // lanes per record in k_bin_count (16 records per warp)

// pairs per record; records past the real count get 0 so the scan over the capacity is exact
__global__ void __launch_bounds__(256) k_bin_count(BinArgs A)
{
    const uint32_t n = records_in(A);
    constexpr uint32_t L = kCountLanes, G = 32 / kCountLanes;
    const uint32_t lane = threadIdx.x & 31u, sub = lane / L, sl = lane % L;
    const uint32_t gmask = ((1u << L) - 1u) << (sub * L);
    const uint32_t groups = gridDim.x * (blockDim.x >> 5) * G;
    for (uint32_t r0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * G; r0 < A.nrec; r0 += groups) {
        const uint32_t r = r0 + sub;
        if (r >= A.nrec) continue;
        uint32_t c = 0;
        if (r < n) {
            RecTiles t;
            rec_tiles_of(A, r, t);
            if (t.mode == kAll) {
                c = sl == 0 ? (uint32_t)t.cnt : 0u;
            } else if (t.mode == kTest) {
                for (int i = (int)sl; i < t.cnt; i += (int)L) c += tile_gets_pair(t, i) ? 1u : 0u;
            }
        }
        c = __reduce_add_sync(gmask, c);
        if (sl == 0) A.rec_tiles[r] = c;
    }
}

// A group of L lanes per record (L = 32 / G, G records per warp from the average pairs per
// record: 1 for large triangles, up to 8 for small ones, so that a warp has several records'
// loads in flight): the group tests its record's box tiles row-major and writes the pairs of
// those that get one, in that order (pairs stay in submission order within every tile).
__global__ void __launch_bounds__(256) k_bin_expand(BinArgs A)
{
    const uint32_t n = records_in(A);
    const uint32_t avg = n ? max(1u, *A.total_dev / n) : 1u;
    const uint32_t G = avg >= 32u ? 1u : (avg >= 16u ? 2u : (avg >= 8u ? 4u : 8u));
    const uint32_t L = 32u / G;
    const uint32_t lane = threadIdx.x & 31u, sub = lane / L, sl = lane % L;
    const uint32_t lmask = L == 32u ? 0xFFFFFFFFu : (1u << L) - 1u;
    const uint32_t gmask = lmask << (sub * L);
    const uint32_t groups = gridDim.x * (blockDim.x >> 5) * G;
    const int sh = A.tile_shift;
    for (uint32_t r = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * G + sub; r < n; r += groups) {
        RecTiles t;
        const DevFrame &F = rec_tiles_of(A, r, t);
        const float *rec = A.records + (size_t)r * kRecWords;
        const float4 b1 = __ldg(reinterpret_cast<const float4 *>(rec) + 1);
        const float4 b2 = __ldg(reinterpret_cast<const float4 *>(rec) + 2);
        const int bx0 = __float_as_int(b1.z), by0 = __float_as_int(b1.w);
        const int bx1 = __float_as_int(b2.x), by1 = __float_as_int(b2.y);
        const uint32_t base = A.rec_tiles[r];
        uint32_t run = 0;  // pairs of this record written so far
        for (int i0 = 0; i0 < t.cnt; i0 += (int)L) {
            const int i = i0 + (int)sl;
            const int tx = t.tx0 + i % t.w, ty = t.ty0 + i / t.w;
            const bool get = i < t.cnt && tile_gets_pair(t, i);
            const uint32_t m = (__ballot_sync(gmask, get) >> (sub * L)) & lmask;
            const uint32_t at = base + run + (uint32_t)__popc(m & ((1u << sl) - 1u));
            run += (uint32_t)__popc(m);
            if (!get || at >= A.npairs) continue;
            const uint32_t tile = F.tile_base + (uint32_t)(ty * F.dims.tiles_x + tx);
            A.keys[at] = tile;
            A.vals[at] = r;
            if (A.tile_area) {  // pixels of the record's box inside this tile
                const int ox = min(bx1, ((tx + 1) << sh) - 1) - max(bx0, tx << sh) + 1;
                const int oy = min(by1, ((ty + 1) << sh) - 1) - max(by0, ty << sh) + 1;
                atomicAdd(A.tile_area + tile, (uint32_t)(ox * oy));
            }
        }
    }
}

// grids cover the work or the GPU (16 CTAs per SM), whichever is smaller; kernels loop over the rest
unsigned stride_grid(uint64_t threads, unsigned block, int sms)
{
    const uint64_t want = (threads + block - 1) / block;
    const uint64_t cap = (uint64_t)(sms > 0 ? sms : 1) * 16;
    return (unsigned)std::max<uint64_t>(1, std::min(want, cap));
}

// Where the sorted tile id changes, the earlier tile's range ends and the later one's
// starts: the first writes the end position into tile_count, the second its start.
__global__ void __launch_bounds__(256) k_tile_bounds(BinArgs A)
{
    const uint32_t n = min(*A.total_dev, A.npairs);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = A.keys[i];
        if (!debug_check(A.debug, k < A.ntiles, DBG_BIN_TILE)) continue;
        if (i == 0 || A.keys[i - 1] != k) A.tile_start[k] = i;
        if (i + 1 == n || A.keys[i + 1] != k) A.tile_count[k] = i + 1;
    }
}

// end position - start = count; a tile without pairs has both still zero. Also the frame
// that owns each tile (the last frame whose first tile is at or before it), so the tile
// kernel reads it instead of searching the frame table per tile.
__global__ void __launch_bounds__(256) k_tile_counts(BinArgs A)
{
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < A.ntiles; t += gridDim.x * blockDim.x) {
        A.tile_count[t] -= A.tile_start[t];
        if (A.tile_frame) {
            uint32_t lo = 0, hi = A.nframes - 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (A.frames[mid].tile_base <= t) lo = mid;
                else hi = mid - 1;
            }
            A.tile_frame[t] = lo;
        }
    }
}

int launch_tile_ranges(const BinArgs &a, cudaStream_t s)
{
    if (a.npairs) k_tile_bounds<<<stride_grid(a.npairs, 256, a.sms), 256, 0, s>>>(a);
    k_tile_counts<<<stride_grid(a.ntiles, 256, a.sms), 256, 0, s>>>(a);
    return a.npairs ? 2 : 1;
}

int launch_bin_count(const BinArgs &a, cudaStream_t s)
{
    if (!a.nrec) return 0;
    k_bin_count<<<stride_grid((uint64_t)a.nrec * kCountLanes, 256, a.sms), 256, 0, s>>>(a);
    return 1;
}

int launch_bin_expand(const BinArgs &a, cudaStream_t s)
{
    if (!a.nrec) return 0;
    k_bin_expand<<<stride_grid((uint64_t)a.nrec * 32, 256, a.sms), 256, 0, s>>>(a);
    return 1;
}

// ------------------------------------------------------------------ persistent work order

// coarse log2 bucket of a tile's record count: 8 steps per octave, 0 for an empty tile
__device__ __forceinline__ uint32_t cost_bucket(uint32_t c)
{
    if (c == 0) return 0;
    const int lg = 31 - __clz(c);
    const uint32_t frac = lg >= 3 ? (c >> (lg - 3)) & 7u : (c << (3 - lg)) & 7u;
    return min(1u + (uint32_t)lg * 8u + frac, 255u);
}

// aux[0..511]: tiles per (class, bucket); aux[512..1023]: placement cursors; all zero at launch
__global__ void __launch_bounds__(256) k_order_hist(const uint32_t *tile_count, const uint32_t *tile_area,
                                                    uint32_t ntiles, int tile_shift, uint32_t *aux)
{
    __shared__ uint32_t h[512];
    h[threadIdx.x] = 0;
    h[threadIdx.x + 256] = 0;
    __syncthreads();
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x)
        atomicAdd(&h[tile_class(tile_count, tile_area, t, tile_shift) * 256 + cost_bucket(tile_count[t])], 1u);
    __syncthreads();
    if (h[threadIdx.x]) atomicAdd(&aux[threadIdx.x], h[threadIdx.x]);
    if (h[threadIdx.x + 256]) atomicAdd(&aux[threadIdx.x + 256], h[threadIdx.x + 256]);
}

// Places every tile after all tiles of earlier groups: class 0 before class 1, costlier
// buckets first within a class. The order inside a bucket is whatever the atomics give:
// tiles are independent, so it changes timing only.
__global__ void __launch_bounds__(256) k_order_scatter(const uint32_t *tile_count, const uint32_t *tile_area,
                                                       uint32_t ntiles, int tile_shift, uint32_t *aux,
                                                       uint32_t *order)
{
    __shared__ uint32_t start[512];
    __shared__ uint32_t warp_tot[8];
    // positions p = 2*thread, 2*thread+1 in placement order: class p / 256, bucket 255 - p % 256
    const int p0 = 2 * (int)threadIdx.x, p1 = p0 + 1;
    const int e0 = (p0 / 256) * 256 + (255 - p0 % 256), e1 = (p1 / 256) * 256 + (255 - p1 % 256);
    const uint32_t v0 = aux[e0], v1 = aux[e1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v0 + v1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; w++) before += warp_tot[w];
    const uint32_t excl = before + x - (v0 + v1);
    start[e0] = excl;
    start[e1] = excl + v0;
    if (blockIdx.x == 0 && threadIdx.x == 127) aux[kOrderSplit] = before + x;  // end of class 0
    __syncthreads();
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
        const uint32_t e = tile_class(tile_count, tile_area, t, tile_shift) * 256 + cost_bucket(tile_count[t]);
        order[start[e] + atomicAdd(&aux[512 + e], 1u)] = t;
    }
}

int launch_tile_order(const uint32_t *tile_count, const uint32_t *tile_area, uint32_t ntiles, int tile_shift,
                      uint32_t *aux, uint32_t *order, int sms, cudaStream_t s)
{
    if (!ntiles) return 0;
    cudaMemsetAsync(aux, 0, kOrderAuxWords * sizeof(uint32_t), s);
    const unsigned g = stride_grid(ntiles, 256, sms);
    k_order_hist<<<g, 256, 0, s>>>(tile_count, tile_area, ntiles, tile_shift, aux);
    k_order_scatter<<<g, 256, 0, s>>>(tile_count, tile_area, ntiles, tile_shift, aux, order);
    return 2;
}

// ------------------------------------------------------------------ stable radix sort by tile

constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kRadixItems = 8;  // per thread
constexpr int kRadixTile = kRadixThreads * kRadixItems;
constexpr int kRadixDigits = 512;  // up to 9-bit digits; a sort uses ceil(bits / 9) balanced passes

size_t radix_hist_words(uint32_t npairs)
{
    const size_t nb = (npairs + kRadixTile - 1) / kRadixTile;
    return nb * kRadixDigits + 64;
}

__global__ void __launch_bounds__(kRadixThreads) k_radix_hist(const uint32_t *keys, uint32_t cap,
                                                             const uint32_t *n_dev, int shift, uint32_t mask,
                                                             uint32_t *hist, uint32_t nblocks)
{
    const uint32_t n = min(*n_dev, cap);
    const int ndig = (int)mask + 1;
    __shared__ uint32_t h[kRadixDigits];
    for (int i = threadIdx.x; i < ndig; i += kRadixThreads) h[i] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * (uint32_t)kRadixTile;
#pragma unroll
    for (int k = 0; k < kRadixItems; k++) {
        const uint32_t i = base + k * kRadixThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & mask], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < ndig; d += kRadixThreads) hist[(size_t)d * nblocks + blockIdx.x] = h[d];
}

// Stable scatter: warp w owns items [w*256, w*256+256) of the block, taken 32 at a time in
// order; match-any groups equal digits, the leader advances the warp's digit counter, and
// per-digit prefix sums over warps and blocks place every item after all earlier ones. The
// block first sorts its items by digit in shared memory, so that each digit's run leaves
// as consecutive addresses (coalesced writes) rather than one scattered word per item.
__global__ void __launch_bounds__(kRadixThreads) k_radix_scatter(const uint32_t *keys, const uint32_t *vals,
                                                                uint32_t cap, const uint32_t *n_dev, int shift,
                                                                uint32_t mask,
                                                                const uint32_t *hist_scan, uint32_t nblocks,
                                                                uint32_t *keys_out, uint32_t *vals_out)
{
    __shared__ uint32_t wcount[kRadixWarps][kRadixDigits];  // per warp and digit: count, then block-local start
    __shared__ uint32_t dstart[kRadixDigits];                // block-local start of each digit's run
    __shared__ uint32_t gdelta[kRadixDigits];                // global start minus block-local start
    __shared__ uint32_t skey[kRadixTile], sval[kRadixTile];
    const uint32_t n = min(*n_dev, cap);
    const int ndig = (int)mask + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kRadixWarps * kRadixDigits; i += kRadixThreads) (&wcount[0][0])[i] = 0;
    __syncthreads();
    const uint32_t bbase = blockIdx.x * (uint32_t)kRadixTile;
    const uint32_t wbase = bbase + warp * 32 * kRadixItems;
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t key[kRadixItems], val[kRadixItems], rank[kRadixItems];
#pragma unroll
    for (int k = 0; k < kRadixItems; k++) {
        const uint32_t i = wbase + k * 32 + lane;
        const bool valid = i < n;
        key[k] = valid ? keys[i] : 0u;
        val[k] = valid ? vals[i] : 0u;
        const uint32_t d = valid ? ((key[k] >> shift) & mask) : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        const uint32_t pre = valid ? wcount[warp][d] : 0u;
        __syncwarp();
        if (valid && lane == leader) wcount[warp][d] = pre + __popc(peers);
        __syncwarp();
        rank[k] = pre + __popc(peers & lt);
    }
    __syncthreads();
    // per digit: the block's count, then each warp's start within the digit's run
    for (int d = threadIdx.x; d < kRadixDigits; d += kRadixThreads) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kRadixWarps; w++) {
            const uint32_t c = d < ndig ? wcount[w][d] : 0u;
            wcount[w][d] = run;
            run += c;
        }
        dstart[d] = run;  // the count for now
    }
    __syncthreads();
    // exclusive scan of the digit counts (512 entries, 2 per thread) into block-local starts
    {
        const int d0 = 2 * threadIdx.x;
        const uint32_t c0 = dstart[d0], c1 = dstart[d0 + 1];
        uint32_t incl = c0 + c1, x = incl;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        __shared__ uint32_t wsum[kRadixWarps];
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        uint32_t before = 0;
        for (int w = 0; w < warp; w++) before += wsum[w];
        const uint32_t excl = before + x - incl;
        __syncthreads();
        dstart[d0] = excl;
        dstart[d0 + 1] = excl + c0;
        if (d0 < ndig) gdelta[d0] = hist_scan[(size_t)d0 * nblocks + blockIdx.x] - excl;
        if (d0 + 1 < ndig) gdelta[d0 + 1] = hist_scan[(size_t)(d0 + 1) * nblocks + blockIdx.x] - (excl + c0);
    }
    __syncthreads();
    // items into shared memory in digit order (stable: warp order, then item order)
#pragma unroll
    for (int k = 0; k < kRadixItems; k++) {
        const uint32_t i = wbase + k * 32 + lane;
        if (i < n) {
            const uint32_t d = (key[k] >> shift) & mask;
            const uint32_t at = dstart[d] + wcount[warp][d] + rank[k];
            skey[at] = key[k];
            sval[at] = val[k];
        }
    }
    __syncthreads();
    // consecutive slots of one digit go to consecutive global positions
    const uint32_t valid_n = n > bbase ? min((uint32_t)kRadixTile, n - bbase) : 0u;
#pragma unroll
    for (int k = 0; k < kRadixItems; k++) {
        const uint32_t at = k * kRadixThreads + threadIdx.x;
        if (at < valid_n) {
            const uint32_t kk = skey[at];
            const uint32_t pos = gdelta[(kk >> shift) & mask] + at;
            keys_out[pos] = kk;
            vals_out[pos] = sval[at];
        }
    }
}

int launch_bin_sort(BinArgs &a, cudaStream_t s)
{
    const uint32_t n = a.npairs;  // capacity; the kernels read the real count from total_dev
    if (n == 0) return 0;
    int launches = 0;
    int bits = 1;
    while (bits < 32 && (1u << bits) < a.ntiles) bits++;
    const int passes = (bits + 8) / 9;
    const int width = (bits + passes - 1) / passes;  // balanced digits of at most 9 bits
    const uint32_t nb = (n + kRadixTile - 1) / kRadixTile;
    for (int shift = 0; shift < bits; shift += width) {
        const int nbits = (bits - shift) < width ? (bits - shift) : width;
        const uint32_t mask = (1u << nbits) - 1u;
        k_radix_hist<<<nb, kRadixThreads, 0, s>>>(a.keys, n, a.total_dev, shift, mask, a.radix_hist, nb);
        launches += 2 + launch_scan(a.radix_hist, a.radix_hist, nb * (mask + 1u), a.scan_temp, a.sort_total_dev,
                                    a.debug, s);
        k_radix_scatter<<<nb, kRadixThreads, 0, s>>>(a.keys, a.vals, n, a.total_dev, shift, mask, a.radix_hist, nb,
                                                     a.keys_alt, a.vals_alt);
        uint32_t *tk = a.keys, *tv = a.vals;
        a.keys = a.keys_alt;
        a.vals = a.vals_alt;
        a.keys_alt = tk;
        a.vals_alt = tv;
    }
    return launches;
}

}  // namespace mtgl
