// k_tile.cuh — K4 tile raster/ROP (replaces rasterize_triangle_smooth's pixel loop,
// raster.c:532-724, and glClear's loops, gl_api.c:409-457).
//
// A CTA owns one tile (8, 16 or 32 pixels square) at a time; thread t owns one pixel for
// the whole pass, so the pixel's colour, depth and stencil stay in registers between
// triangles. Each warp covers an 8x4 block of the tile and walks the tile's record list
// (submission order, built by the binning pass) on its own, 32 records per step, taking
// those whose exact edge test can pass in its block. Every thread runs the reference's
// fragment pipeline for its own pixel: edge functions at the integer pixel position,
// barycentrics, stencil test/ops, depth test, colour (flat / smooth / per-fragment
// lighting), texture with alpha test and texenv, fog, depth write, blend, masked write. Because a pixel is only ever touched by its own thread,
// in-order blending and stencil updates need no atomics. Clears of the pass are applied
// first; a clear that covers the whole tile means that buffer is never read from memory.
//
// The launch is persistent: CTAs take tiles from a work queue (an atomic head over the
// global tile ids, in frame order or, when the pass asks for it, costliest first) until it
// is empty, so frames of very different sizes share one launch without idle SMs at its end.
#pragma once

#include <algorithm>

#include "dev_kernels.h"

namespace mtgl {

constexpr int kChunk = 32;  // records tested per step: one per lane for the overlap ballot

__device__ __forceinline__ bool covers_tile(const ClearOp &c, uint32_t bit, int x0, int y0, int x1, int y1)
{
    return (c.mask & bit) && c.x0 <= x0 && c.y0 <= y0 && c.x1 >= x1 && c.y1 >= y1;
}

// Float order as signed-int order (negative floats reversed), so a warp max is one REDUX.
__device__ __forceinline__ int ordered_key(float f)
{
    const int b = __float_as_int(f);
    return b ^ ((b >> 31) & 0x7FFFFFFF);
}
__device__ __forceinline__ float ordered_float(int k) { return __int_as_float(k ^ ((k >> 31) & 0x7FFFFFFF)); }

// Largest stored depth over the warp's pixels inside the framebuffer.
__device__ __forceinline__ float warp_max_depth(float dep, bool in_fb)
{
    return ordered_float(__reduce_max_sync(0xffffffffu, in_fb ? ordered_key(dep) : INT32_MIN));
}

constexpr uint32_t kNoPending = 0xFFFFFFFFu;

// The 8x4 warp blocks of the tile at (tx0, ty0) that a record must be walked in: bit
// r * (TS / 8) + c for the block at column c, row r. A block is set when the record's box
// (mnx..mxx, mny..mxy) meets it and, for a triangle, when its coverage test can pass there.
// The test is exact: the edge function (px - ax) * A - (py - ay) * B has integer-valued
// operands, so when every product over the tile is below 2^24 in magnitude the per-pixel
// float test has the sign of the exact integer; then each edge's largest value over a block
// (at a corner: the function is affine) is an int32 stepped per block column and row, and a
// block where it is negative for some edge holds no covered pixel (for a negative area the
// signs flip). Otherwise every block the box meets is set. bb = record words 4-7 (x2, y2,
// box min), bb2 = words 8-11 (box max, area, 1/area), q12 = words 48-51.
template <int TS>
__device__ __forceinline__ uint32_t block_mask(const float4 *q, const float4 &bb, const float4 &bb2, const float4 &q12,
                                               uint32_t flags, int tx0, int ty0, int mnx, int mny, int mxx, int mxy)
{
    constexpr int kWX = TS / 8;
    if (mxx < tx0 || mnx > tx0 + TS - 1 || mxy < ty0 || mny > ty0 + TS - 1) return 0u;
    const int c0 = max(mnx - tx0, 0) >> 3, c1 = min(mxx - tx0, TS - 1) >> 3;
    const int r0 = max(mny - ty0, 0) >> 2, r1 = min(mxy - ty0, TS - 1) >> 2;
    uint32_t box = 0u;
    for (int r = r0; r <= r1; r++)
        for (int c = c0; c <= c1; c++) box |= 1u << (r * kWX + c);
    if (((flags >> kRecTypeShift) & 3u) != REC_TRI) return box;
    const float area = bb2.z;
    if (!(area > 0.0f) && !(area < 0.0f)) return 0u;  // zero or NaN area: the test never passes
    const float4 q0 = __ldg(q + 0), q13 = __ldg(q + 13);
    const float ax[3] = {q0.z, bb.x, q0.x}, ay[3] = {q0.w, bb.y, q0.y};
    const float ea[3] = {q12.y, q12.w, q13.y}, eb[3] = {q12.z, q13.x, q13.z};
    const bool pos = area > 0.0f;
    int e00[3], sx[3], sy[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        constexpr float kLim = 16777216.0f;  // 2^24
        if (!(fabsf(ax[k]) < kLim && fabsf(ay[k]) < kLim && fabsf(ea[k]) < kLim && fabsf(eb[k]) < kLim)) return box;
        const int iax = (int)ax[k], iay = (int)ay[k];
        const int a = pos ? (int)ea[k] : -(int)ea[k], b = pos ? (int)eb[k] : -(int)eb[k];
        const long long mx = max(llabs((long long)tx0 - iax), llabs((long long)tx0 + TS - 1 - iax)) * llabs((long long)a);
        const long long my = max(llabs((long long)ty0 - iay), llabs((long long)ty0 + TS - 1 - iay)) * llabs((long long)b);
        if (mx >= (1ll << 24) || my >= (1ll << 24)) return box;
        // largest over block (0, 0) at its right column when a >= 0, its top row when b >= 0
        e00[k] = (tx0 + (a >= 0 ? 7 : 0) - iax) * a - (ty0 + (b >= 0 ? 0 : 3) - iay) * b;
        sx[k] = a * 8;
        sy[k] = b * 4;
    }
    uint32_t mask = 0u;
    for (int r = r0; r <= r1; r++)
        for (int c = c0; c <= c1; c++) {
            bool ok = true;
#pragma unroll
            for (int k = 0; k < 3; k++) ok = ok && e00[k] + c * sx[k] - r * sy[k] >= 0;
            if (ok) mask |= 1u << (r * kWX + c);
        }
    return mask;
}

// The colour stages of a fragment (raster.c:582-705): colour interpolation (or the flat
// colour), per-fragment lighting, texturing with the alpha test and texture environment,
// fog. Returns false when the alpha test discards the fragment.
template <bool TEX, bool EYE>
__device__ __forceinline__ bool frag_color(const DevRaster &R, uint32_t ctl, const float4 *r4, const float *e,
                                           bool have_eye, float b0, float b1, float b2, float4 &c)
{
    const FragState &S = R.fs;
    const float4 c2 = __ldg(r4 + 7);  // C2
    if (ctl & FC_FLAT) {
        c = c2;
    } else {
        const float4 c0 = __ldg(r4 + 5), c1 = __ldg(r4 + 6);  // C0, C1
        c = make_float4(c0.x * b0 + c1.x * b1 + c2.x * b2, c0.y * b0 + c1.y * b1 + c2.y * b2,
                        c0.z * b0 + c1.z * b1 + c2.z * b2, c0.w * b0 + c1.w * b1 + c2.w * b2);
    }
    if (EYE && have_eye) {
        const mtgl_raster_state &rs = R.rs;
        if (rs.lighting) {
            const bool back = (__float_as_uint(__ldg(reinterpret_cast<const float *>(r4) + R_FLAGS)) & 1u) != 0;
            const bool phong = rs.shade_model == GL_PHONG;
            if (phong || (back && rs.lit.two_side)) {
                float3 ep = make_float3(e[0] * b0 + e[6] * b1 + e[12] * b2, e[1] * b0 + e[7] * b1 + e[13] * b2,
                                        e[2] * b0 + e[8] * b1 + e[14] * b2);
                float3 en = make_float3(e[3] * b0 + e[9] * b1 + e[15] * b2, e[4] * b0 + e[10] * b1 + e[16] * b2,
                                        e[5] * b0 + e[11] * b1 + e[17] * b2);
                const mtgl_material *mat = &rs.lit.front;
                if (back && rs.lit.two_side) {
                    en = make_float3(en.x * -1.0f, en.y * -1.0f, en.z * -1.0f);
                    mat = &rs.lit.back;
                }
                c = compute_lighting(rs.lit, ep, en, *mat);
            }
        }
    }
    if (TEX && (ctl & FC_TEXTURE)) {
        float u, v;
        const float4 q4 = __ldg(r4 + 4);  // W0 W1 W2 LOD
        if (!(ctl & FC_AFFINE_UV)) {
            const float4 q9 = __ldg(r4 + 9), q10 = __ldg(r4 + 10);  // UV2 UW0 VW0 | UW1 VW1 UW2 VW2
            const float uow = b0 * q9.z + b1 * q10.x + b2 * q10.z;
            const float vow = b0 * q9.w + b1 * q10.y + b2 * q10.w;
            const float oow = b0 * q4.x + b1 * q4.y + b2 * q4.z;
            const float w = 1.0f / oow;
            u = uow * w;
            v = vow * w;
        } else {
            const float4 q8 = __ldg(r4 + 8), q9 = __ldg(r4 + 9);  // UV0 UV1 | UV2 ..
            u = b0 * q8.x + b1 * q8.z + b2 * q9.x;
            v = b0 * q8.y + b1 * q8.w + b2 * q9.y;
        }
        const float4 tc = unpack_rgba(sample_lod(S, u, v, q4.w));
        // the alpha test applies to textured fragments only (raster.c:639-643)
        if ((ctl & FC_ALPHA) && !cmp_pass(__ldg(&S.alpha_func), tc.w, __ldg(&S.alpha_ref))) return false;
        switch (__ldg(&S.tex_env_mode)) {
        case GL_REPLACE: c = tc; break;
        case GL_DECAL: c = lerp_rgb(c, tc, tc.w); break;
        case GL_BLEND: {
            const float4 ec = __ldg(reinterpret_cast<const float4 *>(S.tex_env_color));
            c = make_float4(c.x * (1.0f - tc.x) + ec.x * tc.x, c.y * (1.0f - tc.y) + ec.y * tc.y,
                            c.z * (1.0f - tc.z) + ec.z * tc.z, c.w * tc.w);
            break;
        }
        case GL_ADD: c = make_float4(c.x + tc.x, c.y + tc.y, c.z + tc.z, c.w * tc.w); break;
        default: c = make_float4(c.x * tc.x, c.y * tc.y, c.z * tc.z, c.w * tc.w); break;
        }
    }
    if (ctl & FC_FOG) {
        const float4 q11 = __ldg(r4 + 11);                                   // EZ0 EZ1 EZ2
        const float4 g3 = __ldg(reinterpret_cast<const float4 *>(&S) + 3);  // .z mode, .w density
        const float4 g4 = __ldg(reinterpret_cast<const float4 *>(&S) + 4);  // .x start, .y end
        const float4 fcol = __ldg(reinterpret_cast<const float4 *>(S.fog_color));
        const float fc = b0 * q11.x + b1 * q11.y + b2 * q11.z;
        c = lerp_rgb(fcol, c, fog_factor(__float_as_uint(g3.z), g3.w, g4.x, g4.y, fc));
    }
    return true;
}

// The barycentrics of the pixel in a triangle record, as the coverage test computes them.
__device__ __forceinline__ void tri_bary(const float4 *r4, float fpx, float fpy, float &b0, float &b1, float &b2)
{
    const float4 q0 = __ldg(r4 + 0), q1 = __ldg(r4 + 1), q2 = __ldg(r4 + 2), q12 = __ldg(r4 + 12),
                 q13 = __ldg(r4 + 13);
    const float e0 = (fpx - q0.z) * q12.y - (fpy - q0.w) * q12.z;
    const float e1 = (fpx - q1.x) * q12.w - (fpy - q1.y) * q13.x;
    const float e2 = (fpx - q0.x) * q13.y - (fpy - q0.y) * q13.z;
    b0 = e0 * q2.w;
    b1 = e1 * q2.w;
    b2 = e2 * q2.w;
}

// The colour a deferred fragment writes (below): its colour stages, clamped and packed (its
// raster state has no blend and writes every channel).
template <bool TEX, bool EYE>
__device__ __forceinline__ uint32_t pending_color(const TileArgs &A, uint32_t ridx, bool have_eye, float fpx,
                                                  float fpy)
{
    const float4 *r4 = reinterpret_cast<const float4 *>(A.records + (size_t)ridx * kRecWords);
    const float *e = have_eye ? A.eye_records + (size_t)ridx * kEyeWords : nullptr;
    float b0, b1, b2;
    tri_bary(r4, fpx, fpy, b0, b1, b2);
    const float4 q11 = __ldg(r4 + 11);
    const DevRaster &R = A.rasters[min(__float_as_uint(q11.w), A.nrasters - 1)];
    float4 c;
    frag_color<TEX, EYE>(R, __ldg(&R.fs.ctl), r4, e, have_eye, b0, b1, b2, c);
    c = clamp4(c);
    return pack_rgba(c.x, c.y, c.z, c.w);
}

// One fragment of rasterize_triangle_smooth's pixel loop (raster.c:534-722) for this
// thread's pixel. Returns true when it wrote the depth buffer. TEX / EYE compile the
// texturing and per-fragment lighting stages in only for passes that use them.
//
// DEFER (deferred colour): in a pass whose every record is a filled triangle whose raster
// state has no blend, writes all four colour channels or none, and cannot have a fragment
// discarded by the alpha test (untextured, or the test off), no fragment reads the stored
// colour, and each fragment that writes colour replaces it. So only the tests, stencil and
// depth writes run per fragment; the pixel keeps the record of the last fragment that
// wrote colour, and its colour stages run once, when the tile is written back. The stored
// colour comes out exactly as if every fragment had been shaded in turn.
template <bool TEX, bool EYE, bool DEFER>
__device__ __forceinline__ bool shade_pixel(const TileArgs &A, uint32_t ridx, const float *__restrict__ r,
                                            const float *__restrict__ e, bool have_eye, int px, int py, float fpx,
                                            float fpy, uint32_t &col, float &dep, uint32_t &st, uint32_t &frags,
                                            uint32_t &pend)
{
    // the record is read as 16-byte words (RecField positions noted beside each use)
    const float4 *r4 = reinterpret_cast<const float4 *>(r);
    const float4 q1 = __ldg(r4 + 1);  // X2 Y2 MINX MINY
    const float4 q2 = __ldg(r4 + 2);  // MAXX MAXY AREA INV_AREA
    if (px < __float_as_int(q1.z) || px > __float_as_int(q2.x) || py < __float_as_int(q1.w) ||
        py > __float_as_int(q2.y))
        return false;
    const float4 q0 = __ldg(r4 + 0);   // X0 Y0 X1 Y1
    const float4 q12 = __ldg(r4 + 12);  // FLAGS EA0 EB0 EA1
    const float4 q13 = __ldg(r4 + 13);  // EB1 EA2 EB2 FRAME
    // edge_function at the integer pixel position (raster.c:299-302, 534-536)
    const float e0 = (fpx - q0.z) * q12.y - (fpy - q0.w) * q12.z;
    const float e1 = (fpx - q1.x) * q12.w - (fpy - q1.y) * q13.x;
    const float e2 = (fpx - q0.x) * q13.y - (fpy - q0.y) * q13.z;
    const float area = q2.z;
    if (!((area > 0 && e0 >= 0 && e1 >= 0 && e2 >= 0) || (area < 0 && e0 <= 0 && e1 <= 0 && e2 <= 0))) return false;
    frags++;
    const float inv_area = q2.w;
    const float b0 = e0 * inv_area, b1 = e1 * inv_area, b2 = e2 * inv_area;
    const float4 q3 = __ldg(r4 + 3);    // Z0 Z1 Z2 DMIN
    // the raster state, only where a stage reads more than the record carries
    auto raster = [&]() -> const DevRaster & {
        return A.rasters[min(__float_as_uint(__ldg(r + R_RASTER)), A.nrasters - 1)];
    };
    // the fragment stages' packed state: the enables and the depth function come with the
    // record's flags; the other operands are loaded as the stages need them (from one cached
    // line, to keep few registers live)
    const uint32_t rflags = __float_as_uint(q12.x);
    const uint32_t ctl = (rflags >> kRecCtlShift) & 0xFFFu;
    const float z = b0 * q3.x + b1 * q3.y + b2 * q3.z;
    const float t = (z + 1.0f) * 0.5f;
    const float depth =
        (ctl & FC_DEFAULT_RANGE) ? t : map_depth_range(t, raster().rs.depth_near, raster().rs.depth_far);

    uint32_t sv = 0;
    if (ctl & FC_STENCIL) {
        const FragState &S = raster().fs;
        const uint4 g = __ldg(reinterpret_cast<const uint4 *>(&S) + 1);  // func, ref, mask, writemask
        sv = st;
        if (!stencil_pass(g.x, (int32_t)g.y, g.z, sv)) {
            st = stencil_write(st, stencil_apply(__ldg(&S.stencil_fail), sv, (int32_t)g.y), g.w);
            return false;
        }
    }
    if ((ctl & FC_DEPTH) && !cmp_pass(GL_NEVER + ((rflags >> kRecDepthFuncShift) & 7u), depth, dep)) {
        if (ctl & FC_STENCIL) {
            const FragState &S = raster().fs;
            st = stencil_write(st, stencil_apply(__ldg(&S.stencil_zfail), sv, __ldg(&S.stencil_ref)),
                               __ldg(&S.stencil_writemask));
        }
        return false;
    }
    if (ctl & FC_STENCIL) {
        const FragState &S = raster().fs;
        st = stencil_write(st, stencil_apply(__ldg(&S.stencil_zpass), sv, __ldg(&S.stencil_ref)),
                           __ldg(&S.stencil_writemask));
    }

    if (DEFER) {
        if (ctl & FC_MASK_ALL) pend = ridx;  // this fragment's colour replaces the pixel's
        if (ctl & FC_DEPTH_WRITE) {
            dep = depth;
            return true;
        }
        return false;
    }
    const DevRaster &R = raster();
    const FragState &S = R.fs;
    float4 c;
    if (!frag_color<TEX, EYE>(R, ctl, r4, e, have_eye, b0, b1, b2, c)) return false;
    bool wrote = false;
    if (ctl & FC_DEPTH_WRITE) {
        dep = depth;
        wrote = true;
    }
    if (ctl & FC_BLEND) c = blend(__ldg(&S.blend_src), __ldg(&S.blend_dst), c, unpack_rgba(col));
    c = clamp4(c);
    if (ctl & FC_MASK_ALL) col = pack_rgba(c.x, c.y, c.z, c.w);
    else if (!(ctl & FC_MASK_NONE)) col = masked_write(__ldg(&S.color_mask), col, c);
    return wrote;
}

// The pixel state a point or line fragment updates (no stencil: the reference's point and
// line paths never touch it).
struct PixelOut {
    uint32_t col;
    float dep;
    uint32_t flags;  // bit 0: covered (a fragment); bit 1: depth written
};

// write_line_pixel (raster.c:86-104) and the pixel loop of draw_points (raster.c:1140-1160):
// depth test, blend with the stored colour, depth write, masked colour write.
__device__ __forceinline__ PixelOut point_ops(const mtgl_raster_state &rs, float depth, float4 c, uint32_t col,
                                              float dep)
{
    PixelOut o{col, dep, 1u};
    if (rs.depth_test && !cmp_pass(rs.depth_func, depth, dep)) return o;
    if (rs.blend) c = blend(rs, c, unpack_rgba(col));
    if (rs.depth_test && rs.depth_mask) {
        o.dep = depth;
        o.flags |= 2u;
    }
    o.col = masked_write(rs, col, c);
    return o;
}

// One pixel of a point or line record (the record's bbox already holds the framebuffer and
// scissor limits). Lines: the Bresenham step reaching this pixel in closed form. For an
// x-major line (|dx| > |dy|) step k sits at x0 + sx*k, y0 + sy*floor((2|dy|k + |dx| - 1) /
// (2|dx|)); for a y-major one the roles swap; each step writes a run of `lw` pixels across
// the major axis. That reproduces draw_line_full's loop exactly (tests/test_arith.py checks
// it against the loop over every |dx|, |dy| <= 130), so each pixel gets the t, colour, depth,
// texel and fog of the step that writes it.
static __device__ __noinline__ PixelOut shade_prim(const TileArgs &A, const float *r, int px, int py, uint32_t col, float dep)
{
    PixelOut none{col, dep, 0u};
    if (px < __float_as_int(r[R_MINX]) || px > __float_as_int(r[R_MAXX]) || py < __float_as_int(r[R_MINY]) ||
        py > __float_as_int(r[R_MAXY]))
        return none;
    const DevRaster &R = A.rasters[min(__float_as_uint(r[R_RASTER]), A.nrasters - 1)];
    const mtgl_raster_state &rs = R.rs;
    if (rec_type(r) == REC_POINT)
        return point_ops(rs, r[R_Z0], make_float4(r[R_C0], r[R_C0 + 1], r[R_C0 + 2], r[R_C0 + 3]), col, dep);

    const int64_t x0 = __float_as_int(r[R_X0]), y0 = __float_as_int(r[R_Y0]);
    const int64_t x1 = __float_as_int(r[R_X1]), y1 = __float_as_int(r[R_Y1]);
    const int64_t lw = __float_as_int(r[R_X2]), half = lw / 2;
    const int64_t dx = x1 - x0, dy = y1 - y0;
    const int64_t adx = dx < 0 ? -dx : dx, ady = dy < 0 ? -dy : dy;
    const int64_t sx = dx < 0 ? -1 : 1, sy = dy < 0 ? -1 : 1;
    int64_t k, across;
    if (adx > ady) {
        k = ((int64_t)px - x0) * sx;
        if (k < 0 || k > adx) return none;
        across = (int64_t)py - (y0 + sy * ((2 * ady * k + adx - 1) / (2 * adx)));
    } else if (ady > 0) {
        k = ((int64_t)py - y0) * sy;
        if (k < 0 || k > ady) return none;
        across = (int64_t)px - (x0 + sx * ((2 * adx * k + ady - 1) / (2 * ady)));
    } else {
        if (py != y0) return none;
        k = 0;
        across = (int64_t)px - x0;
    }
    if (across < -half || across >= lw - half) return none;
    const int32_t total = (int32_t)(adx > ady ? adx : ady);
    const float t = (float)(int32_t)k / (float)(total == 0 ? 1 : total);
    const float z = r[R_Z0] + t * (r[R_Z1] - r[R_Z0]);
    const float depth = map_depth(R, z);
    float4 c = lerp_col(make_float4(r[R_C0], r[R_C0 + 1], r[R_C0 + 2], r[R_C0 + 3]),
                        make_float4(r[R_C1], r[R_C1 + 1], r[R_C1 + 2], r[R_C1 + 3]), t);
    if (R.tex) {
        const float u = r[R_UV0] + t * (r[R_UV1] - r[R_UV0]);
        const float v = r[R_UV0 + 1] + t * (r[R_UV1 + 1] - r[R_UV0 + 1]);
        const float4 tc = unpack_rgba(sample_lod(R.fs, u, v, 0.0f));
        // the reference never leaves its loop when this test fails (raster.c:175, 183 skip the
        // Bresenham step); here the pixel is dropped
        if (rs.alpha_test && !cmp_pass(rs.alpha_func, tc.w, rs.alpha_ref)) return none;
        c = make_float4(c.x * tc.x, c.y * tc.y, c.z * tc.z, c.w * tc.w);
    } else if (rs.alpha_test && !cmp_pass(rs.alpha_func, c.w, rs.alpha_ref)) {
        return none;
    }
    if (rs.fog) c = lerp_rgb(ld4(rs.fog_color), c, fog_factor(rs, -(r[R_EZ0] + t * (r[R_EZ1] - r[R_EZ0]))));
    return point_ops(rs, depth, c, col, dep);
}

// One covered fragment of record `ridx` for this thread's pixel, whatever the record draws.
template <bool TEX, bool EYE, bool DEFER>
__device__ __forceinline__ bool shade_any(const TileArgs &A, uint32_t ridx, uint32_t rflags, bool have_eye, int px,
                                          int py, float fpx, float fpy, uint32_t &col, float &dep, uint32_t &st,
                                          uint32_t &frags, uint32_t &pend)
{
    const float *r = A.records + (size_t)ridx * kRecWords;
    if (DEFER || ((rflags >> kRecTypeShift) & 3u) == REC_TRI) {  // deferred passes hold triangles only
        const float *e = have_eye ? A.eye_records + (size_t)ridx * kEyeWords : nullptr;
        return shade_pixel<TEX, EYE, DEFER>(A, ridx, r, e, have_eye, px, py, fpx, fpy, col, dep, st, frags, pend);
    }
    const PixelOut po = shade_prim(A, r, px, py, col, dep);
    col = po.col;
    dep = po.dep;
    frags += po.flags & 1u;
    return (po.flags & 2u) != 0;
}

// Without per-fragment lighting the kernel fits 48 registers: ask for 1280 resident
// threads per SM (5 CTAs of 16x16, 20 of 8x8); with it, 64 registers and 1024 threads. A
// 32x32 CTA is 1024 threads on its own.
template <int TS, bool EYE>
constexpr int tile_min_blocks()
{
    return TS == 32 ? 1 : (EYE ? 1024 : 1280) / (TS * TS);
}

// ROUNDS selects how a warp runs the fragments of its records, both in submission order per
// pixel (the tile order puts tiles of small records in the first part of the work list):
// - per record (ROUNDS false): the warp steps through the records meeting its 8x4 block,
//   each covered lane runs the fragment pipeline, and the depth rejection is retried with
//   the warp's max depth as it falls;
// - by rounds (ROUNDS true, small records): every lane first finds the records covering
//   its pixel (broadcast reads), then takes its next covering record per round, so the
//   fragment pipeline runs with most lanes busy; rounds = the deepest coverage among the
//   warp's pixels, instead of the number of records meeting the block.
template <int TS, bool TEX, bool EYE, bool ROUNDS, bool DEFER>
__global__ void __launch_bounds__(TS *TS, tile_min_blocks<TS, EYE>()) k_tile(TileArgs A)
{
    constexpr int kWarpsX = TS / 8;  // 8x4-pixel warp blocks per tile row band
    constexpr uint32_t kNoTile = 0xFFFFFFFFu, kSkipTile = 0xFFFFFFFEu;
    __shared__ uint32_t s_tile, s_frame;

    if (A.guard && (A.guard[0] > A.records_cap || A.guard[1] > A.pairs_cap)) return;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ox = (warp % kWarpsX) * 8, oy = (warp / kWarpsX) * 4;  // warp block within the tile
    const bool have_eye = EYE && A.eye_records != nullptr;
    uint32_t frags = 0;

    uint32_t next_it = 0;  // thread 0: the work item claimed for the CTA's next tile
    for (bool first = true;; first = false) {
        if (!A.ctas && !first) break;  // one tile per CTA
        // Thread 0 takes the next work item and resolves its tile and frame; two barriers per
        // tile (the previous tile is done; the new one is published). Persistent CTAs claim
        // each item one tile ahead, so the queue's atomic is not waited for between tiles.
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t it, hi;
            if (A.ctas) {
                // this launch's items: the small-record part of the list, or the rest
                const uint32_t split = A.split ? min(*A.split, A.ntiles) : (ROUNDS ? A.ntiles : 0u);
                hi = ROUNDS ? split : A.ntiles;
                const uint32_t lo = ROUNDS ? 0u : split;
                uint32_t *head = A.queue + (ROUNDS ? 0 : 1);
                it = first ? lo + atomicAdd(head, 1u) : next_it;
                if (it < hi) next_it = lo + atomicAdd(head, 1u);
            } else {
                it = blockIdx.x;
                hi = A.ntiles;
            }
            uint32_t tile = kNoTile, f = 0;
            if (it < hi) {
                tile = A.order ? A.order[it] : it;
                // unordered classified launches take the tiles of their own class, in tile order
                if (A.tile_area && tile_class(A.tile_count, A.tile_area, tile, A.tile_shift) != (ROUNDS ? 0u : 1u))
                    tile = kSkipTile;
                // the frame owning the tile: last frame whose tile_base <= tile
                if (tile != kSkipTile && A.nframes > 1 && A.tile_frame) {
                    f = A.tile_frame[tile];
                } else if (tile != kSkipTile && A.nframes > 1) {
                    uint32_t flo = 0, fhi = A.nframes - 1;
                    while (flo < fhi) {
                        const uint32_t mid = (flo + fhi + 1) >> 1;
                        if (A.frames[mid].tile_base <= tile) flo = mid;
                        else fhi = mid - 1;
                    }
                    f = flo;
                }
            }
            s_tile = tile;
            s_frame = f;
        }
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile == kNoTile) break;
        if (tile == kSkipTile) continue;
        const uint32_t f = s_frame;
        const DevFrame &F = A.frames[f];
        const uint32_t count = A.tile_count[tile];
        const ClearOp *clears = A.clears + F.clear_base;
        const int nclears = (int)F.nclears;
        if (count == 0 && nclears == 0) continue;

        const uint32_t local = tile - F.tile_base;
        const int tx = (int)(local % (uint32_t)F.dims.tiles_x), ty = (int)(local / (uint32_t)F.dims.tiles_x);
        const int wx0 = tx * TS + ox, wy0 = ty * TS + oy;
        const int px = wx0 + (lane & 7);
        const int py = wy0 + (lane >> 3);
        const bool in_fb = px < F.dims.width && py < F.dims.height;
        const size_t pix = (size_t)py * F.dims.width + px;

        // buffers a clear fully covers are never loaded
        const int bx0 = tx * TS, by0 = ty * TS;
        const int bx1 = min(bx0 + TS, F.dims.width), by1 = min(by0 + TS, F.dims.height);
        bool load_c = true, load_d = true, load_s = true;
        for (int i = 0; i < nclears; i++) {
            const ClearOp &c = clears[i];
            if (covers_tile(c, GL_COLOR_BUFFER_BIT, bx0, by0, bx1, by1)) load_c = false;
            if (covers_tile(c, GL_DEPTH_BUFFER_BIT, bx0, by0, bx1, by1)) load_d = false;
            if (covers_tile(c, GL_STENCIL_BUFFER_BIT, bx0, by0, bx1, by1)) load_s = false;
        }
        uint32_t col = 0, st = 0;
        float dep = 1.0f;
        if (in_fb) {
            if (load_c) col = F.color[pix];
            if (load_d) dep = F.depth[pix];
            if (load_s) st = F.stencil[pix];
            for (int i = 0; i < nclears; i++) {
                const ClearOp &c = clears[i];
                if (px >= c.x0 && px < c.x1 && py >= c.y0 && py < c.y1) {
                    if (c.mask & GL_COLOR_BUFFER_BIT) col = c.color;
                    if (c.mask & GL_DEPTH_BUFFER_BIT) dep = c.depth;
                    if (c.mask & GL_STENCIL_BUFFER_BIT) st = c.stencil & 0xFFu;
                }
            }
        }

        const float fpx = (float)px, fpy = (float)py;
        const uint32_t start = A.tile_start[tile];
        // hierarchical z: the warp's largest stored depth, refreshed whenever the warp writes depth
        float wzmax = warp_max_depth(dep, in_fb);
        uint32_t pend = kNoPending;  // record whose deferred colour the pixel still owes

        // The CTA first scans the tile's list once: thread t takes records t, t + CTA size, ...,
        // loads each one's box and edge words and writes the 8x4 warp blocks the triangle can
        // cover (the exact edge test per block) beside the record's entry. A record is then
        // read from memory once per CTA rather than once per warp. After one barrier each warp
        // walks the list on its own, 32 entries per step, taking those whose mask names its
        // block: no barrier between warps, which differ in how much work their blocks hold.
        const float4 *recs4 = reinterpret_cast<const float4 *>(A.records);
        if (!debug_check(A.debug, (uint64_t)start + count <= A.entries_cap, DBG_TILE_ENTRY)) continue;
        for (uint32_t i = threadIdx.x; i < count; i += TS * TS) {
            const uint32_t idx = __ldg(A.tile_vals + start + i);
            if (!debug_check(A.debug, idx < A.records_cap, DBG_TILE_RECORD)) {
                A.pair_mask[start + i] = 0u;
                continue;
            }
            const float4 *q = recs4 + (size_t)idx * (kRecWords / 4);
            const float4 bb = __ldg(q + 1), bb2 = __ldg(q + 2), q12 = __ldg(q + 12);
            A.pair_mask[start + i] = block_mask<TS>(q, bb, bb2, q12, __float_as_uint(q12.x), tx * TS, ty * TS,
                                                    __float_as_int(bb.z), __float_as_int(bb.w),
                                                    __float_as_int(bb2.x), __float_as_int(bb2.y));
        }
        __syncthreads();
        for (uint32_t base = 0; base < count; base += kChunk) {
            const int n = (int)min((uint32_t)kChunk, count - base);
            // Lane j takes entry base+j when its mask names the warp's block; the depth
            // rejection is tried with the warp's max depth as of now and the record's depth
            // bound over the block. That value is still an upper bound when record j is reached
            // unless an earlier record of the step may raise depths, so rejection is only taken
            // when none before j can. The set bits, lowest first, are this warp's records of the
            // step in submission order.
            uint32_t idx = 0, flags = 0;
            float dmin = 0.0f;
            bool take = false;
            if (lane < n) {
                idx = __ldg(A.tile_vals + start + base + lane);
                take = ((A.pair_mask[start + base + lane] >> warp) & 1u) != 0;
            }
            if (take) {
                const float4 *q = recs4 + (size_t)idx * (kRecWords / 4);
                flags = __float_as_uint(__ldg(reinterpret_cast<const float *>(q) + R_FLAGS));
                dmin = __ldg(reinterpret_cast<const float *>(q) + R_DMIN);
                const uint32_t zcl = (flags >> 1) & 3u;
                if (zcl == ZC_LESS || zcl == ZC_LEQUAL) {
                    const float4 bb = __ldg(q + 1), bb2 = __ldg(q + 2);
                    const int mnx = __float_as_int(bb.z), mny = __float_as_int(bb.w);
                    const int mxx = __float_as_int(bb2.x), mxy = __float_as_int(bb2.y);
                    dmin = fmaxf(dmin, depth_plane_bound(__ldg(q + 14), mnx, mny, max(wx0, mnx), min(wx0 + 7, mxx),
                                                         max(wy0, mny), min(wy0 + 3, mxy)));
                }
            }
            const uint32_t raise_mask = __ballot_sync(0xffffffffu, (flags & kFlagRaisesDepth) != 0);
            const uint32_t zc_l = (flags >> 1) & 3u;
            if (take && (raise_mask & ((1u << lane) - 1u)) == 0) {
                if (zc_l == ZC_NEVER || (zc_l != ZC_NONE && (dmin > wzmax || (zc_l == ZC_LESS && dmin == wzmax))))
                    take = false;
            }
            uint32_t todo = __ballot_sync(0xffffffffu, take);
            if (ROUNDS) {
                uint32_t cov = 0;
                while (todo) {
                    const int j = __ffs(todo) - 1;
                    todo &= todo - 1;
                    const uint32_t ridx = __shfl_sync(0xffffffffu, idx, j);
                    const uint32_t rflags = __shfl_sync(0xffffffffu, flags, j);
                    const float4 *q = recs4 + (size_t)ridx * (kRecWords / 4);
                    const float4 q1 = __ldg(q + 1), q2 = __ldg(q + 2);
                    bool in = !(px < __float_as_int(q1.z) || px > __float_as_int(q2.x) ||
                                py < __float_as_int(q1.w) || py > __float_as_int(q2.y));
                    if (((rflags >> kRecTypeShift) & 3u) == REC_TRI) {  // points and lines test when shaded
                        const float4 q0 = __ldg(q + 0), q12 = __ldg(q + 12), q13 = __ldg(q + 13);
                        const float e0 = (fpx - q0.z) * q12.y - (fpy - q0.w) * q12.z;
                        const float e1 = (fpx - q1.x) * q12.w - (fpy - q1.y) * q13.x;
                        const float e2 = (fpx - q0.x) * q13.y - (fpy - q0.y) * q13.z;
                        const float area = q2.z;
                        in = in && ((area > 0 && e0 >= 0 && e1 >= 0 && e2 >= 0) ||
                                    (area < 0 && e0 <= 0 && e1 <= 0 && e2 <= 0));
                    }
                    if (in) cov |= 1u << j;
                }
                while (__any_sync(0xffffffffu, cov != 0)) {
                    const int j = cov ? __ffs(cov) - 1 : 0;
                    const uint32_t ridx = __shfl_sync(0xffffffffu, idx, j);
                    const uint32_t rflags = __shfl_sync(0xffffffffu, flags, j);
                    bool wrote = false;
                    if (cov) {
                        cov &= cov - 1;
                        wrote = shade_any<TEX, EYE, DEFER>(A, ridx, rflags, have_eye, px, py, fpx, fpy, col, dep, st, frags, pend);
                    }
                    if (__any_sync(0xffffffffu, wrote)) wzmax = warp_max_depth(dep, in_fb);
                }
            } else {
                while (todo) {
                    const int j = __ffs(todo) - 1;
                    todo &= todo - 1;
                    const uint32_t ridx = __shfl_sync(0xffffffffu, idx, j);
                    const uint32_t rflags = __shfl_sync(0xffffffffu, flags, j);
                    const float rdmin = __shfl_sync(0xffffffffu, dmin, j);
                    // warp-uniform rejection: no fragment of this triangle can pass the depth test here
                    const uint32_t zc = (rflags >> 1) & 3u;
                    if (zc == ZC_NEVER || (zc != ZC_NONE && (rdmin > wzmax || (zc == ZC_LESS && rdmin == wzmax))))
                        continue;
                    const bool wrote =
                        shade_any<TEX, EYE, DEFER>(A, ridx, rflags, have_eye, px, py, fpx, fpy, col, dep, st, frags, pend);
                    if (__any_sync(0xffffffffu, wrote)) wzmax = warp_max_depth(dep, in_fb);
                }
            }
        }

        if (DEFER && pend != kNoPending) col = pending_color<TEX, EYE>(A, pend, have_eye, fpx, fpy);
        if (in_fb && debug_check(A.debug, pix < (size_t)F.dims.width * (size_t)F.dims.height, DBG_TILE_PIXEL)) {
            F.color[pix] = col;
            F.depth[pix] = dep;
            F.stencil[pix] = (uint8_t)st;
        }
    }
    if (A.fragments) {
        const uint32_t fw = __reduce_add_sync(0xffffffffu, frags);
        if (lane == 0 && fw) atomicAdd(A.fragments, (unsigned long long)fw);
    }
}

// A K4 variant's launches; DEFER variants are instantiated in k_tile_defer.cu, the others in
// k_tile.cu, so that the two halves compile in parallel.
template <int TS, bool TEX, bool EYE, bool DEFER>
struct TileVariant {
    static int occupancy()
    {
        static int occ = -1;
        if (occ < 0) {
            int n = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_tile<TS, TEX, EYE, false, DEFER>, TS * TS, 0) !=
                cudaSuccess)
                n = 1;
            occ = n > 0 ? n : 1;
        }
        return occ;
    }
    static int launch(const TileArgs &a, cudaStream_t s)
    {
        const unsigned grid = a.ctas ? (unsigned)std::min<uint32_t>((uint32_t)a.ctas, a.ntiles) : a.ntiles;
        if ((a.split || a.tile_area) && a.ctas && !DEFER) {  // small-record tiles by rounds, then the rest
            k_tile<TS, TEX, EYE, true, DEFER><<<grid, TS * TS, 0, s>>>(a);
            k_tile<TS, TEX, EYE, false, DEFER><<<grid, TS * TS, 0, s>>>(a);
            return 2;
        }
        k_tile<TS, TEX, EYE, false, DEFER><<<grid, TS * TS, 0, s>>>(a);
        return 1;
    }
};

template <int TS, bool DEFER>
int dispatch_tile(const TileArgs &a, cudaStream_t s, bool occ_only)
{
    const bool eye = a.eye_records != nullptr;
    if (a.any_texture && eye)
        return occ_only ? TileVariant<TS, true, true, DEFER>::occupancy()
                        : TileVariant<TS, true, true, DEFER>::launch(a, s);
    if (a.any_texture)
        return occ_only ? TileVariant<TS, true, false, DEFER>::occupancy()
                        : TileVariant<TS, true, false, DEFER>::launch(a, s);
    if (eye)
        return occ_only ? TileVariant<TS, false, true, DEFER>::occupancy()
                        : TileVariant<TS, false, true, DEFER>::launch(a, s);
    return occ_only ? TileVariant<TS, false, false, DEFER>::occupancy()
                    : TileVariant<TS, false, false, DEFER>::launch(a, s);
}

template <bool DEFER>
int dispatch_tile_size(const TileArgs &a, cudaStream_t s, bool occ_only)
{
    switch (a.tile_shift) {
    case 3: return dispatch_tile<8, DEFER>(a, s, occ_only);
    case 5: return dispatch_tile<32, DEFER>(a, s, occ_only);
    default: return dispatch_tile<16, DEFER>(a, s, occ_only);
    }
}

// the deferred-colour launches (k_tile_defer.cu)
int dispatch_tile_deferred(const TileArgs &a, cudaStream_t s, bool occ_only);

}  // namespace mtgl
