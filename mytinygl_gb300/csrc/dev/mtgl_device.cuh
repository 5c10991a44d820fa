// mtgl_device.cuh — device-side data layout and arithmetic of the GB300 back end.
//
// Every float expression here reproduces the reference's operation order (src/graphics.h,
// src/lighting.h, src/raster.c, src/textures.c) and the translation units are compiled
// with -fmad=false and IEEE division/square root, so each result is the value the
// reference computes on x86-64. Float->int conversions emulate x86-64 cvttss2si (NaN and
// out-of-range give INT32_MIN), which is what the reference's casts compile to.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "GL/gl.h"
#include "mytinygl/mtgl_dev.h"

namespace mtgl {

// ------------------------------------------------------------------ debug bounds checks
//
// A build with MTGL_DEBUG_BOUNDS defined (mytinygl_gb300.build(debug_bounds=True)) checks the
// index of every device-memory access the kernels compute from data (framebuffer pixels,
// triangle records, tile-list entries, tile ids, vertex slots). A failed check never traps:
// it records its site code in the context's status word (the first failure wins; read back
// through mtgl_stats.debug_status) and skips the access. In the ordinary build the checks
// compile to nothing.
enum DebugSite : uint32_t {
    DBG_TILE_PIXEL = 1,    // K4: framebuffer pixel index
    DBG_TILE_RECORD = 2,   // K4: record index from a tile list
    DBG_TILE_ENTRY = 3,    // K4: tile-list position
    DBG_BIN_TILE = 4,      // binning: tile id of a sorted pair
    DBG_VERTEX_SLOT = 5,   // K1: vertex slot
    DBG_SETUP_RECORD = 6,  // K2: record position
    // Not an index check, and recorded by every build: a scan's bounded wait for an earlier
    // tile's sum ran out (never expected; the pass's results are then wrong).
    DBG_SCAN_WAIT = 7,
};
__device__ __forceinline__ bool debug_check(uint32_t *status, bool ok, uint32_t site)
{
#ifdef MTGL_DEBUG_BOUNDS
    if (!ok && status) atomicCAS(status, 0u, site);
    return ok;
#else
    (void)status;
    (void)site;
    (void)ok;
    return true;
#endif
}

// ------------------------------------------------------------------ layout constants

constexpr int kTileShiftMin = 3;     // tile edges of 8, 16 or 32 pixels (one CTA per tile)
constexpr int kTileShiftMax = 5;
constexpr int kTileShiftPlain = 4;   // 16x16 tiles for single-frame passes
constexpr int kRecWords = 60;        // words per triangle record (240 bytes)
constexpr int kEyeWords = 20;        // words per triangle eye-space record (per-fragment lighting)

// Triangle record written by the setup kernel, read by the tile kernel (raster.c:451-529
// inputs plus the per-triangle values rasterize_triangle_smooth derives before its loop).
enum RecField {
    R_X0 = 0, R_Y0, R_X1, R_Y1, R_X2, R_Y2,   // screen vertices as floats of the int coordinates
    R_MINX = 6, R_MINY, R_MAXX, R_MAXY,       // int32 bbox after viewport/scissor/framebuffer clamps
    R_AREA = 10, R_INV_AREA,
    R_Z0 = 12, R_Z1, R_Z2,
    R_DMIN = 15,                              // lower bound of every fragment depth (hierarchical z)
    R_W0 = 16, R_W1, R_W2,                    // 1/w
    R_LOD = 19,
    R_C0 = 20, R_C1 = 24, R_C2 = 28,          // RGBA each
    R_UV0 = 32, R_UV1 = 34, R_UV2 = 36,       // raw texcoords
    R_UW0 = 38, R_VW0, R_UW1, R_VW1, R_UW2, R_VW2,
    R_EZ0 = 44, R_EZ1, R_EZ2,
    R_RASTER = 47,                            // uint32 raster-state index
    R_FLAGS = 48,                             // bit 0 back facing; bits 1-2 depth rejection mode
    R_EA0 = 49, R_EB0, R_EA1, R_EB1, R_EA2, R_EB2,  // per-edge (by-ay), (bx-ax) of edge_function
    R_FRAME = 55,                             // uint32 frame index within the pass's frame table
    // the depth plane over the box, for a per-block depth bound (depth_plane_bound):
    // z at (MINX, MINY), dz/dx, dz/dy, and the margin that makes the bound safe (+inf: none)
    R_ZP0 = 56, R_ZGX, R_ZGY, R_ZM
};

// Depth rejection modes (R_FLAGS bits 1-2). A warp skips a triangle when no fragment of it
// can pass the depth test and a failing fragment has no other effect (stencil test off):
// GL_LESS: min fragment depth >= the warp's max stored depth; GL_LEQUAL: >; GL_NEVER: always.
enum ZCull { ZC_NONE = 0, ZC_LESS = 1, ZC_LEQUAL = 2, ZC_NEVER = 3 };
// R_FLAGS bit 3: the triangle may raise stored depths (depth writes with GL_GREATER,
// GL_GEQUAL, GL_NOTEQUAL or GL_ALWAYS); a warp's max depth taken before it is then no bound.
constexpr uint32_t kFlagRaisesDepth = 8u;

// R_FLAGS bits 4-5: what the record draws. Points and lines reuse the record's words:
//   REC_POINT (draw_points / draw_point_at_screen, raster.c:777-844, 1020-1164): a square
//     R_MINX..R_MAXY (already clamped to the framebuffer and scissor) of one depth R_Z0 and
//     one final colour R_C0 (texture, alpha test and fog applied at setup);
//   REC_LINE (draw_line_full, raster.c:107-241): int endpoints R_X0,R_Y0 / R_X1,R_Y1, width
//     R_X2 (int), NDC z R_Z0/R_Z1, colours R_C0/R_C1, uv R_UV0/R_UV1, eye z R_EZ0/R_EZ1,
//     bbox R_MINX..R_MAXY over the widened line clamped to framebuffer and scissor.
enum RecType { REC_TRI = 0, REC_POINT = 1, REC_LINE = 2 };
constexpr int kRecTypeShift = 4;
// R_FLAGS of a triangle record, bits 8-19: its raster state's FragCtl enables; bits 20-22:
// its depth function - GL_NEVER. The tile kernel's tests read them with the edge
// coefficients (same 16-byte word) instead of through the raster state.
constexpr int kRecCtlShift = 8, kRecDepthFuncShift = 20;
__device__ __forceinline__ uint32_t rec_type(const float *r) { return (__float_as_uint(r[R_FLAGS]) >> kRecTypeShift) & 3u; }

// Lower bound of the depth of every fragment a triangle record can write in the rectangle
// [xl, xh] x [yl, yh] of its box (inclusive pixel positions, inside the record's box).
// The record stores a float plane p(x, y) = P0 + GX (x - MINX) + GY (y - MINY) close to the
// exact interpolation Z*(x, y) = sum z_i e_i(x, y) / area, and a margin M covering, for every
// covered pixel of the box, the roundings of the fragment's own z (b_i = e_i * inv_area,
// then the sum), of P0, GX and GY, and of this evaluation (setup_fan_tri derives it). The
// plane's minimum over the rectangle is at the corner the signs of GX and GY pick; the
// depth mapping of the default range, (z + 1) * 0.5, is monotone. With M = +inf (no plane)
// the result is -inf.
__device__ __forceinline__ float depth_plane_bound(const float4 &zp, int minx, int miny, int xl, int xh, int yl,
                                                  int yh)
{
    const float dx = (float)((zp.y >= 0.0f ? xl : xh) - minx);
    const float dy = (float)((zp.z >= 0.0f ? yl : yh) - miny);
    const float z = (zp.x + zp.y * dx) + zp.z * dy - zp.w;
    return (z + 1.0f) * 0.5f;
}

// Post-transform vertices (vertex_t, graphics.h:438-446, without the unused object normal)
// are stored as three streams of 16-byte words, one word per vertex slot each: the clip
// position, the colour, and (u, v, eye z, 0). The count pass of set-up reads only the first.
struct PostVertices {
    float4 *clip;
    float4 *color;
    float4 *uvz;
};
struct __align__(16) PostEye {
    float4 pos_nx;   // eye_pos.xyz, eye_normal.x
    float4 nyz;      // eye_normal.y, eye_normal.z
};

struct DevAttrib {
    const uint8_t *ptr;   // element `base_index` is at ptr
    int64_t base_index;
    uint64_t bytes;       // readable bytes from ptr
    int32_t size, type, stride, enabled;
};

// One draw packet as the kernels see it.
struct DevDraw {
    uint32_t mode;
    int32_t first, count;
    uint32_t index_type;
    const uint8_t *indices;
    int64_t index_min;
    int32_t range_n;       // range mode: vertices index_min .. index_min+range_n-1
    int32_t range_mode;    // 1: slots cover an index range (+1 default slot), 0: one slot per element
    int32_t pos2d;
    DevAttrib pos, color, tex, normal;
    float cur_color[4], cur_tex[2], cur_normal[3];
    const uint32_t *vs_ids;
    uint32_t vs_base;
    uint32_t raster;
    uint32_t vslot_base, vslot_count;
    uint32_t tri_base, tri_count;
};

// The fragment stages' part of a raster state, packed for the tile kernel: a word of the
// stage enables and each stage's operands in 16-byte groups, 160 bytes in all. The
// full state spans about a kilobyte (mostly lights and materials) and scatters these fields
// over several lines; per fragment the kernel now loads the first group, and further groups
// only for the stages its enables switch on.
enum FragCtl : uint32_t {
    FC_STENCIL = 1u << 0, FC_DEPTH = 1u << 1, FC_DEPTH_WRITE = 1u << 2, FC_FLAT = 1u << 3, FC_ALPHA = 1u << 4,
    FC_AFFINE_UV = 1u << 5, FC_FOG = 1u << 6, FC_BLEND = 1u << 7, FC_DEFAULT_RANGE = 1u << 8,
    FC_MASK_ALL = 1u << 9, FC_MASK_NONE = 1u << 10, FC_TEXTURE = 1u << 11
};
// A texture level beyond 1 (MTGL_OPT_MIPMAP_CHAIN): packed RGBA8 texels, row-major.
struct DevMip {
    const uint32_t *px;
    int32_t w, h;
};
struct __align__(16) FragState {
    uint32_t ctl, depth_func, alpha_func, tex_env_mode;
    uint32_t stencil_func;
    int32_t stencil_ref;
    uint32_t stencil_mask, stencil_writemask;
    uint32_t stencil_fail, stencil_zfail, stencil_zpass;
    float alpha_ref;
    uint32_t blend_src, blend_dst, fog_mode;
    float fog_density;
    float fog_start, fog_end;
    uint32_t color_mask;  // bit i: channel i written
    uint32_t pad0;
    float fog_color[4];
    float tex_env_color[4];
    const uint32_t *tex, *mip1;            // texture: levels 0 and 1 (see DevRaster)
    int32_t tex_w, tex_h, mip_w, mip_h;
    int32_t wrap_s, wrap_t, min_filter, mag_filter;
    const DevMip *chain;                   // levels 2.. (MTGL_OPT_MIPMAP_CHAIN), or null
    int32_t chain_levels, pad1;            // how many (0: the reference's two levels)
};

static_assert(sizeof(FragState) == 176 && offsetof(FragState, chain) == 160 && offsetof(FragState, stencil_func) == 16 &&
                  offsetof(FragState, stencil_fail) == 32 && offsetof(FragState, blend_src) == 48 &&
                  offsetof(FragState, fog_start) == 64 && offsetof(FragState, fog_color) == 80 &&
                  offsetof(FragState, tex_env_color) == 96 && offsetof(FragState, tex) == 112 &&
                  offsetof(FragState, tex_w) == 128 && offsetof(FragState, wrap_s) == 144,
              "FragState groups are read as 16-byte words");

// Raster state with the bound texture resolved to device pointers.
struct DevRaster {
    FragState fs;          // derived from rs and tex when the draw is queued
    mtgl_raster_state rs;
    const uint32_t *tex;   // level 0, or null when texturing is off
    const uint32_t *mip1;  // level 1, or null when the reference cannot build it (w or h < 2)
    int32_t tex_w, tex_h, mip_w, mip_h;
    const DevMip *chain;   // levels 2.. of a texture built under MTGL_OPT_MIPMAP_CHAIN
    int32_t chain_levels;
    int32_t default_depth_range;
    int32_t needs_eye;     // per-fragment lighting reads eye-space interpolants
    int32_t depth_rejection;  // MTGL_OPT_DEPTH_REJECTION of the context at enqueue
    uint32_t frame;           // index of the frame (framebuffer) the draw renders into
};

struct ClearOp {
    uint32_t mask;
    int32_t x0, y0, x1, y1;
    uint32_t color;
    float depth;
    uint32_t stencil;
};

struct FrameDims {
    int32_t width, height;
    int32_t tiles_x, tiles_y;
};

// One framebuffer of a pass. A single-context pass has one frame; a batch has one per
// context. Tiles of all frames are numbered consecutively: frame f owns global tiles
// [tile_base, tile_base + tiles_x * tiles_y). Its clears are clears[clear_base .. +nclears).
struct DevFrame {
    uint32_t *color;
    float *depth;
    uint8_t *stencil;
    FrameDims dims;
    uint32_t tile_base;
    uint32_t clear_base, nclears;
    uint32_t pad_;
};

// ------------------------------------------------------------------ scalar helpers

__device__ __forceinline__ int32_t x86_f2i(float f)
{
    return (f >= -2147483648.0f && f < 2147483648.0f) ? (int32_t)f : INT32_MIN;
}

// Exact small conversions on the FP32 adder instead of the conversion unit, which issues at
// a fraction of the FP32 rate. For 0 <= v < 2^23 the float with bits 0x4B000000 | v is
// 2^23 + v; for a float f, 2^23 + f (or 1.5 * 2^23 + f) lies in [2^23, 2^24), where floats
// are the integers, so the sum rounded toward zero (or down) is 2^23 + the integer part of
// f (or 1.5 * 2^23 + floor f), read back from the low mantissa bits.
// (float)v for 0 <= v < 2^23
__device__ __forceinline__ float small_u2f(uint32_t v) { return __int_as_float(0x4B000000 | v) - 0x1p23f; }
// (int32_t)f, truncating, for 0 <= f < 2^23
__device__ __forceinline__ int32_t small_trunc(float f) { return __float_as_int(__fadd_rz(f, 0x1p23f)) - 0x4B000000; }
// (int32_t)floorf(f), with floorf(f) in *fl, for -2^22 <= f < 2^22
__device__ __forceinline__ int32_t small_floor(float f, float *fl)
{
    const float s = __fadd_rd(f, 0x1.8p23f);
    *fl = s - 0x1.8p23f;
    return __float_as_int(s) - 0x4B400000;
}

// (float)v / 255.0f (graphics.h:350-357, textures.c:294-307) for v in [0, 255], without a
// division: the product with the rounded reciprocal, corrected once by its exact residual
// (Markstein's FMA correction). The result equals the IEEE quotient for every byte value
// (checked exhaustively with exact rational arithmetic in tests/test_arith.py).
__device__ __forceinline__ float u8f(uint32_t v)
{
    const float x = small_u2f(v);
    const float r = 0x1.010102p-8f;  // 1.0f / 255.0f rounded to float
    const float q = x * r;
    const float e = __fmaf_rn(-q, 255.0f, x);
    return __fmaf_rn(e, r, q);
}

// one channel of color_to_rgba32: the reference clamps with two compares, which pass a
// NaN through to a conversion giving INT32_MIN, whose low byte is 0; fmaxf / fminf map a NaN
// to 0 first, and every other input to the same clamped value (a -0 may come out as +0,
// which truncates to the same byte)
__device__ __forceinline__ uint32_t pack_channel(float c)
{
    return (uint32_t)small_trunc(fminf(fmaxf(c, 0.0f), 1.0f) * 255.0f) & 0xFFu;
}

// color_to_rgba32 (graphics.h:337-348)
__device__ __forceinline__ uint32_t pack_rgba(float r, float g, float b, float a)
{
    return (pack_channel(a) << 24) | (pack_channel(b) << 16) | (pack_channel(g) << 8) | pack_channel(r);
}

__device__ __forceinline__ float4 unpack_rgba(uint32_t p)
{
    return make_float4(u8f(p & 0xFFu), u8f((p >> 8) & 0xFFu), u8f((p >> 16) & 0xFFu), u8f((p >> 24) & 0xFFu));
}

__device__ __forceinline__ float clamp01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }
__device__ __forceinline__ float4 clamp4(float4 c)
{
    return make_float4(clamp01(c.x), clamp01(c.y), clamp01(c.z), clamp01(c.w));
}

// color_lerp (graphics.h:293-296): a*(1-t) + b*t
__device__ __forceinline__ float4 lerp_col(float4 a, float4 b, float t)
{
    float s = 1.0f - t;
    return make_float4(a.x * s + b.x * t, a.y * s + b.y * t, a.z * s + b.z * t, a.w * s + b.w * t);
}

// color_lerp_rgb (graphics.h:298-305): a + (b-a)*t, keeps a's alpha
__device__ __forceinline__ float4 lerp_rgb(float4 a, float4 b, float t)
{
    return make_float4(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.w);
}

__device__ __forceinline__ float3 normalize3(float x, float y, float z)
{
    float len = sqrtf(x * x + y * y + z * z);
    if (len > 0.0f) {
        float s = 1.0f / len;
        return make_float3(x * s, y * s, z * s);
    }
    return make_float3(x, y, z);
}

// mat4_mul_vec4 (graphics.h:131-138), column-major m
__device__ __forceinline__ float4 mul_m4(const float *m, float x, float y, float z, float w)
{
    return make_float4(m[0] * x + m[4] * y + m[8] * z + m[12] * w, m[1] * x + m[5] * y + m[9] * z + m[13] * w,
                       m[2] * x + m[6] * y + m[10] * z + m[14] * w, m[3] * x + m[7] * y + m[11] * z + m[15] * w);
}

__device__ __forceinline__ bool cmp_pass(uint32_t func, float a, float b)
{
    switch (func) {
    case GL_NEVER: return false;
    case GL_LESS: return a < b;
    case GL_EQUAL: return a == b;
    case GL_LEQUAL: return a <= b;
    case GL_GREATER: return a > b;
    case GL_NOTEQUAL: return a != b;
    case GL_GEQUAL: return a >= b;
    default: return true;
    }
}

// ------------------------------------------------------------------ lighting (lighting.h:53-142)

__device__ __forceinline__ float4 ld4(const float *p) { return make_float4(p[0], p[1], p[2], p[3]); }

__device__ inline float4 compute_lighting(const mtgl_lighting &L, float3 ep, float3 en, const mtgl_material &mat)
{
    // emission + ambient * global ambient, alpha from the diffuse material
    float4 r = make_float4(mat.emission[0] + mat.ambient[0] * L.model_ambient[0],
                           mat.emission[1] + mat.ambient[1] * L.model_ambient[1],
                           mat.emission[2] + mat.ambient[2] * L.model_ambient[2],
                           mat.emission[3] + mat.ambient[3] * L.model_ambient[3]);
    r.w = mat.diffuse[3];
    float3 N = en;
    if (L.normalize) N = normalize3(N.x, N.y, N.z);
    for (int i = 0; i < MTGL_MAX_LIGHTS; i++) {
        const mtgl_light &l = L.lights[i];
        if (!l.enabled) continue;
        float3 Ld;
        float att = 1.0f;
        if (l.position[3] == 0.0f) {
            Ld = make_float3(l.dir_normalized[0], l.dir_normalized[1], l.dir_normalized[2]);
        } else {
            float tx = l.position[0] - ep.x, ty = l.position[1] - ep.y, tz = l.position[2] - ep.z;
            float dist = sqrtf(tx * tx + ty * ty + tz * tz);
            if (dist < 1e-6f) dist = 1e-6f;
            float inv = 1.0f / dist;
            Ld = make_float3(tx * inv, ty * inv, tz * inv);
            float den = l.constant_attenuation + l.linear_attenuation * dist + l.quadratic_attenuation * dist * dist;
            if (den < 1e-6f) den = 1e-6f;
            att = 1.0f / den;
            if (l.spot_cutoff < 180.0f) {
                float ca = -(Ld.x * l.spot_dir_normalized[0] + Ld.y * l.spot_dir_normalized[1] +
                             Ld.z * l.spot_dir_normalized[2]);
                if (ca < l.cos_cutoff) att = 0.0f;
                else att *= powf(ca, l.spot_exponent);
            }
        }
        if (att <= 0.0f) continue;
        r.x = r.x + (mat.ambient[0] * l.ambient[0]) * att;
        r.y = r.y + (mat.ambient[1] * l.ambient[1]) * att;
        r.z = r.z + (mat.ambient[2] * l.ambient[2]) * att;
        r.w = r.w + (mat.ambient[3] * l.ambient[3]) * att;
        float ndl = N.x * Ld.x + N.y * Ld.y + N.z * Ld.z;
        if (ndl > 0.0f) {
            float k = att * ndl;
            r.x = r.x + (mat.diffuse[0] * l.diffuse[0]) * k;
            r.y = r.y + (mat.diffuse[1] * l.diffuse[1]) * k;
            r.z = r.z + (mat.diffuse[2] * l.diffuse[2]) * k;
            r.w = r.w + (mat.diffuse[3] * l.diffuse[3]) * k;
            if (mat.shininess > 0.0f) {
                float3 V = L.local_viewer ? normalize3(ep.x * -1.0f, ep.y * -1.0f, ep.z * -1.0f)
                                          : make_float3(0.0f, 0.0f, 1.0f);
                float3 Hh = normalize3(Ld.x + V.x, Ld.y + V.y, Ld.z + V.z);
                float ndh = N.x * Hh.x + N.y * Hh.y + N.z * Hh.z;
                if (ndh > 0.0f) {
                    float sp = powf(ndh, mat.shininess) * att;
                    r.x = r.x + (mat.specular[0] * l.specular[0]) * sp;
                    r.y = r.y + (mat.specular[1] * l.specular[1]) * sp;
                    r.z = r.z + (mat.specular[2] * l.specular[2]) * sp;
                    r.w = r.w + (mat.specular[3] * l.specular[3]) * sp;
                }
            }
        }
    }
    return clamp4(r);
}

// ------------------------------------------------------------------ texture sampling (textures.c:271-557)

struct TexView {
    const uint32_t *px;
    int32_t w, h;
};

// get_texel_wrapped's coordinate rule (textures.c:272-291): GL_REPEAT is ((x % n) + n) % n,
// anything else clamps to [0, n-1]. For a power-of-two n the REPEAT result is x & (n - 1)
// (the same value for every int x, negative ones included), which avoids two integer
// divisions per coordinate.
__device__ __forceinline__ int32_t wrap_coord(int32_t x, int32_t n, bool repeat)
{
    if (repeat) return (n & (n - 1)) == 0 ? (x & (n - 1)) : ((x % n) + n) % n;
    return x < 0 ? 0 : (x >= n ? n - 1 : x);
}

// wrap_coord(x + 1) from xa = wrap_coord(x): under GL_REPEAT it is (xa + 1) mod n
__device__ __forceinline__ int32_t wrap_next(int32_t xa, int32_t x, int32_t n, bool repeat)
{
    if (repeat) return xa + 1 == n ? 0 : xa + 1;
    return wrap_coord(x + 1, n, false);
}

__device__ __forceinline__ uint32_t texel_at(const TexView &t, int32_t x, int32_t y)
{
    return __ldg(t.px + (size_t)y * t.w + x);
}

__device__ __forceinline__ uint32_t sample_level(const TexView &t, int32_t ws, int32_t wt, float u, float v, bool linear)
{
    float tx = u * (float)t.w - 0.5f;
    float ty = v * (float)t.h - 0.5f;
    if (linear) {
        int32_t x0, y0;
        float fx, fy;
        if (fabsf(tx) < 0x1p22f && fabsf(ty) < 0x1p22f) {  // every in-range coordinate
            float flx, fly;
            x0 = small_floor(tx, &flx);
            y0 = small_floor(ty, &fly);
            fx = tx - flx;
            fy = ty - fly;
        } else {
            x0 = x86_f2i(floorf(tx));
            y0 = x86_f2i(floorf(ty));
            fx = tx - (float)x0;
            fy = ty - (float)y0;
        }
        const bool rs = ws == GL_REPEAT, rt = wt == GL_REPEAT;
        const int32_t xa = wrap_coord(x0, t.w, rs), xb = wrap_next(xa, x0, t.w, rs);
        const int32_t ya = wrap_coord(y0, t.h, rt), yb = wrap_next(ya, y0, t.h, rt);
        float4 c00 = unpack_rgba(texel_at(t, xa, ya));
        float4 c10 = unpack_rgba(texel_at(t, xb, ya));
        float4 c01 = unpack_rgba(texel_at(t, xa, yb));
        float4 c11 = unpack_rgba(texel_at(t, xb, yb));
        float4 top = lerp_col(c00, c10, fx);
        float4 bot = lerp_col(c01, c11, fx);
        float4 r = lerp_col(top, bot, fy);
        return pack_rgba(r.x, r.y, r.z, r.w);
    }
    const float hx = tx + 0.5f, hy = ty + 0.5f;
    int32_t x, y;
    float fl;
    if (fabsf(hx) < 0x1p22f && fabsf(hy) < 0x1p22f) {
        x = small_floor(hx, &fl);
        y = small_floor(hy, &fl);
    } else {
        x = x86_f2i(floorf(hx));
        y = x86_f2i(floorf(hy));
    }
    if (x < 0) x = 0;
    if (x >= t.w) x = t.w - 1;
    if (y < 0) y = 0;
    if (y >= t.h) y = t.h - 1;
    return __ldg(t.px + (size_t)y * t.w + x);
}

// a pointer field through the read-only path
__device__ __forceinline__ const uint32_t *ldg_ptr(const uint32_t *const *p)
{
    return reinterpret_cast<const uint32_t *>(__ldg(reinterpret_cast<const unsigned long long *>(p)));
}

__device__ __forceinline__ uint32_t sample_mip1(const FragState &S, int32_t ws, int32_t wt, float u, float v,
                                                int32_t filter)
{
    const uint32_t *mip1 = ldg_ptr(&S.mip1);
    if (!mip1) return 0xFFFFFFFFu;  // level 1 cannot be built (textures.c:317, 416-419)
    TexView m{mip1, __ldg(&S.mip_w), __ldg(&S.mip_h)};
    bool lin = filter == GL_LINEAR || filter == GL_LINEAR_MIPMAP_NEAREST || filter == GL_LINEAR_MIPMAP_LINEAR;
    return sample_level(m, ws, wt, u, v, lin);
}

// (float)x86_f2i(f): the truncated value as a float (INT32_MIN outside the int range)
__device__ __forceinline__ float trunc_f2i_f(float f)
{
    const float a = fabsf(f);
    if (!(a < 0x1p22f)) return (float)x86_f2i(f);
    const float t = __fadd_rz(a, 0x1p23f) - 0x1p23f;  // trunc |f|: +0 for |f| < 1, as (float)0 is
    return f < 0.0f ? -t : t;  // a -0 here only meets u - t, where it acts as +0
}

// Level d of a texture with a chain (0: base, 1: mip1, 2..: the chain).
__device__ __forceinline__ TexView chain_level(const FragState &S, int d)
{
    if (d == 0) return TexView{ldg_ptr(&S.tex), __ldg(&S.tex_w), __ldg(&S.tex_h)};
    if (d == 1) return TexView{ldg_ptr(&S.mip1), __ldg(&S.mip_w), __ldg(&S.mip_h)};
    const DevMip *m = reinterpret_cast<const DevMip *>(__ldg(reinterpret_cast<const unsigned long long *>(&S.chain)));
    return TexView{ldg_ptr(&m[d - 2].px), __ldg(&m[d - 2].w), __ldg(&m[d - 2].h)};
}

// The mipmap filters over a whole chain (MTGL_OPT_MIPMAP_CHAIN; no counterpart in the
// reference): levels 0 .. top, lod > 0. *_MIPMAP_NEAREST takes level floor(lod + 0.5);
// *_MIPMAP_LINEAR blends levels floor(lod) and floor(lod) + 1 by the fraction, as the
// reference blends levels 0 and 1 (lerp of the unpacked texels, repacked); from the top
// level up, that level alone.
static __device__ __noinline__ uint32_t sample_chain(const FragState &S, int32_t ws, int32_t wt, float u, float v, float lod,
                                              int32_t filter, int top)
{
    const bool lin = filter == GL_LINEAR_MIPMAP_NEAREST || filter == GL_LINEAR_MIPMAP_LINEAR;
    if (filter == GL_NEAREST_MIPMAP_NEAREST || filter == GL_LINEAR_MIPMAP_NEAREST) {
        const int d = lod >= (float)top ? top : (int)(lod + 0.5f);
        return sample_level(chain_level(S, min(d, top)), ws, wt, u, v, lin);
    }
    if (lod >= (float)top) return sample_level(chain_level(S, top), ws, wt, u, v, lin);
    const int d = (int)lod;
    const float t = lod - (float)d;
    const uint32_t c0 = sample_level(chain_level(S, d), ws, wt, u, v, lin);
    const uint32_t c1 = sample_level(chain_level(S, d + 1), ws, wt, u, v, lin);
    const float4 r = lerp_col(unpack_rgba(c0), unpack_rgba(c1), t);
    return pack_rgba(r.x, r.y, r.z, r.w);
}

// texture_sample_lod (textures.c:457-557) on the packed texture state
__device__ inline uint32_t sample_lod(const FragState &S, float u, float v, float lod)
{
    const int4 mode = __ldg(reinterpret_cast<const int4 *>(&S.wrap_s));  // wrap s, wrap t, min, mag filter
    const int32_t ws = mode.x, wt = mode.y;
    if (ws == GL_REPEAT) {
        u = u - trunc_f2i_f(u);
        if (u < 0) u += 1.0f;
    } else {
        if (u < 0.0f) u = 0.0f;
        if (u > 1.0f) u = 1.0f;
    }
    if (wt == GL_REPEAT) {
        v = v - trunc_f2i_f(v);
        if (v < 0) v += 1.0f;
    } else {
        if (v < 0.0f) v = 0.0f;
        if (v > 1.0f) v = 1.0f;
    }
    int32_t filter = (lod > 0.0f) ? mode.z : mode.w;
    if (lod > 0.0f && filter != GL_NEAREST && filter != GL_LINEAR) {
        const int chain = __ldg(&S.chain_levels);
        if (chain > 0) return sample_chain(S, ws, wt, u, v, lod, filter, 1 + chain);
    }
    if (filter == GL_NEAREST_MIPMAP_NEAREST || filter == GL_LINEAR_MIPMAP_NEAREST) {
        if (lod >= 0.5f) return sample_mip1(S, ws, wt, u, v, filter);
        filter = (filter == GL_NEAREST_MIPMAP_NEAREST) ? GL_NEAREST : GL_LINEAR;
    } else if (filter == GL_NEAREST_MIPMAP_LINEAR || filter == GL_LINEAR_MIPMAP_LINEAR) {
        // From lod 1 up the weight of level 1 is 1: lerp_col(c0, c1, 1) gives c1's channels
        // exactly (c0 * 0 + c1 * 1), and packing them gives c1 back (truncating
        // ((float)b / 255) * 255 returns b for every byte), so level 0 is not sampled.
        if (lod >= 1.0f) return sample_mip1(S, ws, wt, u, v, filter);
        if (lod > 0.0f) {
            float cl = (lod > 1.0f) ? 1.0f : lod;
            const TexView base{ldg_ptr(&S.tex), __ldg(&S.tex_w), __ldg(&S.tex_h)};
            uint32_t c0 = sample_level(base, ws, wt, u, v, filter == GL_LINEAR_MIPMAP_LINEAR);
            uint32_t c1 = sample_mip1(S, ws, wt, u, v, filter);
            float4 r = lerp_col(unpack_rgba(c0), unpack_rgba(c1), cl);
            return pack_rgba(r.x, r.y, r.z, r.w);
        }
        filter = (filter == GL_NEAREST_MIPMAP_LINEAR) ? GL_NEAREST : GL_LINEAR;
    }
    const TexView base{ldg_ptr(&S.tex), __ldg(&S.tex_w), __ldg(&S.tex_h)};
    return sample_level(base, ws, wt, u, v, filter == GL_LINEAR);
}

// ------------------------------------------------------------------ fragment helpers (raster.c:343-448, 672-705)

__device__ __forceinline__ float4 blend_factor(uint32_t f, float4 s, float4 d)
{
    switch (f) {
    case GL_ZERO: return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    case GL_ONE: return make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    case GL_SRC_COLOR: return s;
    case GL_ONE_MINUS_SRC_COLOR: return make_float4(1 - s.x, 1 - s.y, 1 - s.z, 1 - s.w);
    case GL_DST_COLOR: return d;
    case GL_ONE_MINUS_DST_COLOR: return make_float4(1 - d.x, 1 - d.y, 1 - d.z, 1 - d.w);
    case GL_SRC_ALPHA: return make_float4(s.w, s.w, s.w, s.w);
    case GL_ONE_MINUS_SRC_ALPHA: { float k = 1 - s.w; return make_float4(k, k, k, k); }
    case GL_DST_ALPHA: return make_float4(d.w, d.w, d.w, d.w);
    case GL_ONE_MINUS_DST_ALPHA: { float k = 1 - d.w; return make_float4(k, k, k, k); }
    case GL_SRC_ALPHA_SATURATE: {
        float k = (s.w < (1 - d.w)) ? s.w : (1 - d.w);
        return make_float4(k, k, k, 1.0f);
    }
    default: return make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    }
}

__device__ __forceinline__ float4 blend(uint32_t src, uint32_t dst, float4 s, float4 d)
{
    float4 sf = blend_factor(src, s, d);
    float4 df = blend_factor(dst, s, d);
    return clamp4(make_float4(s.x * sf.x + d.x * df.x, s.y * sf.y + d.y * df.y, s.z * sf.z + d.z * df.z,
                              s.w * sf.w + d.w * df.w));
}

__device__ __forceinline__ float4 blend(const mtgl_raster_state &rs, float4 s, float4 d)
{
    return blend(rs.blend_src, rs.blend_dst, s, d);
}

__device__ __forceinline__ bool stencil_pass(uint32_t func, int32_t ref, uint32_t mask, uint32_t val)
{
    int32_t mr = (int32_t)((uint32_t)ref & mask);
    int32_t mv = (int32_t)(val & mask);
    switch (func) {
    case GL_NEVER: return false;
    case GL_LESS: return mr < mv;
    case GL_EQUAL: return mr == mv;
    case GL_LEQUAL: return mr <= mv;
    case GL_GREATER: return mr > mv;
    case GL_NOTEQUAL: return mr != mv;
    case GL_GEQUAL: return mr >= mv;
    default: return true;
    }
}

__device__ __forceinline__ uint32_t stencil_apply(uint32_t op, uint32_t v, int32_t ref)
{
    switch (op) {
    case GL_KEEP: return v;
    case GL_ZERO: return 0u;
    case GL_REPLACE: return (uint32_t)ref & 0xFFu;
    case GL_INCR: return v < 255u ? v + 1u : 255u;
    case GL_INCR_WRAP: return (v + 1u) & 0xFFu;
    case GL_DECR: return v > 0u ? v - 1u : 0u;
    case GL_DECR_WRAP: return (v - 1u) & 0xFFu;
    case GL_INVERT: return (~v) & 0xFFu;
    default: return v;
    }
}

__device__ __forceinline__ uint32_t stencil_write(uint32_t old, uint32_t nv, uint32_t writemask)
{
    uint32_t m8 = writemask & 0xFFu;
    return ((old & ~m8) | (nv & m8)) & 0xFFu;
}

__device__ __forceinline__ float fog_factor(uint32_t mode, float density, float start, float end, float fog_coord)
{
    float f;
    switch (mode) {
    case GL_LINEAR:
        f = (end != start) ? (end - fog_coord) / (end - start) : 1.0f;
        break;
    case GL_EXP: f = expf(-density * fog_coord); break;
    case GL_EXP2: {
        float d = density * fog_coord;
        f = expf(-d * d);
        break;
    }
    default: f = 1.0f; break;
    }
    if (f < 0.0f) f = 0.0f;
    if (f > 1.0f) f = 1.0f;
    return f;
}

__device__ __forceinline__ float fog_factor(const mtgl_raster_state &rs, float fog_coord)
{
    return fog_factor(rs.fog_mode, rs.fog_density, rs.fog_start, rs.fog_end, fog_coord);
}

// the double-precision depth range map, out of line: inlined, its few FP64 instructions
// are issued (predicated off) for every fragment of the default range as well, and the
// FP64 pipe of this GPU is narrow
static __device__ __noinline__ float map_depth_range(float t, double near_d, double far_d)
{
    return (float)((double)t * (far_d - near_d) + near_d);
}

// depth range mapping (raster.c:548): float NDC term, double range, float result
__device__ __forceinline__ float map_depth(const DevRaster &R, float z)
{
    float t = (z + 1.0f) * 0.5f;
    if (R.default_depth_range) return t;  // (double)t * 1.0 + 0.0 rounds back to t
    return map_depth_range(t, R.rs.depth_near, R.rs.depth_far);
}

// write_pixel_masked (raster.c:20-45) on a packed destination pixel; mask bit i: channel i
__device__ __forceinline__ uint32_t masked_write(uint32_t mask, uint32_t dst, float4 c)
{
    if (mask == 15u) return pack_rgba(c.x, c.y, c.z, c.w);
    if (mask == 0u) return dst;
    float4 d = unpack_rgba(dst);
    if (mask & 1u) d.x = c.x;
    if (mask & 2u) d.y = c.y;
    if (mask & 4u) d.z = c.z;
    if (mask & 8u) d.w = c.w;
    return pack_rgba(d.x, d.y, d.z, d.w);
}

__device__ __forceinline__ uint32_t masked_write(const mtgl_raster_state &rs, uint32_t dst, float4 c)
{
    const uint32_t *m = rs.color_mask;
    return masked_write((m[0] ? 1u : 0u) | (m[1] ? 2u : 0u) | (m[2] ? 4u : 0u) | (m[3] ? 8u : 0u), dst, c);
}

}  // namespace mtgl
