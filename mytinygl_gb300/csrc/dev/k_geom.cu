// k_geom.cu — K1 vertex stage and K2 assembly / clip / cull / triangle setup.
//
// K1 runs emit_vertex (gl_api.c:263-348) for every vertex slot of the pass: one thread per
// slot, attribute fetch with the conversions of get_array_element and glColor4f
// (gl_api.c:694-723, 1758-1797). K2 runs once per input triangle in submission order:
// primitive assembly (raster.c:961-1017, 1199-1231), Sutherland-Hodgman clipping against
// N,F,L,R,B,T (clipping.h:37-126), perspective divide (raster.c:729-746), the fan loop with
// culling (raster.c:751-774, 901-958) and the per-triangle part of
// rasterize_triangle_smooth (raster.c:458-529). The count pass sizes the output; after an
// exclusive scan the emit pass writes each record at its submission-order position.
// Triangles that straddle a clip plane leave k_setup for a list, grouped by clip class
// (k_clip_sort) and clipped by k_clip: one crossed plane in registers, anything else by
// Sutherland-Hodgman in local memory; their records land at the same positions.
#include <algorithm>

#include "dev_kernels.h"

namespace mtgl {

__device__ __forceinline__ int find_base(const uint32_t *base, int n, uint32_t g)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(base + mid) <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ float ld_f32(const uint8_t *p)
{
    if ((reinterpret_cast<uintptr_t>(p) & 3u) == 0) return __ldg(reinterpret_cast<const float *>(p));
    uint32_t v = (uint32_t)__ldg(p) | ((uint32_t)__ldg(p + 1) << 8) | ((uint32_t)__ldg(p + 2) << 16) |
                 ((uint32_t)__ldg(p + 3) << 24);
    return __uint_as_float(v);
}

__device__ __forceinline__ uint32_t read_index(const uint8_t *idx, uint32_t type, uint32_t k)
{
    if (type == GL_UNSIGNED_INT) {
        const uint8_t *p = idx + 4ull * k;
        if ((reinterpret_cast<uintptr_t>(p) & 3u) == 0) return __ldg(reinterpret_cast<const uint32_t *>(p));
        return (uint32_t)__ldg(p) | ((uint32_t)__ldg(p + 1) << 8) | ((uint32_t)__ldg(p + 2) << 16) |
               ((uint32_t)__ldg(p + 3) << 24);
    }
    if (type == GL_UNSIGNED_SHORT) {
        const uint8_t *p = idx + 2ull * k;
        return (uint32_t)__ldg(p) | ((uint32_t)__ldg(p + 1) << 8);
    }
    return __ldg(idx + k);
}

// get_array_element (gl_api.c:1758-1797); reads past a buffer's end give zeros (the
// reference reads whatever memory follows, which is undefined).
template <int N>
__device__ __forceinline__ void fetch_attr(const DevAttrib &a, int64_t index, float *out)
{
    if (index < 0) {
#pragma unroll
        for (int i = 0; i < N; i++) out[i] = (i < 3) ? 0.0f : 1.0f;
        return;
    }
    const int comp = a.type == GL_FLOAT ? 4 : 1;
    const int64_t rel = index - a.base_index;
    const uint64_t need = (uint64_t)a.size * (uint64_t)comp;
    if (!a.ptr || rel < 0 || a.stride <= 0 || (uint64_t)rel * (uint64_t)a.stride + need > a.bytes) {
#pragma unroll
        for (int i = 0; i < N; i++) out[i] = (i == 3) ? 1.0f : 0.0f;
        return;
    }
    const uint8_t *p = a.ptr + (uint64_t)rel * (uint64_t)a.stride;
#pragma unroll
    for (int i = 0; i < N; i++) {
        if (i < a.size) out[i] = (a.type == GL_FLOAT) ? ld_f32(p + 4 * i) : u8f(__ldg(p + i));
        else out[i] = (i == 3) ? 1.0f : 0.0f;
    }
}

// glColor4f's sanitising (gl_api.c:711-723)
__device__ __forceinline__ float sanitize(float v, bool alpha)
{
    if (isnan(v) || isinf(v)) v = alpha ? 1.0f : 0.0f;
    return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
}

__global__ void __launch_bounds__(128) k_vertex(GeomArgs A)
{
    // The vertex state (matrices, lights, materials: about 1.4 KB) is the same for every
    // slot of a block in the common case; the block then copies it to shared memory once
    // and reads it from there instead of through L1 per vertex.
    static_assert(sizeof(mtgl_vertex_state) % 4 == 0 && alignof(mtgl_vertex_state) == 4, "copied as 32-bit words");
    __shared__ uint32_t s_vs[sizeof(mtgl_vertex_state) / 4];
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = g < A.total_slots;
    int d = 0;
    uint32_t k = 0, vsi = 0;
    int64_t src = -1;
    if (live) {
        d = find_base(A.draw_vslot_base, A.ndraws, g);
        const DevDraw &D0 = A.draws[d];
        k = g - D0.vslot_base;
        vsi = D0.vs_base;
        if (D0.range_mode) {
            src = ((int64_t)k < (int64_t)D0.range_n) ? D0.index_min + (int64_t)k : -1;
        } else {
            src = D0.index_type ? (int64_t)(int32_t)read_index(D0.indices, D0.index_type, k) : (int64_t)D0.first + k;
            if (D0.vs_ids) vsi += __ldg(D0.vs_ids + k);
        }
    }
    __shared__ uint32_t s_vsi;
    if (threadIdx.x == 0) s_vsi = vsi;
    __syncthreads();
    const bool shared_vs = __syncthreads_and(!live || vsi == s_vsi) != 0;
    if (shared_vs) {
        const uint32_t *src_vs = reinterpret_cast<const uint32_t *>(A.vstates + s_vsi);
        for (uint32_t i = threadIdx.x; i < sizeof(mtgl_vertex_state) / 4; i += blockDim.x) s_vs[i] = __ldg(src_vs + i);
        __syncthreads();
    }
    if (!live) return;
    const DevDraw &D = A.draws[d];
    const mtgl_vertex_state &V =
        shared_vs ? *reinterpret_cast<const mtgl_vertex_state *>(s_vs) : A.vstates[vsi];

    float p[4], c[4], t[2], n[3];
    fetch_attr<4>(D.pos, src, p);
    const float x = p[0], y = p[1], z = D.pos2d ? 0.0f : p[2];
    if (D.color.enabled) {
        fetch_attr<4>(D.color, src, c);
#pragma unroll
        for (int i = 0; i < 4; i++) c[i] = sanitize(c[i], i == 3);
    } else {
#pragma unroll
        for (int i = 0; i < 4; i++) c[i] = D.cur_color[i];
    }
    if (D.tex.enabled) fetch_attr<2>(D.tex, src, t);
    else { t[0] = D.cur_tex[0]; t[1] = D.cur_tex[1]; }
    if (D.normal.enabled) fetch_attr<3>(D.normal, src, n);
    else { n[0] = D.cur_normal[0]; n[1] = D.cur_normal[1]; n[2] = D.cur_normal[2]; }

    const float4 eye = mul_m4(V.modelview, x, y, z, 1.0f);
    const float4 n4 = mul_m4(V.normal_matrix, n[0], n[1], n[2], 0.0f);
    const float3 en = normalize3(n4.x, n4.y, n4.z);
    const float3 ep = make_float3(eye.x, eye.y, eye.z);
    float4 vc = make_float4(c[0], c[1], c[2], c[3]);
    if (V.lighting && !V.phong) {
        mtgl_material front = V.lit.front;
        if (V.color_material &&
            (V.color_material_face == GL_FRONT || V.color_material_face == GL_FRONT_AND_BACK)) {
            // GL_COLOR_MATERIAL: the clamped vertex colour replaces material fields (gl_api.c:285-312)
            const float cc[4] = {clamp01(c[0]), clamp01(c[1]), clamp01(c[2]), clamp01(c[3])};
            const uint32_t mode = V.color_material_mode;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                if (mode == GL_AMBIENT || mode == GL_AMBIENT_AND_DIFFUSE) front.ambient[i] = cc[i];
                if (mode == GL_DIFFUSE || mode == GL_AMBIENT_AND_DIFFUSE) front.diffuse[i] = cc[i];
                if (mode == GL_SPECULAR) front.specular[i] = cc[i];
                if (mode == GL_EMISSION) front.emission[i] = cc[i];
            }
        }
        vc = compute_lighting(V.lit, ep, en, front);
    }
    const float4 clip = mul_m4(V.projection, eye.x, eye.y, eye.z, eye.w);
    const float4 t4 = mul_m4(V.texture, t[0], t[1], 0.0f, 1.0f);
    float2 uv;
    if (t4.w != 0.0f && t4.w != 1.0f) uv = make_float2(t4.x / t4.w, t4.y / t4.w);
    else uv = make_float2(t4.x, t4.y);

    if (!debug_check(A.debug, g < A.total_slots, DBG_VERTEX_SLOT)) return;
    A.verts.clip[g] = clip;
    A.verts.color[g] = vc;
    A.verts.uvz[g] = make_float4(uv.x, uv.y, -eye.z, 0.0f);
    if (A.eyes) {
        PostEye e;
        e.pos_nx = make_float4(ep.x, ep.y, ep.z, en.x);
        e.nyz = make_float4(en.y, en.z, 0.0f, 0.0f);
        A.eyes[g] = e;
    }
}

// ------------------------------------------------------------------ K2

// A vertex through clipping: clip position, colour, uv, eye z and, only in passes that
// light per fragment, the eye position and normal (elsewhere they are the constants the
// vertex stage leaves, (0,0,0) and (0,0,1), which every lerp keeps).
template <bool EYE>
struct CVx;
template <>
struct CVx<true> {
    float4 clip;
    float4 col;
    float2 uv;
    float ez;
    float3 ep, en;
};
template <>
struct CVx<false> {
    float4 clip;
    float4 col;
    float2 uv;
    float ez;
};
__device__ __forceinline__ float3 cv_ep(const CVx<true> &v) { return v.ep; }
__device__ __forceinline__ float3 cv_en(const CVx<true> &v) { return v.en; }
__device__ __forceinline__ float3 cv_ep(const CVx<false> &) { return make_float3(0.0f, 0.0f, 0.0f); }
__device__ __forceinline__ float3 cv_en(const CVx<false> &) { return make_float3(0.0f, 0.0f, 1.0f); }

// vertex_lerp (graphics.h:465-475): colour uses a*(1-t)+b*t, the rest a+t*(b-a)
template <bool EYE>
__device__ __forceinline__ CVx<EYE> cv_lerp(const CVx<EYE> &a, const CVx<EYE> &b, float t)
{
    CVx<EYE> v;
    v.clip = make_float4(a.clip.x + t * (b.clip.x - a.clip.x), a.clip.y + t * (b.clip.y - a.clip.y),
                         a.clip.z + t * (b.clip.z - a.clip.z), a.clip.w + t * (b.clip.w - a.clip.w));
    v.col = lerp_col(a.col, b.col, t);
    v.uv = make_float2(a.uv.x + t * (b.uv.x - a.uv.x), a.uv.y + t * (b.uv.y - a.uv.y));
    v.ez = a.ez + t * (b.ez - a.ez);
    if constexpr (EYE) {
        v.ep = make_float3(a.ep.x + t * (b.ep.x - a.ep.x), a.ep.y + t * (b.ep.y - a.ep.y),
                           a.ep.z + t * (b.ep.z - a.ep.z));
        v.en = make_float3(a.en.x + t * (b.en.x - a.en.x), a.en.y + t * (b.en.y - a.en.y),
                           a.en.z + t * (b.en.z - a.en.z));
    }
    return v;
}

// A vertex through clipping when only its position matters: the count pass of a filled
// triangle's clip, where whether and how many records come out depends on positions alone.
struct ClipPos {
    float4 clip;
};
__device__ __forceinline__ ClipPos cv_lerp(const ClipPos &a, const ClipPos &b, float t)
{
    return ClipPos{make_float4(a.clip.x + t * (b.clip.x - a.clip.x), a.clip.y + t * (b.clip.y - a.clip.y),
                               a.clip.z + t * (b.clip.z - a.clip.z), a.clip.w + t * (b.clip.w - a.clip.w))};
}

__device__ __forceinline__ float plane_dist(const float4 &v, int p)
{
    switch (p) {
    case 0: return v.z + v.w;   // near
    case 1: return v.w - v.z;   // far
    case 2: return v.x + v.w;   // left
    case 3: return v.w - v.x;   // right
    case 4: return v.y + v.w;   // bottom
    default: return v.w - v.y;  // top
    }
}

template <class V>
__device__ __forceinline__ void snap_plane(V &v, int p)
{
    switch (p) {
    case 2: v.clip.x = -v.clip.w; break;
    case 3: v.clip.x = v.clip.w; break;
    case 4: v.clip.y = -v.clip.w; break;
    case 5: v.clip.y = v.clip.w; break;
    case 0: v.clip.z = -v.clip.w; break;
    default: v.clip.z = v.clip.w; break;
    }
}

// MAX_CLIP_VERTS (clipping.h:16). A planar triangle gains at most one vertex per plane, so
// nine suffice; only non-finite inputs, undefined in the reference, could ask for more, and
// those extra vertices are dropped instead of written out of bounds.
constexpr int kClipMax = 12;

// A vertex's inside mask: bit p set when it is inside plane p (plane_dist >= 0; a NaN
// distance is outside). The planes are constants here, so the six tests are plain adds.
__device__ __forceinline__ uint32_t inside_mask(const float4 &v)
{
    uint32_t m = 0;
#pragma unroll
    for (int p = 0; p < 6; p++) m |= (plane_dist(v, p) >= 0.0f ? 1u : 0u) << p;
    return m;
}
constexpr uint32_t kAllInside = 63u;

// Where clip_triangle's six passes can start. A pass over a triangle whose three vertices
// are all inside its plane copies them unchanged, in order, so passes are skipped while that
// holds; at the first plane with all three outside the pass returns an empty polygon, so the
// triangle produces nothing. Takes the vertices' inside masks; returns 0..5 (the first pass
// that must run), kClipNone (all inside: no clipping) or kClipEmpty.
constexpr int kClipNone = 6, kClipEmpty = 7;
__device__ __forceinline__ int clip_start(uint32_t ma, uint32_t mb, uint32_t mc)
{
    const uint32_t all = ma & mb & mc;
    if (all == kAllInside) return kClipNone;
    const int p = __ffs(~all) - 1;  // the first plane not all-inside
    return ((ma | mb | mc) >> p) & 1u ? p : kClipEmpty;
}

// The Sutherland-Hodgman pass of plane p over a triangle, in registers, for the common case
// of a triangle crossing one plane. Writes the pass's output polygon (3 or 4 vertices, in the
// pass's order) and returns its size; returns 0 when the general clipper must run instead:
// an intersection the pass drops (|den| <= 1e-10), or an output vertex not inside a later
// plane (a later pass would change the polygon; a pass whose vertices are all inside copies
// them unchanged, in order).
template <class V>
__device__ __forceinline__ int clip_one_plane(const V &v0, const V &v1, const V &v2, int p, V &o0, V &o1, V &o2,
                                              V &o3)
{
    const float d0 = plane_dist(v0.clip, p), d1 = plane_dist(v1.clip, p), d2 = plane_dist(v2.clip, p);
    const bool i0 = d0 >= 0.0f, i1 = d1 >= 0.0f, i2 = d2 >= 0.0f;
    // the intersection the pass puts on edge a -> b
    auto cross = [p](const V &a, const V &b, float da, float db, V &out) -> bool {
        const float den = da - db;
        if (!(fabsf(den) > 1e-10f)) return false;
        out = cv_lerp(a, b, da / den);
        snap_plane(out, p);
        return true;
    };
    bool ok;
    int n;
    if (i0 && !i1 && !i2) {         // edges 2->0, 0->1 cross: X20 v0 X01
        ok = cross(v2, v0, d2, d0, o0) && cross(v0, v1, d0, d1, o2);
        o1 = v0;
        n = 3;
    } else if (!i0 && i1 && !i2) {  // X01 v1 X12
        ok = cross(v0, v1, d0, d1, o0) && cross(v1, v2, d1, d2, o2);
        o1 = v1;
        n = 3;
    } else if (!i0 && !i1 && i2) {  // X20 X12 v2
        ok = cross(v2, v0, d2, d0, o0) && cross(v1, v2, d1, d2, o1);
        o2 = v2;
        n = 3;
    } else if (i0 && i1 && !i2) {   // X20 v0 v1 X12
        ok = cross(v2, v0, d2, d0, o0) && cross(v1, v2, d1, d2, o3);
        o1 = v0;
        o2 = v1;
        n = 4;
    } else if (!i0 && i1 && i2) {   // X20 X01 v1 v2
        ok = cross(v2, v0, d2, d0, o0) && cross(v0, v1, d0, d1, o1);
        o2 = v1;
        o3 = v2;
        n = 4;
    } else if (i0 && !i1 && i2) {   // v0 X01 X12 v2
        ok = cross(v0, v1, d0, d1, o1) && cross(v1, v2, d1, d2, o2);
        o0 = v0;
        o3 = v2;
        n = 4;
    } else {
        return 0;
    }
    if (!ok) return 0;
    uint32_t in = inside_mask(o0.clip) & inside_mask(o1.clip) & inside_mask(o2.clip);
    if (n == 4) in &= inside_mask(o3.clip);
    const uint32_t later = kAllInside & ~((2u << p) - 1u);  // the planes after p
    return (in & later) == later ? n : 0;
}

// The clip list is processed grouped by these classes, so that a warp's lanes take the same
// path: for a triangle whose vertices are all inside every plane after its first crossed
// plane p (nearly always clipped in registers), 8 * p + its in/out pattern at p; 48 + the
// same for the others. Takes the vertices' inside masks and p = clip_start(...).
__device__ __forceinline__ uint32_t clip_class(uint32_t ma, uint32_t mb, uint32_t mc, int p)
{
    const uint32_t later = ((~(ma & mb & mc) & kAllInside) >> (p + 1)) ? 48u : 0u;
    const uint32_t m = ((ma >> p) & 1u) | (((mb >> p) & 1u) << 1) | (((mc >> p) & 1u) << 2);
    return later + 8u * (uint32_t)p + m;
}

// clip_triangle (clipping.h:106-126): Sutherland-Hodgman passes from plane `first` on (the
// earlier ones copy the triangle unchanged, see clip_start); result in bufA[0..n)
template <class V>
__device__ __noinline__ int clip_triangle(V *bufA, V *bufB, int first)
{
    int n = 3;
    V *in = bufA, *out = bufB;
    for (int p = first; p < 6; p++) {
        int m = 0;
        const V *prev = &in[n - 1];
        float pd = plane_dist(prev->clip, p);
        for (int i = 0; i < n; i++) {
            const V *cur = &in[i];
            float cd = plane_dist(cur->clip, p);
            if (pd >= 0) {
                if (cd >= 0) {
                    if (m < kClipMax) out[m++] = *cur;
                } else {
                    float den = pd - cd;
                    if (fabsf(den) > 1e-10f && m < kClipMax) {
                        out[m] = cv_lerp(*prev, *cur, pd / den);
                        snap_plane(out[m], p);
                        m++;
                    }
                }
            } else if (cd >= 0) {
                float den = pd - cd;
                if (fabsf(den) > 1e-10f && m < kClipMax) {
                    out[m] = cv_lerp(*prev, *cur, pd / den);
                    snap_plane(out[m], p);
                    m++;
                }
                if (m < kClipMax) out[m++] = *cur;
            }
            prev = cur;
            pd = cd;
        }
        n = m;
        V *tmp = in;
        in = out;
        out = tmp;
        if (n == 0) return 0;
    }
    // after six passes the result is in `in`; move it to bufA if needed
    if (in != bufA)
        for (int i = 0; i < n; i++) bufA[i] = in[i];
    return n;
}

template <class V>
__device__ __forceinline__ void persp_divide(V &v)
{
    if (fabsf(v.clip.w) < 1e-6f) {
        v.clip = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        return;
    }
    float iw = 1.0f / v.clip.w;
    v.clip.x *= iw;
    v.clip.y *= iw;
    v.clip.z *= iw;
    v.clip.w = iw;
}

__device__ __forceinline__ void ndc_to_screen(const mtgl_raster_state &rs, float x, float y, int32_t &sx, int32_t &sy)
{
    sx = x86_f2i((x + 1.0f) * 0.5f * (float)rs.viewport[2] + (float)rs.viewport[0]);
    sy = x86_f2i((1.0f - y) * 0.5f * (float)rs.viewport[3] + (float)rs.viewport[1]);
}

__device__ __forceinline__ float idiff(int32_t a, int32_t b) { return (float)(int32_t)((uint32_t)a - (uint32_t)b); }

__device__ __forceinline__ bool culled(const mtgl_raster_state &rs, float sa)
{
    if (!rs.cull_face) return false;
    bool front = (rs.front_face == GL_CCW) ? (sa < 0) : (sa > 0);
    if (rs.cull_face_mode == GL_FRONT) return front;
    if (rs.cull_face_mode == GL_BACK) return !front;
    return true;
}

__device__ __forceinline__ void element_triple(uint32_t mode, uint32_t k, uint32_t &a, uint32_t &b, uint32_t &c)
{
    switch (mode) {
    case GL_TRIANGLE_STRIP:
        if (k % 2 == 0) { a = k; b = k + 1; c = k + 2; }
        else { a = k + 1; b = k; c = k + 2; }
        break;
    case GL_TRIANGLE_FAN:
    case GL_POLYGON:
        a = 0; b = k + 1; c = k + 2;
        break;
    case GL_QUADS: {
        uint32_t q = 4 * (k / 2);
        if (k % 2 == 0) { a = q; b = q + 1; c = q + 2; }
        else { a = q; b = q + 2; c = q + 3; }
        break;
    }
    case GL_QUAD_STRIP: {
        uint32_t i = 2 * (k / 2);
        if (k % 2 == 0) { a = i; b = i + 1; c = i + 3; }
        else { a = i; b = i + 3; c = i + 2; }
        break;
    }
    default:
        a = 3 * k; b = 3 * k + 1; c = 3 * k + 2;
        break;
    }
}

__device__ __forceinline__ uint32_t element_slot(const DevDraw &D, uint32_t e)
{
    if (!D.range_mode) return D.vslot_base + e;
    const int32_t idx = (int32_t)read_index(D.indices, D.index_type, e);
    const int64_t rel = (int64_t)idx - D.index_min;
    // negative indices read the default attributes (gl_api.c:1766); the range check only
    // guards against an index range that does not describe the indices
    if (idx < 0 || rel < 0 || rel >= (int64_t)D.range_n) return D.vslot_base + (uint32_t)D.range_n;
    return D.vslot_base + (uint32_t)rel;
}

template <bool EYE>
__device__ __forceinline__ void load_cv(const GeomArgs &A, uint32_t slot, CVx<EYE> &v)
{
    v.clip = A.verts.clip[slot];
    v.col = A.verts.color[slot];
    const float4 uvz = A.verts.uvz[slot];
    v.uv = make_float2(uvz.x, uvz.y);
    v.ez = uvz.z;
    if constexpr (EYE) {
        const PostEye e = A.eyes[slot];
        v.ep = make_float3(e.pos_nx.x, e.pos_nx.y, e.pos_nx.z);
        v.en = make_float3(e.pos_nx.w, e.nyz.x, e.nyz.y);
    }
}

// Which depth rejection the tile kernel may apply to this triangle (ZCull). Only when the
// stencil test is off (a depth-failed fragment then changes nothing), the depth function is
// GL_LESS / GL_LEQUAL / GL_NEVER, the vertex depths are finite, and the triangle is small
// enough that every edge-function value is an exact float integer (span_x * span_y < 2^23),
// which the depth bound below relies on.
__device__ __forceinline__ uint32_t depth_rejection(const DevRaster &R, float z0, float z1, float z2, float fx0,
                                                   float fy0, float fx1, float fy1, float fx2, float fy2)
{
    const mtgl_raster_state &rs = R.rs;
    if (!R.depth_rejection || !rs.depth_test || rs.stencil_test) return ZC_NONE;
    if (rs.depth_func == GL_NEVER) return ZC_NEVER;
    if (rs.depth_func != GL_LESS && rs.depth_func != GL_LEQUAL) return ZC_NONE;
    if (!isfinite(z0) || !isfinite(z1) || !isfinite(z2)) return ZC_NONE;
    // The spans are differences of integer-valued floats, exact in float below 2^24; their
    // product is taken exactly in 64-bit integers (no FP64: this GPU's FP64 pipe is narrow).
    const float sx = fmaxf(fmaxf(fx0, fx1), fx2) - fminf(fminf(fx0, fx1), fx2);
    const float sy = fmaxf(fmaxf(fy0, fy1), fy2) - fminf(fminf(fy0, fy1), fy2);
    bool small;
    if (sx == 0.0f || sy == 0.0f) small = true;
    else if (sx < 0x1p23f && sy < 0x1p23f) small = (uint64_t)small_trunc(sx) * (uint64_t)small_trunc(sy) < (1ull << 23);
    else small = false;
    if (!small) return ZC_NONE;
    return rs.depth_func == GL_LESS ? ZC_LESS : ZC_LEQUAL;
}

// Lower bound of every fragment depth of the triangle. For a covered pixel the tile kernel
// computes b_i = e_i * inv_area >= 0 from exact edge values, so the weights e_i / area sum to
// one and z = b0*z0 + b1*z1 + b2*z2 differs from that convex combination by at most
// 5 * 2^-24 * max|z_i| (two roundings in b_i, three in the sum). The margin 2^-18 * max|z_i|
// covers that and the rounding of the subtraction; the depth mapping is monotone.
__device__ __forceinline__ float depth_lower_bound(const DevRaster &R, float z0, float z1, float z2)
{
    const float zmin = fminf(fminf(z0, z1), z2), zmax = fmaxf(fmaxf(z0, z1), z2);
    const float zabs = fmaxf(fmaxf(fabsf(z0), fabsf(z1)), fabsf(z2));
    const float margin = zabs * 0x1p-18f + 1e-37f;
    const float dlo = map_depth(R, zmin - margin), dhi = map_depth(R, zmax + margin);
    return fminf(dlo, dhi);
}

// The depth plane of a triangle record (R_ZP0..R_ZM, read by depth_plane_bound). Only for
// records whose edge values are exact integers over the box (depth_rejection's condition)
// and finite vertex depths. With u = 2^-24, S0 = sum |b_i z_i| at (minX, minY), SX = sum
// |z_i EA_i| / |area|, SY = sum |z_i EB_i| / |area|, W, H the box's extents and Z = max |z_i|,
// the errors are at most: a covered fragment's z below Z* by 5u Z (b_i >= 0 sum to one);
// P0 from Z*(minX, minY) by 5u S0 (the fragment formula at that point); GX, GY from the
// exact slopes by 5u SX, 5u SY, so the plane by 5u (SX W + SY H) over the box; the
// evaluation by 4u (S0 + SX W + SY H) and the subtraction by u of the result. M takes
// 16u times the sum, nearly twice what these need, which also absorbs the roundings of M.
// tests/test_arith.py checks the bound against every covered pixel of random triangles.
__device__ __forceinline__ float4 depth_plane(float z0, float z1, float z2, float fx0, float fy0, float fx1, float fy1,
                                              float fx2, float fy2, float area, float inv_area, int32_t minX,
                                              int32_t minY, int32_t maxX, int32_t maxY)
{
    const float ea0 = fy2 - fy1, eb0 = fx2 - fx1, ea1 = fy0 - fy2, eb1 = fx0 - fx2, ea2 = fy1 - fy0, eb2 = fx1 - fx0;
    const float px = (float)minX, py = (float)minY;
    // the fragment formula at (minX, minY) (edge values exact integers there)
    const float e0 = (px - fx1) * ea0 - (py - fy1) * eb0;
    const float e1 = (px - fx2) * ea1 - (py - fy2) * eb1;
    const float e2 = (px - fx0) * ea2 - (py - fy0) * eb2;
    const float b0 = e0 * inv_area, b1 = e1 * inv_area, b2 = e2 * inv_area;
    const float p0 = b0 * z0 + b1 * z1 + b2 * z2;
    const float gx = (z0 * ea0 + z1 * ea1 + z2 * ea2) / area;
    const float gy = -((z0 * eb0 + z1 * eb1 + z2 * eb2) / area);
    const float aa = fabsf(area);
    const float s0 = fabsf(b0 * z0) + fabsf(b1 * z1) + fabsf(b2 * z2);
    const float sx = (fabsf(z0 * ea0) + fabsf(z1 * ea1) + fabsf(z2 * ea2)) / aa;
    const float sy = (fabsf(z0 * eb0) + fabsf(z1 * eb1) + fabsf(z2 * eb2)) / aa;
    const float zabs = fmaxf(fmaxf(fabsf(z0), fabsf(z1)), fabsf(z2));
    const float m = 0x1p-20f * (s0 + sx * (float)(maxX - minX) + sy * (float)(maxY - minY) + zabs) + 1e-37f;
    if (!isfinite(p0) || !isfinite(gx) || !isfinite(gy) || !isfinite(m)) return make_float4(0.0f, 0.0f, 0.0f, INFINITY);
    return make_float4(p0, gx, gy, m);
}

// ------------------------------------------------------------------ points and lines

// Depth writes with a function that can raise stored depths (the tile kernel's depth
// rejection must not trust a bound taken before such a record).
__device__ __forceinline__ bool raises_depth(const mtgl_raster_state &rs)
{
    return rs.depth_test && rs.depth_mask &&
           (rs.depth_func == GL_GREATER || rs.depth_func == GL_GEQUAL || rs.depth_func == GL_NOTEQUAL ||
            rs.depth_func == GL_ALWAYS);
}

// Clamps [x0,x1]x[y0,y1] to the framebuffer and, when enabled, the scissor box: the pixels
// write_line_pixel / draw_points would touch (raster.c per-pixel bounds and scissor checks).
__device__ __forceinline__ bool clamp_box(const mtgl_raster_state &rs, const FrameDims &dims, int64_t &x0, int64_t &y0,
                                          int64_t &x1, int64_t &y1)
{
    x0 = x0 < 0 ? 0 : x0;
    y0 = y0 < 0 ? 0 : y0;
    x1 = x1 > dims.width - 1 ? dims.width - 1 : x1;
    y1 = y1 > dims.height - 1 ? dims.height - 1 : y1;
    if (rs.scissor_test) {
        const int64_t sx0 = rs.scissor[0], sy0 = rs.scissor[1];
        const int64_t sx1 = sx0 + rs.scissor[2] - 1, sy1 = sy0 + rs.scissor[3] - 1;
        x0 = x0 < sx0 ? sx0 : x0;
        y0 = y0 < sy0 ? sy0 : y0;
        x1 = x1 > sx1 ? sx1 : x1;
        y1 = y1 > sy1 ? sy1 : y1;
    }
    return x0 <= x1 && y0 <= y1;
}

__device__ __forceinline__ void rec_header(float4 *r4, int64_t x0, int64_t y0, int64_t x1, int64_t y1,
                                           uint32_t raster_id, uint32_t frame, uint32_t flags)
{
    r4[1].z = __int_as_float((int32_t)x0);
    r4[1].w = __int_as_float((int32_t)y0);
    r4[2].x = __int_as_float((int32_t)x1);
    r4[2].y = __int_as_float((int32_t)y1);
    r4[11].w = __uint_as_float(raster_id);
    r4[12] = make_float4(__uint_as_float(flags), 0.0f, 0.0f, 0.0f);
    r4[13].w = __uint_as_float(frame);
    r4[3].w = 0.0f;  // no depth-rejection bound
}

// One point square of final colour c and depth `depth` (the caller applied texture, alpha
// test and fog). Returns the records produced (0 or 1).
__device__ __forceinline__ uint32_t point_rec(const mtgl_raster_state &rs, uint32_t raster_id, uint32_t frame,
                                              const FrameDims &dims, int64_t x0, int64_t y0, int64_t x1, int64_t y1,
                                              float depth, float4 c, float *rec)
{
    if (!clamp_box(rs, dims, x0, y0, x1, y1)) return 0;
    if (rec) {
        float4 *r4 = reinterpret_cast<float4 *>(rec);
        rec_header(r4, x0, y0, x1, y1, raster_id, frame,
                   ((uint32_t)REC_POINT << kRecTypeShift) | (raises_depth(rs) ? kFlagRaisesDepth : 0u));
        rec[R_Z0] = depth;
        r4[5] = c;
    }
    return 1;
}

// draw_point_at_screen (raster.c:777-844): a polygon-mode vertex, one pixel, vertex colour,
// alpha test on the colour, fog from -eye_z.
__device__ __forceinline__ uint32_t screen_point(const DevRaster &R, uint32_t raster_id, uint32_t frame,
                                                 const FrameDims &dims, int32_t x, int32_t y, float z, float4 c,
                                                 float ez, float *rec)
{
    const mtgl_raster_state &rs = R.rs;
    if (x < 0 || x >= dims.width || y < 0 || y >= dims.height) return 0;
    const float depth = map_depth(R, z);
    if (rs.alpha_test && !cmp_pass(rs.alpha_func, c.w, rs.alpha_ref)) return 0;
    if (rs.fog) c = lerp_rgb(ld4(rs.fog_color), c, fog_factor(rs, -ez));
    return point_rec(rs, raster_id, frame, dims, x, y, x, y, depth, c, rec);
}

// flush_points' per-vertex part (raster.c:1020-1164): clip-volume test, divide, screen
// position, texture at lod 0 with the alpha test on its alpha (else on the colour), fog,
// and the point_size square.
template <class V>
__device__ __forceinline__ uint32_t vertex_point(const DevRaster &R, uint32_t raster_id, uint32_t frame,
                                                 const FrameDims &dims, const V &v, float *rec)
{
    const mtgl_raster_state &rs = R.rs;
    const float4 p = v.clip;
    if (p.x < -p.w || p.x > p.w || p.y < -p.w || p.y > p.w || p.z < -p.w || p.z > p.w || p.w <= 0.0f) return 0;
    const float nx = p.x / p.w, ny = p.y / p.w, nz = p.z / p.w;
    int32_t cx, cy;
    ndc_to_screen(rs, nx, ny, cx, cy);
    const float depth = map_depth(R, nz);
    float4 c = v.col;
    if (R.tex) {
        const float4 tc = unpack_rgba(sample_lod(R.fs, v.uv.x, v.uv.y, 0.0f));
        if (rs.alpha_test && !cmp_pass(rs.alpha_func, tc.w, rs.alpha_ref)) return 0;
        c = make_float4(c.x * tc.x, c.y * tc.y, c.z * tc.z, c.w * tc.w);
    } else if (rs.alpha_test && !cmp_pass(rs.alpha_func, c.w, rs.alpha_ref)) {
        return 0;
    }
    if (rs.fog) c = lerp_rgb(ld4(rs.fog_color), c, fog_factor(rs, -v.ez));
    int32_t ps = x86_f2i(rs.point_size + 0.5f);
    if (ps < 1) ps = 1;
    const int64_t xs = (int64_t)cx - ps / 2, ys = (int64_t)cy - ps / 2;
    return point_rec(rs, raster_id, frame, dims, xs, ys, xs + ps - 1, ys + ps - 1, depth, c, rec);
}

// draw_line_full's setup (raster.c:107-241): endpoints, width and the interpolants; the tile
// kernel finds each pixel's Bresenham step in closed form.
__device__ __forceinline__ uint32_t line_rec(const DevRaster &R, uint32_t raster_id, uint32_t frame,
                                             const FrameDims &dims, int32_t x0, int32_t y0, float z0, int32_t x1,
                                             int32_t y1, float z1, float4 c0, float4 c1, float ez0, float ez1,
                                             float2 uv0, float2 uv1, float *rec)
{
    const mtgl_raster_state &rs = R.rs;
    int32_t lw = x86_f2i(rs.line_width + 0.5f);
    if (lw < 1) lw = 1;
    const int32_t half = lw / 2;
    const int64_t adx = llabs((int64_t)x1 - x0), ady = llabs((int64_t)y1 - y0);
    int64_t bx0 = x0 < x1 ? x0 : x1, bx1 = x0 < x1 ? x1 : x0;
    int64_t by0 = y0 < y1 ? y0 : y1, by1 = y0 < y1 ? y1 : y0;
    if (adx > ady) {  // x-major: each step writes a vertical run of lw pixels
        by0 -= half;
        by1 += lw - half - 1;
    } else {          // y-major (and a single point): horizontal runs
        bx0 -= half;
        bx1 += lw - half - 1;
    }
    if (!clamp_box(rs, dims, bx0, by0, bx1, by1)) return 0;
    if (rec) {
        float4 *r4 = reinterpret_cast<float4 *>(rec);
        rec_header(r4, bx0, by0, bx1, by1, raster_id, frame,
                   ((uint32_t)REC_LINE << kRecTypeShift) | (raises_depth(rs) ? kFlagRaisesDepth : 0u));
        r4[0] = make_float4(__int_as_float(x0), __int_as_float(y0), __int_as_float(x1), __int_as_float(y1));
        r4[1].x = __int_as_float(lw);
        rec[R_Z0] = z0;
        rec[R_Z1] = z1;
        r4[5] = c0;
        r4[6] = c1;
        r4[8] = make_float4(uv0.x, uv0.y, uv1.x, uv1.y);
        rec[R_EZ0] = ez0;
        rec[R_EZ1] = ez1;
    }
    return 1;
}

// clip_line (clipping.h:138-229): Cohen-Sutherland against the six planes, outside
// endpoint first, snapping the new endpoint onto the plane. The reference's loop has no
// bound; 32 rounds are far more than finite inputs take (each round moves one endpoint
// onto a plane it was outside of).
__device__ __forceinline__ int outcode(const float4 &v)
{
    int c = 0;
    if (v.x < -v.w) c |= 1;
    else if (v.x > v.w) c |= 2;
    if (v.y < -v.w) c |= 4;
    else if (v.y > v.w) c |= 8;
    if (v.z < -v.w) c |= 16;
    else if (v.z > v.w) c |= 32;
    return c;
}

template <class V>
__device__ bool clip_line(V &a, V &b)
{
    int ca = outcode(a.clip), cb = outcode(b.clip);
    for (int round = 0; round < 32; round++) {
        if (!(ca | cb)) return true;
        if (ca & cb) return false;
        const int co = ca ? ca : cb;
        const float4 &p0 = a.clip, &p1 = b.clip;
        float d0, d1;
        int plane;
        if (co & 1) { d0 = p0.x + p0.w; d1 = p1.x + p1.w; plane = 2; }
        else if (co & 2) { d0 = p0.w - p0.x; d1 = p1.w - p1.x; plane = 3; }
        else if (co & 4) { d0 = p0.y + p0.w; d1 = p1.y + p1.w; plane = 4; }
        else if (co & 8) { d0 = p0.w - p0.y; d1 = p1.w - p1.y; plane = 5; }
        else if (co & 16) { d0 = p0.z + p0.w; d1 = p1.z + p1.w; plane = 0; }
        else { d0 = p0.w - p0.z; d1 = p1.w - p1.z; plane = 1; }
        const float denom = d0 - d1;
        if (fabsf(denom) < 1e-10f) return false;
        V cl = cv_lerp(a, b, d0 / denom);
        snap_plane(cl, plane);
        if (co == ca) {
            a = cl;
            ca = outcode(a.clip);
        } else {
            b = cl;
            cb = outcode(b.clip);
        }
    }
    return false;
}

// draw_line_segment (raster.c:244-285): clip, divide (|w| < 1e-6 maps to the origin), screen.
template <class V>
__device__ uint32_t segment_line(const DevRaster &R, uint32_t raster_id, uint32_t frame, const FrameDims &dims, V a,
                                 V b, float *rec)
{
    if (!clip_line(a, b)) return 0;
    float z0, z1;
    if (fabsf(a.clip.w) >= 1e-6f) {
        const float iw = 1.0f / a.clip.w;
        a.clip.x *= iw;
        a.clip.y *= iw;
        z0 = a.clip.z * iw;
    } else {
        a.clip.x = 0.0f;
        a.clip.y = 0.0f;
        z0 = 0.0f;
    }
    if (fabsf(b.clip.w) >= 1e-6f) {
        const float iw = 1.0f / b.clip.w;
        b.clip.x *= iw;
        b.clip.y *= iw;
        z1 = b.clip.z * iw;
    } else {
        b.clip.x = 0.0f;
        b.clip.y = 0.0f;
        z1 = 0.0f;
    }
    int32_t x0, y0, x1, y1;
    ndc_to_screen(R.rs, a.clip.x, a.clip.y, x0, y0);
    ndc_to_screen(R.rs, b.clip.x, b.clip.y, x1, y1);
    return line_rec(R, raster_id, frame, dims, x0, y0, z0, x1, y1, z1, a.col, b.col, a.ez, b.ez, a.uv, b.uv, rec);
}

// Where a fan triangle's records go: slot i of the primitive's output range, or nowhere
// (count pass, or past the record capacity).
struct RecOut {
    float *recs, *eyes;
    uint32_t base, cap;
    __device__ float *rec(uint32_t i) const
    {
        return (recs && base + i < cap) ? recs + (size_t)(base + i) * kRecWords : nullptr;  // beyond: dropped
    }
    __device__ float *eye(uint32_t i) const
    {
        return (eyes && base + i < cap) ? eyes + (size_t)(base + i) * kEyeWords : nullptr;
    }
};

// The part of a fan triangle's set-up that decides whether it produces a record: screen
// positions, culling, and for a filled triangle the box clamped to the viewport, scissor and
// framebuffer and the area test (rasterize_triangle_smooth's set-up, raster.c:451-529).
// Returns kTriNone (no record), kTriPolygonMode (drawn as points or lines: the caller's
// polygon-mode path; only the positions and `back` are set) or kTriFill (a record).
constexpr int kTriNone = 0, kTriPolygonMode = 1, kTriFill = 2;
struct TriBox {
    int32_t x[3], y[3];
    int32_t minX, minY, maxX, maxY;
    float area;
    bool back;
};
__device__ __forceinline__ int tri_box(const mtgl_raster_state &rs, const FrameDims &dims, const float4 &a,
                                       const float4 &b, const float4 &c, TriBox &t)
{
    ndc_to_screen(rs, a.x, a.y, t.x[0], t.y[0]);
    ndc_to_screen(rs, b.x, b.y, t.x[1], t.y[1]);
    ndc_to_screen(rs, c.x, c.y, t.x[2], t.y[2]);
    const int32_t x0 = t.x[0], y0 = t.y[0], x1 = t.x[1], y1 = t.y[1], x2 = t.x[2], y2 = t.y[2];
    const float sa = idiff(x1, x0) * idiff(y2, y0) - idiff(x2, x0) * idiff(y1, y0);
    if (culled(rs, sa)) return kTriNone;
    t.back = (rs.front_face == GL_CCW) ? (sa >= 0) : (sa < 0);
    const uint32_t pm = t.back ? rs.polygon_mode_back : rs.polygon_mode_front;
    if (pm == GL_POINT || pm == GL_LINE) return kTriPolygonMode;

    int32_t minX = x0 < x1 ? (x0 < x2 ? x0 : x2) : (x1 < x2 ? x1 : x2);
    int32_t minY = y0 < y1 ? (y0 < y2 ? y0 : y2) : (y1 < y2 ? y1 : y2);
    int32_t maxX = x0 > x1 ? (x0 > x2 ? x0 : x2) : (x1 > x2 ? x1 : x2);
    int32_t maxY = y0 > y1 ? (y0 > y2 ? y0 : y2) : (y1 > y2 ? y1 : y2);
    if (minX < rs.viewport[0]) minX = rs.viewport[0];
    if (minY < rs.viewport[1]) minY = rs.viewport[1];
    if (maxX >= rs.viewport[0] + rs.viewport[2]) maxX = rs.viewport[0] + rs.viewport[2] - 1;
    if (maxY >= rs.viewport[1] + rs.viewport[3]) maxY = rs.viewport[1] + rs.viewport[3] - 1;
    if (rs.scissor_test) {
        if (minX < rs.scissor[0]) minX = rs.scissor[0];
        if (minY < rs.scissor[1]) minY = rs.scissor[1];
        if (maxX >= rs.scissor[0] + rs.scissor[2]) maxX = rs.scissor[0] + rs.scissor[2] - 1;
        if (maxY >= rs.scissor[1] + rs.scissor[3]) maxY = rs.scissor[1] + rs.scissor[3] - 1;
    }
    if (minX > maxX || minY > maxY) return kTriNone;
    // pixels outside the framebuffer read defaults and write nothing (framebuffer.h:92-134)
    if (minX < 0) minX = 0;
    if (minY < 0) minY = 0;
    if (maxX > dims.width - 1) maxX = dims.width - 1;
    if (maxY > dims.height - 1) maxY = dims.height - 1;
    if (minX > maxX || minY > maxY) return kTriNone;

    const float fx0 = (float)x0, fy0 = (float)y0, fx1 = (float)x1, fy1 = (float)y1, fx2 = (float)x2, fy2 = (float)y2;
    t.area = (fx2 - fx0) * (fy1 - fy0) - (fy2 - fy0) * (fx1 - fx0);
    if (fabsf(t.area) < 0.5f) return kTriNone;
    t.minX = minX;
    t.minY = minY;
    t.maxX = maxX;
    t.maxY = maxY;
    return kTriFill;
}

// Per fan triangle: the setup half of rasterize_triangle_smooth. Returns true when the
// triangle produces a record; writes it when `rec` is non-null.
template <class V>
__device__ __forceinline__ uint32_t setup_fan_tri(const DevRaster &R, uint32_t raster_id, uint32_t frame,
                                                  const FrameDims &dims, const V &a, const V &b, const V &c,
                                                  const RecOut &o, uint32_t at)
{
    const mtgl_raster_state &rs = R.rs;
    TriBox tb;
    const int kind = tri_box(rs, dims, a.clip, b.clip, c.clip, tb);
    if (kind == kTriNone) return 0;
    const int32_t x0 = tb.x[0], y0 = tb.y[0], x1 = tb.x[1], y1 = tb.y[1], x2 = tb.x[2], y2 = tb.y[2];
    const bool back = tb.back;
    if (kind == kTriPolygonMode) {
        const uint32_t pm = back ? rs.polygon_mode_back : rs.polygon_mode_front;
        // render_triangle's polygon modes (raster.c:901-958): vertex colours, lit per vertex
        // under GL_PHONG (phong_vertex_colors), then three points or three edges
        float4 c0 = a.col, c1 = b.col, c2 = c.col;
        if (rs.lighting && rs.shade_model == GL_PHONG) {
            c0 = compute_lighting(rs.lit, cv_ep(a), cv_en(a), rs.lit.front);
            c1 = compute_lighting(rs.lit, cv_ep(b), cv_en(b), rs.lit.front);
            c2 = compute_lighting(rs.lit, cv_ep(c), cv_en(c), rs.lit.front);
        }
        uint32_t n = 0;
        if (pm == GL_POINT) {
            n += screen_point(R, raster_id, frame, dims, x0, y0, a.clip.z, c0, a.ez, o.rec(at + n));
            n += screen_point(R, raster_id, frame, dims, x1, y1, b.clip.z, c1, b.ez, o.rec(at + n));
            n += screen_point(R, raster_id, frame, dims, x2, y2, c.clip.z, c2, c.ez, o.rec(at + n));
        } else {
            n += line_rec(R, raster_id, frame, dims, x0, y0, a.clip.z, x1, y1, b.clip.z, c0, c1, a.ez, b.ez, a.uv, b.uv,
                          o.rec(at + n));
            n += line_rec(R, raster_id, frame, dims, x1, y1, b.clip.z, x2, y2, c.clip.z, c1, c2, b.ez, c.ez, b.uv, c.uv,
                          o.rec(at + n));
            n += line_rec(R, raster_id, frame, dims, x2, y2, c.clip.z, x0, y0, a.clip.z, c2, c0, c.ez, a.ez, c.uv, a.uv,
                          o.rec(at + n));
        }
        return n;
    }
    float *rec = o.rec(at);
    float *eyerec = o.eye(at);
    if (!rec) return 1;
    const int32_t minX = tb.minX, minY = tb.minY, maxX = tb.maxX, maxY = tb.maxY;
    const float fx0 = (float)x0, fy0 = (float)y0, fx1 = (float)x1, fy1 = (float)y1, fx2 = (float)x2, fy2 = (float)y2;
    const float area = tb.area;

    const float inv_area = 1.0f / area;
    float lod = 0.0f;
    if (R.tex) {
        const float screen_area = fabsf(area) * 0.5f;
        const float du1 = (b.uv.x - a.uv.x) * (float)R.tex_w;
        const float dv1 = (b.uv.y - a.uv.y) * (float)R.tex_h;
        const float du2 = (c.uv.x - a.uv.x) * (float)R.tex_w;
        const float dv2 = (c.uv.y - a.uv.y) * (float)R.tex_h;
        const float texel_area = fabsf(du1 * dv2 - du2 * dv1) * 0.5f;
        if (screen_area > 0.0f) {
            const float tpp = texel_area / screen_area;
            if (tpp > 0.0f) {
                lod = log2f(tpp) * 0.5f;
                if (lod < 0.0f) lod = 0.0f;
            }
        }
    }
    const uint32_t zc = depth_rejection(R, a.clip.z, b.clip.z, c.clip.z, fx0, fy0, fx1, fy1, fx2, fy2);
    const float dmin = zc == ZC_LESS || zc == ZC_LEQUAL ? depth_lower_bound(R, a.clip.z, b.clip.z, c.clip.z) : 0.0f;
    float4 *r4 = reinterpret_cast<float4 *>(rec);
    r4[0] = make_float4(fx0, fy0, fx1, fy1);
    r4[1] = make_float4(fx2, fy2, __int_as_float(minX), __int_as_float(minY));
    r4[2] = make_float4(__int_as_float(maxX), __int_as_float(maxY), area, inv_area);
    r4[3] = make_float4(a.clip.z, b.clip.z, c.clip.z, dmin);
    r4[4] = make_float4(a.clip.w, b.clip.w, c.clip.w, lod);
    r4[5] = make_float4(a.col.x, a.col.y, a.col.z, a.col.w);
    r4[6] = make_float4(b.col.x, b.col.y, b.col.z, b.col.w);
    r4[7] = make_float4(c.col.x, c.col.y, c.col.z, c.col.w);
    r4[8] = make_float4(a.uv.x, a.uv.y, b.uv.x, b.uv.y);
    r4[9] = make_float4(c.uv.x, c.uv.y, a.uv.x * a.clip.w, a.uv.y * a.clip.w);
    r4[10] = make_float4(b.uv.x * b.clip.w, b.uv.y * b.clip.w, c.uv.x * c.clip.w, c.uv.y * c.clip.w);
    r4[11] = make_float4(a.ez, b.ez, c.ez, __uint_as_float(raster_id));
    // edge_function(a, b, p) = (px - ax) * (by - ay) - (py - ay) * (bx - ax): the per-edge
    // differences are the same floats whether formed per pixel or once here
    const uint32_t flags = (back ? 1u : 0u) | (zc << 1) | (raises_depth(rs) ? kFlagRaisesDepth : 0u) |
                           ((R.fs.ctl & 0xFFFu) << kRecCtlShift) |
                           (((rs.depth_func - GL_NEVER) & 7u) << kRecDepthFuncShift);
    r4[12] = make_float4(__uint_as_float(flags), fy2 - fy1, fx2 - fx1, fy0 - fy2);
    r4[13] = make_float4(fx0 - fx2, fy1 - fy0, fx1 - fx0, __uint_as_float(frame));
    r4[14] = (zc == ZC_LESS || zc == ZC_LEQUAL) && R.default_depth_range
                 ? depth_plane(a.clip.z, b.clip.z, c.clip.z, fx0, fy0, fx1, fy1, fx2, fy2, area, inv_area, minX, minY,
                               maxX, maxY)
                 : make_float4(0.0f, 0.0f, 0.0f, INFINITY);
    if (eyerec) {
        const float3 aep = cv_ep(a), aen = cv_en(a), bep = cv_ep(b), ben = cv_en(b), cep = cv_ep(c), cen = cv_en(c);
        float4 *e4 = reinterpret_cast<float4 *>(eyerec);
        e4[0] = make_float4(aep.x, aep.y, aep.z, aen.x);
        e4[1] = make_float4(aen.y, aen.z, bep.x, bep.y);
        e4[2] = make_float4(bep.z, ben.x, ben.y, ben.z);
        e4[3] = make_float4(cep.x, cep.y, cep.z, cen.x);
        e4[4] = make_float4(cen.y, cen.z, 0.0f, 0.0f);
    }
    return 1;
}

// vertex elements of line k of a GL_LINES / _STRIP / _LOOP draw (raster.c:1166-1196)
__device__ __forceinline__ void element_pair(uint32_t mode, uint32_t k, uint32_t count, uint32_t &a, uint32_t &b)
{
    if (mode == GL_LINES) {
        a = 2 * k;
        b = 2 * k + 1;
    } else {
        a = k;
        b = (mode == GL_LINE_LOOP && k + 1 == count) ? 0 : k + 1;
    }
}

// K2, one thread per primitive (a point, a line or a triangle of the draw's mode). The count
// pass stores how many records the primitive produces; the emit pass writes them at the
// primitive's offset (exclusive scan of the counts), so records keep submission order.
// Triangles that straddle a clip plane go to a list that k_clip handles: the clipper's
// per-thread vertex buffers live in local memory, and keeping them off this kernel's
// threads keeps that memory small enough to stay in cache.
template <bool EYE>
struct Prim {
    const DevDraw *D;
    const DevRaster *R;
    uint32_t k, frame;
    FrameDims dims;
};

template <bool EYE>
__device__ __forceinline__ Prim<EYE> prim_of(const GeomArgs &A, uint32_t t)
{
    Prim<EYE> p;
    const int d = find_base(A.draw_tri_base, A.ndraws, t);
    p.D = &A.draws[d];
    p.k = t - p.D->tri_base;
    p.R = &A.rasters[p.D->raster];
    p.frame = min(p.R->frame, A.nframes - 1);
    p.dims = A.frames[p.frame].dims;
    return p;
}

__device__ __forceinline__ RecOut rec_out(const GeomArgs &A, uint32_t t, bool emit, bool eye)
{
    RecOut o;
    o.recs = emit ? A.records : nullptr;
    o.eyes = (emit && eye) ? A.eye_records : nullptr;
    o.base = emit ? A.tri_offsets[t] : 0;
    o.cap = A.records_cap;
    return o;
}

template <bool EMIT, bool EYE>
__global__ void __launch_bounds__(128) k_setup(GeomArgs A)
{
    using V = CVx<EYE>;
    // the emit pass takes the primitives the count pass listed (those with records to write,
    // straddling triangles aside); records go to each one's scanned offset, in order
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    bool live = true;
    if (EMIT) {
        if (t >= min(A.list_counts[1], A.total_tris)) return;
        t = A.emit_list[t];
    } else {
        live = t < A.total_tris;  // the count pass keeps every thread for its block's appends
    }
    uint32_t produced = 0;
    bool straddles = false;  // count pass: goes to the clip list, with its clip class
    uint32_t cls = 0;

    if (live) {
        const Prim<EYE> P = prim_of<EYE>(A, t);
        const DevDraw &D = *P.D;
        const DevRaster &R = *P.R;
        const RecOut o = rec_out(A, t, EMIT, EYE);
        if (D.mode == GL_POINTS) {
            V v;
            load_cv(A, element_slot(D, P.k), v);
            produced = vertex_point(R, D.raster, P.frame, P.dims, v, o.rec(0));
        } else if (D.mode == GL_LINES || D.mode == GL_LINE_STRIP || D.mode == GL_LINE_LOOP) {
            uint32_t e0, e1;
            element_pair(D.mode, P.k, (uint32_t)D.count, e0, e1);
            V v0, v1;
            load_cv(A, element_slot(D, e0), v0);
            load_cv(A, element_slot(D, e1), v1);
            produced = segment_line(R, D.raster, P.frame, P.dims, v0, v1, o.rec(0));
        } else {
            uint32_t e0, e1, e2;
            element_triple(D.mode, P.k, e0, e1, e2);
            const uint32_t s0 = element_slot(D, e0), s1 = element_slot(D, e1), s2 = element_slot(D, e2);
            if (!EMIT && R.rs.polygon_mode_front == GL_FILL && R.rs.polygon_mode_back == GL_FILL) {
                // counting a filled triangle: its positions alone decide (as in k_clip's count pass)
                ClipPos v0{A.verts.clip[s0]}, v1{A.verts.clip[s1]}, v2{A.verts.clip[s2]};
                const uint32_t m0 = inside_mask(v0.clip), m1 = inside_mask(v1.clip), m2 = inside_mask(v2.clip);
                const int start = clip_start(m0, m1, m2);
                if (start == kClipNone) {
                    persp_divide(v0);
                    persp_divide(v1);
                    persp_divide(v2);
                    TriBox tb;
                    produced = tri_box(R.rs, P.dims, v0.clip, v1.clip, v2.clip, tb) == kTriFill ? 1u : 0u;
                } else if (start != kClipEmpty) {
                    cls = A.clip_sorted ? clip_class(m0, m1, m2, start) : 0u;
                    straddles = true;
                }
            } else {
                V v0, v1, v2;
                load_cv(A, s0, v0);
                load_cv(A, s1, v1);
                load_cv(A, s2, v2);
                const uint32_t m0 = inside_mask(v0.clip), m1 = inside_mask(v1.clip), m2 = inside_mask(v2.clip);
                const int start = clip_start(m0, m1, m2);
                if (start == kClipNone) {  // the clipper would return the triangle unchanged
                    persp_divide(v0);
                    persp_divide(v1);
                    persp_divide(v2);
                    produced = setup_fan_tri(R, D.raster, P.frame, P.dims, v0, v1, v2, o, 0);
                } else if (start != kClipEmpty) {
                    if (EMIT) return;  // k_clip emits it
                    cls = A.clip_sorted ? clip_class(m0, m1, m2, start) : 0u;
                    straddles = true;
                }
            }
        }
    }
    if (EMIT) return;
    // Primitives with records to write go to the emit list, straddling triangles to the clip
    // list (k_clip stores their counts). The appends are combined per block: one atomic per
    // list and block, and per warp one per clip class present in the warp.
    constexpr int kWarps = 128 / 32;
    __shared__ uint32_t s_n[2][kWarps], s_at[2][kWarps];  // per list and warp: entries, first slot
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t below = (1u << lane) - 1u;
    const bool emit = live && !straddles && produced != 0;
    const uint32_t emits = __ballot_sync(0xffffffffu, emit), want = __ballot_sync(0xffffffffu, straddles);
    if (lane == 0) {
        s_n[0][warp] = (uint32_t)__popc(emits);
        s_n[1][warp] = (uint32_t)__popc(want);
    }
    __syncthreads();
    if (threadIdx.x < 2) {  // thread 0: the emit list, thread 1: the clip list
        const uint32_t l = threadIdx.x;
        uint32_t total = 0;
        for (int w = 0; w < kWarps; w++) total += s_n[l][w];
        uint32_t at = total ? atomicAdd(A.list_counts + (l == 0 ? 1 : 0), total) : 0u;
        for (int w = 0; w < kWarps; w++) {
            s_at[l][w] = at;
            at += s_n[l][w];
        }
    }
    __syncthreads();
    if (emit) {
        const uint32_t slot = s_at[0][warp] + (uint32_t)__popc(emits & below);
        if (slot < A.total_tris) A.emit_list[slot] = t;
    }
    if (want) {
        uint32_t rank = 0;
        const uint32_t bucket = cls * kClipSlots + (blockIdx.x & (kClipSlots - 1));
        if (A.clip_sorted) {
            const uint32_t peers = __match_any_sync(0xffffffffu, straddles ? bucket : 0xFFFFFFFFu);
            const int leader = __ffs(peers) - 1;
            uint32_t rb = 0;
            if (straddles && (int)lane == leader) rb = atomicAdd(A.class_count + bucket, (uint32_t)__popc(peers));
            rb = __shfl_sync(0xffffffffu, rb, leader);
            rank = rb + (uint32_t)__popc(peers & below);
        }
        if (straddles) {
            const uint32_t slot = s_at[1][warp] + (uint32_t)__popc(want & below);
            if (slot < A.total_tris) {
                A.clip_list[slot] = t;
                if (A.clip_sorted) A.clip_class[slot] = (bucket << 20) | rank;
            }
            return;
        }
    }
    if (live) A.tri_counts[t] = produced;
}

// A straddling triangle clipped (from its first crossed plane: in registers when that plane is
// the only one crossed, else the general clipper), divided and fanned; returns the records
// produced, written through `o` in the emit pass.
template <class V>
__device__ __forceinline__ uint32_t clip_fan(const DevRaster &R, uint32_t raster_id, uint32_t frame,
                                             const FrameDims &dims, const V &v0, const V &v1, const V &v2,
                                             const RecOut &o)
{
    const int start = clip_start(inside_mask(v0.clip), inside_mask(v1.clip), inside_mask(v2.clip));
    uint32_t produced = 0;
    V bufA[kClipMax];
    int nv = 0;
    if (start < kClipNone) {
        nv = clip_one_plane(v0, v1, v2, start, bufA[0], bufA[1], bufA[2], bufA[3]);
        if (!nv) {
            V bufB[kClipMax];
            bufA[0] = v0;
            bufA[1] = v1;
            bufA[2] = v2;
            nv = clip_triangle(bufA, bufB, start);
        }
    }
    if (nv >= 3) {
        for (int j = 0; j < nv; j++) persp_divide(bufA[j]);
        for (int j = 1; j + 1 < nv; j++)
            produced += setup_fan_tri(R, raster_id, frame, dims, bufA[0], bufA[j], bufA[j + 1], o, produced);
    }
    return produced;
}

// clip_fan's count for a filled triangle (both polygon modes GL_FILL): the same clipping of
// the positions (the other attributes never decide a filled triangle's records), then
// tri_box per fan triangle.
__device__ __forceinline__ uint32_t clip_fan_count(const DevRaster &R, const FrameDims &dims, const ClipPos &v0,
                                                   const ClipPos &v1, const ClipPos &v2)
{
    const int start = clip_start(inside_mask(v0.clip), inside_mask(v1.clip), inside_mask(v2.clip));
    ClipPos bufA[kClipMax];
    int nv = 0;
    if (start < kClipNone) {
        nv = clip_one_plane(v0, v1, v2, start, bufA[0], bufA[1], bufA[2], bufA[3]);
        if (!nv) {
            ClipPos bufB[kClipMax];
            bufA[0] = v0;
            bufA[1] = v1;
            bufA[2] = v2;
            nv = clip_triangle(bufA, bufB, start);
        }
    }
    uint32_t produced = 0;
    if (nv >= 3) {
        for (int j = 0; j < nv; j++) persp_divide(bufA[j]);
        for (int j = 1; j + 1 < nv; j++) {
            TriBox tb;
            produced += tri_box(R.rs, dims, bufA[0].clip, bufA[j].clip, bufA[j + 1].clip, tb) == kTriFill ? 1u : 0u;
        }
    }
    return produced;
}

// The listed triangles: Sutherland-Hodgman from the first plane that is not all-inside, then
// the fan. Grid-strided over the list (its length is on the device), with the grid capped
// so that the resident threads' clip buffers fit in cache.
template <bool EMIT, bool EYE>
__global__ void __launch_bounds__(64) k_clip(GeomArgs A)
{
    using V = CVx<EYE>;
    const uint32_t n = min(A.list_counts[0], A.total_tris);
    const uint32_t *list = A.clip_sorted ? A.clip_sorted : A.clip_list;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t t = list[i];
        if (EMIT && A.tri_counts[t] == 0) continue;
        const Prim<EYE> P = prim_of<EYE>(A, t);
        const DevDraw &D = *P.D;
        const DevRaster &R = *P.R;
        const RecOut o = rec_out(A, t, EMIT, EYE);
        uint32_t e0, e1, e2;
        element_triple(D.mode, P.k, e0, e1, e2);
        const uint32_t s0 = element_slot(D, e0), s1 = element_slot(D, e1), s2 = element_slot(D, e2);
        uint32_t produced;
        if (!EMIT && R.rs.polygon_mode_front == GL_FILL && R.rs.polygon_mode_back == GL_FILL) {
            // counting a filled triangle: clip the positions alone
            produced = clip_fan_count(R, P.dims, ClipPos{A.verts.clip[s0]}, ClipPos{A.verts.clip[s1]},
                                      ClipPos{A.verts.clip[s2]});
        } else {
            V v0, v1, v2;
            load_cv(A, s0, v0);
            load_cv(A, s1, v1);
            load_cv(A, s2, v2);
            produced = clip_fan(R, D.raster, P.frame, P.dims, v0, v1, v2, o);
        }
        if (!EMIT) A.tri_counts[t] = produced;
    }
}

// groups the clip list by class (clip_class): entry i goes to its bucket's start + its rank
// (buckets class-major, so each class's entries are contiguous)
__global__ void __launch_bounds__(256) k_clip_sort(GeomArgs A)
{
    const uint32_t n = min(A.list_counts[0], A.total_tris);
    if (blockIdx.x * blockDim.x >= n) return;  // no entries for this block (uniform)
    // exclusive prefix of the bucket counts (class-major), in shared memory: each thread sums
    // kPer consecutive buckets, the warps scan those sums, then each thread writes its starts
    constexpr uint32_t kPer = kClipBuckets / 256;
    static_assert(kClipBuckets % 256 == 0, "buckets per thread");
    __shared__ uint32_t start[kClipBuckets];
    __shared__ uint32_t warp_sum[8];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t c[kPer], sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kPer; k++) {
        c[k] = A.class_count[threadIdx.x * kPer + k];
        sum += c[k];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += v;
    }
    if (lane == 31) warp_sum[warp] = incl;
    __syncthreads();
    uint32_t run = incl - sum;
    for (uint32_t w = 0; w < warp; w++) run += warp_sum[w];
#pragma unroll
    for (uint32_t k = 0; k < kPer; k++) {
        start[threadIdx.x * kPer + k] = run;
        run += c[k];
    }
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t w = A.clip_class[i];
        A.clip_sorted[start[w >> 20] + (w & 0xFFFFFu)] = A.clip_list[i];
    }
}

int launch_vertex(const GeomArgs &a, cudaStream_t s)
{
    if (!a.total_slots) return 0;
    k_vertex<<<(a.total_slots + 127) / 128, 128, 0, s>>>(a);
    return 1;
}

namespace {

unsigned clip_grid(const GeomArgs &a)
{
    const uint64_t want = ((uint64_t)a.total_tris + 63) / 64;
    const uint64_t cap = (uint64_t)(a.sms > 0 ? a.sms : 1) * 8;  // 512 clipping threads per SM
    return (unsigned)std::max<uint64_t>(1, std::min(want, cap));
}

template <bool EMIT>
int launch_setup(const GeomArgs &a, cudaStream_t s)
{
    const unsigned g = (a.total_tris + 127) / 128;
    int launches = 2;
    if (a.eyes) k_setup<EMIT, true><<<g, 128, 0, s>>>(a);
    else k_setup<EMIT, false><<<g, 128, 0, s>>>(a);
    if (!EMIT && a.clip_sorted) {  // the count pass groups the list once; the emit pass reuses it
        k_clip_sort<<<clip_grid(a), 256, 0, s>>>(a);
        launches++;
    }
    if (a.eyes) k_clip<EMIT, true><<<clip_grid(a), 64, 0, s>>>(a);
    else k_clip<EMIT, false><<<clip_grid(a), 64, 0, s>>>(a);
    return launches;
}

}  // namespace

int launch_setup_count(const GeomArgs &a, cudaStream_t s)
{
    if (!a.total_tris) return 0;
    cudaMemsetAsync(a.list_counts, 0, 2 * sizeof(uint32_t), s);
    if (a.clip_sorted) cudaMemsetAsync(a.class_count, 0, kClipBuckets * sizeof(uint32_t), s);
    return launch_setup<false>(a, s);
}

int launch_setup_emit(const GeomArgs &a, cudaStream_t s)
{
    if (!a.total_tris) return 0;
    return launch_setup<true>(a, s);
}

}  // namespace mtgl
