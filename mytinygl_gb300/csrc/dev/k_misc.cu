// k_misc.cu — clears without draws, mip level 1 construction, the glDrawPixels blit and colour read-back.
#include <algorithm>

#include "dev_kernels.h"

namespace mtgl {

constexpr int kMaxClearOps = 16;
struct ClearBatch {
    ClearOp op[kMaxClearOps];
    int n;
};

// glClear (gl_api.c:409-457): colour, depth, stencil over a scissor-limited rectangle,
// every op applied in order, one pixel per thread.
__global__ void __launch_bounds__(256) k_clear(ClearBatch B, FrameDims dims, uint32_t *color, float *depth,
                                               uint8_t *stencil)
{
    const int x = (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y;
    if (x >= dims.width || y >= dims.height) return;
    const size_t i = (size_t)y * dims.width + x;
    for (int k = 0; k < B.n; k++) {
        const ClearOp &c = B.op[k];
        if (x < c.x0 || x >= c.x1 || y < c.y0 || y >= c.y1) continue;
        if (c.mask & GL_COLOR_BUFFER_BIT) color[i] = c.color;
        if (c.mask & GL_DEPTH_BUFFER_BIT) depth[i] = c.depth;
        if (c.mask & GL_STENCIL_BUFFER_BIT) stencil[i] = (uint8_t)c.stencil;
    }
}

void launch_clear(const ClearOp *ops, int nops, FrameDims dims, uint32_t *color, float *depth, uint8_t *stencil,
                  cudaStream_t s)
{
    for (int base = 0; base < nops; base += kMaxClearOps) {
        ClearBatch b;
        b.n = nops - base < kMaxClearOps ? nops - base : kMaxClearOps;
        for (int i = 0; i < b.n; i++) b.op[i] = ops[base + i];
        dim3 grid((dims.width + 255) / 256, dims.height);
        k_clear<<<grid, 256, 0, s>>>(b, dims, color, depth, stencil);
    }
}

// texture_generate_mip1 (textures.c:311-354): 2x2 box filter in float, truncated to RGBA8.
// Built when the image is uploaded; the reference builds it on first use, with the same result.
__global__ void __launch_bounds__(256) k_mip1(const uint32_t *base, int32_t w, int32_t h, uint32_t *mip)
{
    const int32_t mw = w / 2, mh = h / 2;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)mw * mh) return;
    const int32_t x = (int32_t)(i % mw), y = (int32_t)(i / mw);
    const int32_t sx = 2 * x, sy = 2 * y;
    const float4 c00 = unpack_rgba(base[(size_t)sy * w + sx]);
    const float4 c10 = unpack_rgba(base[(size_t)sy * w + sx + 1]);
    const float4 c01 = unpack_rgba(base[(size_t)(sy + 1) * w + sx]);
    const float4 c11 = unpack_rgba(base[(size_t)(sy + 1) * w + sx + 1]);
    float4 c = make_float4(c00.x + c10.x, c00.y + c10.y, c00.z + c10.z, c00.w + c10.w);
    c = make_float4(c.x + c01.x, c.y + c01.y, c.z + c01.z, c.w + c01.w);
    c = make_float4(c.x + c11.x, c.y + c11.y, c.z + c11.z, c.w + c11.w);
    c = make_float4(c.x * 0.25f, c.y * 0.25f, c.z * 0.25f, c.w * 0.25f);
    mip[i] = pack_rgba(c.x, c.y, c.z, c.w);
}

void launch_mip1(const uint32_t *base, int32_t w, int32_t h, uint32_t *mip, cudaStream_t s)
{
    const int64_t n = (int64_t)(w / 2) * (h / 2);
    if (n <= 0) return;
    k_mip1<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(base, w, h, mip);
}

// glDrawPixels (gl_api.c:1287-1376): alpha test, depth test against depth 0, blend, depth
// write of 0, unmasked colour write; image row 0 lands on framebuffer row height-1-raster_y.
__global__ void __launch_bounds__(256) k_draw_pixels(const uint32_t *img, int32_t rx, int32_t ry, int32_t w, int32_t h,
                                                     const DevRaster *raster, FrameDims dims, uint32_t *color,
                                                     float *depth)
{
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= w) return;
    const mtgl_raster_state &rs = raster->rs;
    for (int row = blockIdx.y; row < h; row += gridDim.y) {
        const int32_t fy = dims.height - 1 - (ry + row);
        const int32_t fx = rx + col;
        if (fy < 0 || fy >= dims.height || fx < 0 || fx >= dims.width) continue;
        const uint32_t p = img[(size_t)row * w + col];
        const size_t i = (size_t)fy * dims.width + fx;
        if (rs.alpha_test && !cmp_pass(rs.alpha_func, u8f(p >> 24), rs.alpha_ref)) continue;
        if (rs.depth_test && !cmp_pass(rs.depth_func, 0.0f, depth[i])) continue;
        float4 s = unpack_rgba(p);
        if (rs.blend) s = blend(rs, s, unpack_rgba(color[i]));
        if (rs.depth_test && rs.depth_mask) depth[i] = 0.0f;
        color[i] = pack_rgba(s.x, s.y, s.z, s.w);
    }
}

void launch_draw_pixels(const uint32_t *img, int32_t rx, int32_t ry, int32_t w, int32_t h, const DevRaster *raster,
                        FrameDims dims, uint32_t *color, float *depth, cudaStream_t s)
{
    if (w <= 0 || h <= 0) return;
    dim3 grid((w + 255) / 256, h < 65535 ? h : 65535);
    k_draw_pixels<<<grid, 256, 0, s>>>(img, rx, ry, w, h, raster, dims, color, depth);
}

// Colour read-back into page-locked host memory the device addresses directly: work units
// of kReadbackUnit pixels over all items of the launch, each block finding its unit's item
// by binary search over the items' first units; 16-byte copies where both ends allow them.
__global__ void __launch_bounds__(256) k_readback(const __grid_constant__ ReadbackArgs a)
{
    for (uint32_t u = blockIdx.x; u < a.units; u += gridDim.x) {
        int lo = 0, hi = a.count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.item[mid].first_unit <= u) lo = mid;
            else hi = mid - 1;
        }
        const ReadbackItem &it = a.item[lo];
        const uint32_t p0 = (u - it.first_unit) * kReadbackUnit;
        const uint32_t p1 = min(p0 + kReadbackUnit, it.n);
        uint32_t v1 = p0;  // end of the 16-byte part
        if (((reinterpret_cast<uintptr_t>(it.src) | reinterpret_cast<uintptr_t>(it.dst)) & 15u) == 0) {
            v1 = p0 + ((p1 - p0) & ~3u);
            for (uint32_t p = p0 + threadIdx.x * 4u; p < v1; p += blockDim.x * 4u)
                *reinterpret_cast<uint4 *>(it.dst + p) = __ldg(reinterpret_cast<const uint4 *>(it.src + p));
        }
        for (uint32_t p = v1 + threadIdx.x; p < p1; p += blockDim.x) it.dst[p] = __ldg(it.src + p);
    }
}

int launch_readback(const ReadbackItem *items, int n, int sms, cudaStream_t s)
{
    int launches = 0;
    for (int k = 0; k < n; k += kReadbackMax) {
        ReadbackArgs a;
        a.count = std::min(n - k, kReadbackMax);
        uint32_t units = 0;
        for (int i = 0; i < a.count; i++) {
            a.item[i] = items[k + i];
            a.item[i].first_unit = units;
            units += (a.item[i].n + kReadbackUnit - 1) / kReadbackUnit;
        }
        a.units = units;
        if (!units) continue;
        const unsigned grid = std::min<unsigned>(units, (unsigned)std::max(sms, 1) * 8u);
        k_readback<<<grid, 256, 0, s>>>(a);
        launches++;
    }
    return launches;
}

}  // namespace mtgl
