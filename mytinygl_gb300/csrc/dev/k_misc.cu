// k_misc.cu — clears without draws, mip level 1 construction and the glDrawPixels blit.
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

}  // namespace mtgl
