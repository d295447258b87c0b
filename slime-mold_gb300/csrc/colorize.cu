// colorize.cu - headless display feed: the colourise pass of
// src/display.wgsl:44-86 (trail -> 256-entry LUT -> RGBA8 with aspect fit and
// black bars) written to a device buffer instead of a storage texture.
#include "kernels.h"

namespace slime {
namespace {

__global__ void colorize_kernel(const float* __restrict__ trail, int W, int H, const uint8_t* __restrict__ lut,
                                int tw, int th, float scale, float off_x, float off_y,
                                uchar4* __restrict__ rgba) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= tw || iy >= th) return;
    float sim_w = slm_i2f(W), sim_h = slm_i2f(H);
    float fx = slm_div(slm_sub(slm_i2f(ix), off_x), scale); // display.wgsl:72-73
    float fy = slm_div(slm_sub(slm_i2f(iy), off_y), scale);
    uchar4 o = make_uchar4(0, 0, 0, 255);
    if (fx >= 0.0f && fx < sim_w && fy >= 0.0f && fy < sim_h) { // :76
        int x = slm_f2i(fx), y = slm_f2i(fy);
        float intensity = slm_clamp(__ldg(trail + (size_t)y * W + x), 0.0f, 1.0f);
        int idx = slm_f2i(slm_mul(intensity, 255.0f)); // get_lut_color, :29-42
        o = make_uchar4(lut[idx], lut[idx + 256], lut[idx + 512], 255);
    }
    rgba[(size_t)iy * tw + ix] = o;
}

} // namespace

cudaError_t launch_colorize(const float* trail, uint32_t W, uint32_t H, const uint8_t* lut, uint32_t tw,
                            uint32_t th, uint8_t* rgba, cudaStream_t s) {
    // Aspect fit, display.wgsl:53-69, computed once on the host with the same
    // binary32 operations.
    float sim_w = (float)W, sim_h = (float)H, tex_w = (float)tw, tex_h = (float)th;
    float sim_aspect = slm_div(sim_w, sim_h), tex_aspect = slm_div(tex_w, tex_h);
    float scale, off_x = 0.0f, off_y = 0.0f;
    if (tex_aspect > sim_aspect) {
        scale = slm_div(tex_h, sim_h);
        off_x = slm_mul(slm_sub(tex_w, slm_mul(sim_w, scale)), 0.5f);
    } else {
        scale = slm_div(tex_w, sim_w);
        off_y = slm_mul(slm_sub(tex_h, slm_mul(sim_h, scale)), 0.5f);
    }
    dim3 block(16, 16), grid((tw + 15) / 16, (th + 15) / 16);
    colorize_kernel<<<grid, block, 0, s>>>(trail, (int)W, (int)H, lut, (int)tw, (int)th, scale, off_x, off_y,
                                           (uchar4*)rgba);
    return cudaGetLastError();
}

} // namespace slime
