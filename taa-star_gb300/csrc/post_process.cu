// post_process.cu - the post-process pass of the reference's frame
// (shaders/post_process.comp, dispatched at source/taa.hpp:1141-1158): the
// split-screen line, the zoom source box and its magnified inset, and the
// debug image shown on either side of the split (its alpha made visible in
// red and blue when that side's mask .w is positive).
//
// One thread per output texel, 32 x 8 threads per CTA so that a warp reads and
// writes 256 contiguous bytes of a row.  Texels that are copied unchanged from
// the input move as their RGBA16F bits; a debug texel goes through FP32 (the
// alpha added in FP32, then rounded to RGBA16F, as the shader's vec4 and the
// image store do).  The inset's source position is FP32 arithmetic in the
// shader's order (compiled with -fmad=false: no contraction), truncated toward
// zero; every fetch is clamped to the image.
#include <cuda_fp16.h>

#include "kernels.h"

namespace taa_dev {

namespace {

__device__ __forceinline__ uint32_t half2_bits(float lo, float hi) {
    const __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__global__ void __launch_bounds__(256) post_process_kernel(const PostArgs a) {
    const int x = (int)blockIdx.x * 32 + (int)(threadIdx.x & 31u);
    const int y = (int)blockIdx.y * 8 + (int)(threadIdx.x >> 5);
    if (x >= a.w || y >= a.h) return;
    uint2* dst = texel_ptr_w<uint2>(a.out, x, y);
    constexpr uint32_t kOne = 0x3c00u;  // 1.0 in FP16
    // the split-screen line (post_process.comp:43-46)
    if (x == a.split_x) {
        *dst = make_uint2(0u, 0u);
        return;
    }
    const int* zs = a.zoom_src;
    const int* zd = a.zoom_dst;
    // the border one texel outside the zoomed source box (49-54): red
    if (a.zoom && a.show_zoom_box) {
        const bool col = (x == zs[0] - 1 || x == zs[0] + zs[2]) && y >= zs[1] - 1 && y <= zs[1] + zs[3];
        const bool row = (y == zs[1] - 1 || y == zs[1] + zs[3]) && x >= zs[0] - 1 && x <= zs[0] + zs[2];
        if (col || row) {
            *dst = make_uint2(kOne, 0u);
            return;
        }
    }
    // the inset (57-70): a white border, inside it the source box magnified
    int fx = x, fy = y;
    if (a.zoom && x >= zd[0] && y >= zd[1] && x < zd[0] + zd[2] && y < zd[1] + zd[3]) {
        const bool col = (x == zd[0] || x == zd[0] + zd[2] - 1) && y >= zd[1] && y <= zd[1] + zd[3] - 1;
        const bool row = (y == zd[1] || y == zd[1] + zd[3] - 1) && x >= zd[0] && x <= zd[0] + zd[2] - 1;
        if (col || row) {
            *dst = make_uint2(kOne | (kOne << 16), kOne);
            return;
        }
        const float ux = ((float)(x - zd[0]) + 0.5f) / (float)zd[2];
        const float uy = ((float)(y - zd[1]) + 0.5f) / (float)zd[3];
        fx = trunc_index((float)zs[0] + ux * (float)zs[2]);
        fy = trunc_index((float)zs[1] + uy * (float)zs[3]);
    }
    fx = clampi(fx, 0, a.w - 1);
    fy = clampi(fy, 0, a.h - 1);
    // the debug image or the input, by the side of the split (73-89)
    const bool left = a.split_x < 0 || x < a.split_x;
    if (left ? a.show_l : a.show_r) {
        float4 d = half4_to_float4(__ldg(texel_ptr<uint2>(a.debug, fx, fy)));
        if ((left ? a.mask_l_w : a.mask_r_w) > 0.f) {
            d.x = d.x + d.w;
            d.z = d.z + d.w;
        }
        *dst = make_uint2(half2_bits(d.x, d.y), half2_bits(d.z, 1.0f));
        return;
    }
    *dst = __ldg(texel_ptr<uint2>(a.in, fx, fy));
}

}  // namespace

cudaError_t launch_post_process(const PostArgs& a, cudaStream_t stream) {
    const dim3 grid((unsigned)((a.w + 31) / 32), (unsigned)((a.h + 7) / 8));
    post_process_kernel<<<grid, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace taa_dev
