// post_process.cu - the post-process pass of the reference's frame
// (shaders/post_process.comp, dispatched at source/taa.hpp:1141-1158): the
// split-screen line, the zoom source box and its magnified inset, and the
// debug image shown on either side of the split (its alpha made visible in
// red and blue when that side's mask .w is positive).
//
// A warp takes 128 texels of a row, each lane four of them 32 apart (every
// access of the warp 256 contiguous bytes), eight rows to a CTA; a thread
// issues its four loads before its first store.  Texels copied unchanged from
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

// What one output texel shows and where it reads it from.
enum PostKind : int { kBlack, kRed, kWhite, kDebug, kInput };

__device__ __forceinline__ PostKind post_source(const PostArgs& a, int x, int y, int& fx, int& fy) {
    fx = x;
    fy = y;
    // the split-screen line (post_process.comp:43-46)
    if (x == a.split_x) return kBlack;
    const int* zs = a.zoom_src;
    const int* zd = a.zoom_dst;
    // the border one texel outside the zoomed source box (49-54)
    if (a.zoom && a.show_zoom_box) {
        const bool col = (x == zs[0] - 1 || x == zs[0] + zs[2]) && y >= zs[1] - 1 && y <= zs[1] + zs[3];
        const bool row = (y == zs[1] - 1 || y == zs[1] + zs[3]) && x >= zs[0] - 1 && x <= zs[0] + zs[2];
        if (col || row) return kRed;
    }
    // the inset (57-70): a white border, inside it the source box magnified
    if (a.zoom && x >= zd[0] && y >= zd[1] && x < zd[0] + zd[2] && y < zd[1] + zd[3]) {
        const bool col = (x == zd[0] || x == zd[0] + zd[2] - 1) && y >= zd[1] && y <= zd[1] + zd[3] - 1;
        const bool row = (y == zd[1] || y == zd[1] + zd[3] - 1) && x >= zd[0] && x <= zd[0] + zd[2] - 1;
        if (col || row) return kWhite;
        const float ux = ((float)(x - zd[0]) + 0.5f) / (float)zd[2];
        const float uy = ((float)(y - zd[1]) + 0.5f) / (float)zd[3];
        fx = trunc_index((float)zs[0] + ux * (float)zs[2]);
        fy = trunc_index((float)zs[1] + uy * (float)zs[3]);
    }
    fx = clampi(fx, 0, a.w - 1);
    fy = clampi(fy, 0, a.h - 1);
    // the debug image or the input, by the side of the split (73-89)
    const bool left = a.split_x < 0 || x < a.split_x;
    return (left ? a.show_l : a.show_r) ? kDebug : kInput;
}

// A warp covers kSpan consecutive texels of one row, each lane kPer of them
// kWarpX apart (coalesced); the texels' sources are resolved and all loads
// issued before the first store.
constexpr int kPer = 4, kWarpX = 32, kSpan = kPer * kWarpX, kRows = 8;

__global__ void __launch_bounds__(256) post_process_kernel(const PostArgs a) {
    const int lane = (int)(threadIdx.x & 31u);
    const int y = (int)blockIdx.y * kRows + (int)(threadIdx.x >> 5);
    if (y >= a.h) return;
    const int x0 = (int)blockIdx.x * kSpan + lane;
    PostKind kind[kPer];
    uint2 v[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int x = x0 + j * kWarpX;
        int fx = 0, fy = 0;
        kind[j] = x < a.w ? post_source(a, x, y, fx, fy) : kBlack;
        v[j] = make_uint2(0u, 0u);
        if (x < a.w && kind[j] >= kDebug) v[j] = __ldg(texel_ptr<uint2>(kind[j] == kDebug ? a.debug : a.in, fx, fy));
    }
    constexpr uint32_t kOne = 0x3c00u;  // 1.0 in FP16
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int x = x0 + j * kWarpX;
        if (x >= a.w) break;
        uint2 o = v[j];
        if (kind[j] == kRed) {
            o = make_uint2(kOne, 0u);
        } else if (kind[j] == kWhite) {
            o = make_uint2(kOne | (kOne << 16), kOne);
        } else if (kind[j] == kDebug) {
            float4 d = half4_to_float4(v[j]);
            if ((x < a.split_x || a.split_x < 0 ? a.mask_l_w : a.mask_r_w) > 0.f) {
                d.x = d.x + d.w;  // the alpha made visible in red and blue
                d.z = d.z + d.w;
            }
            o = make_uint2(half2_bits(d.x, d.y), half2_bits(d.z, 1.0f));
        }
        *texel_ptr_w<uint2>(a.out, x, y) = o;
    }
}

}  // namespace

cudaError_t launch_post_process(const PostArgs& a, cudaStream_t stream) {
    const dim3 grid((unsigned)((a.w + kSpan - 1) / kSpan), (unsigned)((a.h + kRows - 1) / kRows));
    post_process_kernel<<<grid, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace taa_dev
