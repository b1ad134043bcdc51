// fxaa.cu - the FXAA pass of the ray-trace-assist path, fused into one kernel.
//
// The reference runs two dispatches after the resolve when the segmentation
// mask asks for FXAA (source/taa.hpp:1063-1104): a prepare pass writing rgb and
// the luma dot(rgb, (0.299, 0.587, 0.114)) into an RGBA16F temp image
// (shaders/antialias_fxaa_prepare.comp:19-26), then FXAA 3.11 quality preset 12
// (shaders/antialias_fxaa.comp:34-64, shaders/Fxaa3_11_mod.h:726-1249) on the
// pixels with (segmask & 3) == 1, a copy of the temp texel elsewhere.
//
// Here one kernel reads the result image and the mask and writes the output:
// the luma of every tap is computed from the RGBA16F texel and rounded to FP16
// where the reference stores it, so the temp image and its 16 B/px of traffic
// are gone.  Unmarked pixels stream (8 B in, 4 B mask, 8 B out); marked pixels
// run the edge search on taps the L1 serves.
//
// The arithmetic follows the oracle's restatement (oracle/taa_oracle.cpp
// fxaa_pixel) operation for operation; the unit is compiled with -fmad=false.
// Sampler: bilinear, clamp to edge, exact weights, snapping to a texel centre
// within 1/512 texel; taps at whole-texel offsets from the pixel centre read
// texels.
#include "common.cuh"
#include "kernels.h"

namespace taa_dev {
namespace {

constexpr float kSnap = 1.0f / 512.0f;

// the prepared texel: rgb of the result image and its FP16-stored luma
__device__ __forceinline__ float4 prepared(const Img& im, int x, int y) {
    float4 c = fetch_rgba16f(im, x, y);
    float l = c.x * 0.299f + c.y * 0.587f + c.z * 0.114f;
    c.w = __half2float(__float2half_rn(l));
    return c;
}
__device__ __forceinline__ float prepared_luma(const Img& im, int x, int y) { return prepared(im, x, y).w; }

// one coordinate of the bilinear footprint: lower texel and weight
__device__ __forceinline__ void axis(float uvc, int size, int& i0, float& f) {
    float p = uvc * (float)size - 0.5f;
    float c = floorf(p + 0.5f);
    if (fabsf(p - c) < kSnap) p = c;
    float p0 = floorf(p);
    f = p - p0;
    i0 = trunc_index(p0);
    if (!(f == f)) f = 0.f;
}

__device__ __forceinline__ float lerp2(float a, float b, float c, float d, float fx, float fy) {
    float gx = 1.0f - fx, gy = 1.0f - fy;
    float top = a * gx + b * fx, bot = c * gx + d * fx;
    return top * gy + bot * fy;
}

__device__ __forceinline__ float sample_luma(const Img& im, float u, float v) {
    int x0, y0;
    float fx, fy;
    axis(u, im.w, x0, fx);
    axis(v, im.h, y0, fy);
    return lerp2(prepared_luma(im, x0, y0), prepared_luma(im, x0 + 1, y0), prepared_luma(im, x0, y0 + 1),
                 prepared_luma(im, x0 + 1, y0 + 1), fx, fy);
}

__device__ __forceinline__ float3 sample_rgb(const Img& im, float u, float v) {
    int x0, y0;
    float fx, fy;
    axis(u, im.w, x0, fx);
    axis(v, im.h, y0, fy);
    float4 a = fetch_rgba16f(im, x0, y0), b = fetch_rgba16f(im, x0 + 1, y0);
    float4 c = fetch_rgba16f(im, x0, y0 + 1), d = fetch_rgba16f(im, x0 + 1, y0 + 1);
    return make_float3(lerp2(a.x, b.x, c.x, d.x, fx, fy), lerp2(a.y, b.y, c.y, d.y, fx, fy),
                       lerp2(a.z, b.z, c.z, d.z, fx, fy));
}

struct FxaaArgs {
    Img in;        // RGBA16F result image
    Img seg;       // R32UI segmentation mask (p == nullptr: every pixel marked)
    ImgW out;      // RGBA16F
    float rcp_x, rcp_y;
    float subpix, thr, thr_min;
};

// FxaaPixelShader, quality PC path (Fxaa3_11_mod.h:841-1249)
__device__ float4 fxaa_pixel(const FxaaArgs& a, int x, int y) {
    const Img& t = a.in;
    const float rx = a.rcp_x, ry = a.rcp_y;
    float posMx = ((float)x + 0.5f) * rx, posMy = ((float)y + 0.5f) * ry;
    const float4 rgbyM = prepared(t, x, y);
    const float lumaM = rgbyM.w;
    float lumaS = prepared_luma(t, x, y + 1), lumaE = prepared_luma(t, x + 1, y);
    float lumaN = prepared_luma(t, x, y - 1), lumaW = prepared_luma(t, x - 1, y);
    float maxSM = gmax(lumaS, lumaM), minSM = gmin(lumaS, lumaM);
    float maxESM = gmax(lumaE, maxSM), minESM = gmin(lumaE, minSM);
    float maxWN = gmax(lumaN, lumaW), minWN = gmin(lumaN, lumaW);
    float rangeMax = gmax(maxWN, maxESM), rangeMin = gmin(minWN, minESM);
    float rangeMaxScaled = rangeMax * a.thr;
    float range = rangeMax - rangeMin;
    float rangeMaxClamped = gmax(a.thr_min, rangeMaxScaled);
    if (range < rangeMaxClamped) return rgbyM;
    float lumaNW = prepared_luma(t, x - 1, y - 1), lumaSE = prepared_luma(t, x + 1, y + 1);
    float lumaNE = prepared_luma(t, x + 1, y - 1), lumaSW = prepared_luma(t, x - 1, y + 1);
    float lumaNS = lumaN + lumaS, lumaWE = lumaW + lumaE;
    float subpixRcpRange = 1.0f / range;
    float subpixNSWE = lumaNS + lumaWE;
    float edgeHorz1 = (-2.0f * lumaM) + lumaNS;
    float edgeVert1 = (-2.0f * lumaM) + lumaWE;
    float lumaNESE = lumaNE + lumaSE, lumaNWNE = lumaNW + lumaNE;
    float edgeHorz2 = (-2.0f * lumaE) + lumaNESE;
    float edgeVert2 = (-2.0f * lumaN) + lumaNWNE;
    float lumaNWSW = lumaNW + lumaSW, lumaSWSE = lumaSW + lumaSE;
    float edgeHorz4 = (fabsf(edgeHorz1) * 2.0f) + fabsf(edgeHorz2);
    float edgeVert4 = (fabsf(edgeVert1) * 2.0f) + fabsf(edgeVert2);
    float edgeHorz3 = (-2.0f * lumaW) + lumaNWSW;
    float edgeVert3 = (-2.0f * lumaS) + lumaSWSE;
    float edgeHorz = fabsf(edgeHorz3) + edgeHorz4;
    float edgeVert = fabsf(edgeVert3) + edgeVert4;
    float subpixNWSWNESE = lumaNWSW + lumaNESE;
    float lengthSign = rx;
    const bool horzSpan = edgeHorz >= edgeVert;
    float subpixA = subpixNSWE * 2.0f + subpixNWSWNESE;
    if (!horzSpan) {
        lumaN = lumaW;
        lumaS = lumaE;
    } else {
        lengthSign = ry;
    }
    float subpixB = (subpixA * (1.0f / 12.0f)) - lumaM;
    float gradientN = lumaN - lumaM, gradientS = lumaS - lumaM;
    float lumaNN = lumaN + lumaM, lumaSS = lumaS + lumaM;
    const bool pairN = fabsf(gradientN) >= fabsf(gradientS);
    float gradient = gmax(fabsf(gradientN), fabsf(gradientS));
    if (pairN) lengthSign = -lengthSign;
    float subpixC = gclamp(fabsf(subpixB) * subpixRcpRange, 0.0f, 1.0f);
    float posBx = posMx, posBy = posMy;
    const float offx = horzSpan ? rx : 0.0f, offy = horzSpan ? 0.0f : ry;
    if (!horzSpan) posBx += lengthSign * 0.5f;
    else posBy += lengthSign * 0.5f;
    float posNx = posBx - offx * 1.0f, posNy = posBy - offy * 1.0f;
    float posPx = posBx + offx * 1.0f, posPy = posBy + offy * 1.0f;
    float subpixD = (-2.0f * subpixC) + 3.0f;
    float lumaEndN = sample_luma(t, posNx, posNy);
    float subpixE = subpixC * subpixC;
    float lumaEndP = sample_luma(t, posPx, posPy);
    if (!pairN) lumaNN = lumaSS;
    float gradientScaled = gradient * 1.0f / 4.0f;
    float lumaMM = lumaM - lumaNN * 0.5f;
    float subpixF = subpixD * subpixE;
    const bool lumaMLTZero = lumaMM < 0.0f;
    lumaEndN -= lumaNN * 0.5f;
    lumaEndP -= lumaNN * 0.5f;
    bool doneN = fabsf(lumaEndN) >= gradientScaled;
    bool doneP = fabsf(lumaEndP) >= gradientScaled;
    if (!doneN) {
        posNx -= offx * 1.5f;
        posNy -= offy * 1.5f;
    }
    bool doneNP = (!doneN) || (!doneP);
    if (!doneP) {
        posPx += offx * 1.5f;
        posPy += offy * 1.5f;
    }
    // preset 12: steps 1.0, 1.5, then 2.0, 4.0, 12.0 (Fxaa3_11_mod.h:433-440)
    const float kStep[3] = {2.0f, 4.0f, 12.0f};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (!doneNP) break;
        if (!doneN) lumaEndN = sample_luma(t, posNx, posNy);
        if (!doneP) lumaEndP = sample_luma(t, posPx, posPy);
        if (!doneN) lumaEndN = lumaEndN - lumaNN * 0.5f;
        if (!doneP) lumaEndP = lumaEndP - lumaNN * 0.5f;
        doneN = fabsf(lumaEndN) >= gradientScaled;
        doneP = fabsf(lumaEndP) >= gradientScaled;
        if (!doneN) {
            posNx -= offx * kStep[i];
            posNy -= offy * kStep[i];
        }
        doneNP = (!doneN) || (!doneP);
        if (!doneP) {
            posPx += offx * kStep[i];
            posPy += offy * kStep[i];
        }
    }
    float dstN = horzSpan ? posMx - posNx : posMy - posNy;
    float dstP = horzSpan ? posPx - posMx : posPy - posMy;
    const bool goodSpanN = (lumaEndN < 0.0f) != lumaMLTZero;
    float spanLength = dstP + dstN;
    const bool goodSpanP = (lumaEndP < 0.0f) != lumaMLTZero;
    float spanLengthRcp = 1.0f / spanLength;
    const bool directionN = dstN < dstP;
    float dst = gmin(dstN, dstP);
    const bool goodSpan = directionN ? goodSpanN : goodSpanP;
    float subpixG = subpixF * subpixF;
    float pixelOffset = (dst * (-spanLengthRcp)) + 0.5f;
    float subpixH = subpixG * a.subpix;
    float pixelOffsetGood = goodSpan ? pixelOffset : 0.0f;
    float pixelOffsetSubpix = gmax(pixelOffsetGood, subpixH);
    if (!horzSpan) posMx += pixelOffsetSubpix * lengthSign;
    else posMy += pixelOffsetSubpix * lengthSign;
    float3 c = sample_rgb(t, posMx, posMy);
    return make_float4(c.x, c.y, c.z, lumaM);
}

constexpr int kBX = 32, kBY = 8;

__global__ void __launch_bounds__(kBX * kBY) fxaa_kernel(const FxaaArgs a) {
    const int x = blockIdx.x * kBX + threadIdx.x, y = blockIdx.y * kBY + threadIdx.y;
    if (x >= a.in.w || y >= a.in.h) return;
    bool marked = true;
    if (a.seg.p) marked = (__ldg(texel_ptr<uint32_t>(a.seg, x, y)) & 3u) == 1u;  // antialias_fxaa.comp:39-40
    float4 c = marked ? fxaa_pixel(a, x, y) : prepared(a.in, x, y);
    store_rgba16f(a.out, x, y, c);
}

}  // namespace

cudaError_t launch_fxaa(const Img& in, const Img& segmask, const ImgW& out, const float rcp[2], float subpix,
                        float edge_threshold, float edge_threshold_min, cudaStream_t s) {
    FxaaArgs a{in, segmask, out, rcp[0], rcp[1], subpix, edge_threshold, edge_threshold_min};
    dim3 block(kBX, kBY), grid((in.w + kBX - 1) / kBX, (in.h + kBY - 1) / kBY);
    fxaa_kernel<<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace taa_dev
