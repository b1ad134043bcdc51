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

// FxaaPixelShader, quality PC path (Fxaa3_11_mod.h:841-1249).  Not inlined:
// the streaming path around it stays small, and marked pixels are few; its
// arguments are scalars so that the call passes them in registers.
__device__ __noinline__ float4 fxaa_pixel(const char* in, size_t pitch, int w, int h, float rx, float ry,
                                          float subpix, float thr, float thr_min, int x, int y) {
    const Img t{in, pitch, w, h};
    float posMx = ((float)x + 0.5f) * rx, posMy = ((float)y + 0.5f) * ry;
    // the 3x3 neighbourhood in one round of loads (the corners are needed
    // unless the early exit below is taken)
    const float4 rgbyM = prepared(t, x, y);
    const float lumaM = rgbyM.w;
    float lumaS = prepared_luma(t, x, y + 1), lumaE = prepared_luma(t, x + 1, y);
    float lumaN = prepared_luma(t, x, y - 1), lumaW = prepared_luma(t, x - 1, y);
    const float lumaNW = prepared_luma(t, x - 1, y - 1), lumaSE = prepared_luma(t, x + 1, y + 1);
    const float lumaNE = prepared_luma(t, x + 1, y - 1), lumaSW = prepared_luma(t, x - 1, y + 1);
    float maxSM = gmax(lumaS, lumaM), minSM = gmin(lumaS, lumaM);
    float maxESM = gmax(lumaE, maxSM), minESM = gmin(lumaE, minSM);
    float maxWN = gmax(lumaN, lumaW), minWN = gmin(lumaN, lumaW);
    float rangeMax = gmax(maxWN, maxESM), rangeMin = gmin(minWN, minESM);
    float rangeMaxScaled = rangeMax * thr;
    float range = rangeMax - rangeMin;
    float rangeMaxClamped = gmax(thr_min, rangeMaxScaled);
    if (range < rangeMaxClamped) return rgbyM;
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
    // The walk along the edge (Fxaa3_11_mod.h:993-1190): each end moves out by
    // 1.0, 1.5, 2.0, 4.0, 12.0 texels (preset 12, 433-440) while its luma stays
    // within a quarter gradient of the pair's average, sampling after each of
    // the first four moves.  The two ends do not depend on each other, so the
    // four taps of each end are fetched in one round and the walk is replayed
    // on them: the same positions, values and decisions as the step-by-step loop.
    const float kWalk[5] = {1.0f, 1.5f, 2.0f, 4.0f, 12.0f};
    float pnx[5], pny[5], ppx[5], ppy[5];
    pnx[0] = posBx - offx * kWalk[0];
    pny[0] = posBy - offy * kWalk[0];
    ppx[0] = posBx + offx * kWalk[0];
    ppy[0] = posBy + offy * kWalk[0];
#pragma unroll
    for (int k = 1; k < 5; ++k) {
        pnx[k] = pnx[k - 1] - offx * kWalk[k];
        pny[k] = pny[k - 1] - offy * kWalk[k];
        ppx[k] = ppx[k - 1] + offx * kWalk[k];
        ppy[k] = ppy[k - 1] + offy * kWalk[k];
    }
    float ln[4], lp[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        ln[k] = sample_luma(t, pnx[k], pny[k]);
        lp[k] = sample_luma(t, ppx[k], ppy[k]);
    }
    float subpixD = (-2.0f * subpixC) + 3.0f;
    float subpixE = subpixC * subpixC;
    if (!pairN) lumaNN = lumaSS;
    float gradientScaled = gradient * 1.0f / 4.0f;
    float lumaMM = lumaM - lumaNN * 0.5f;
    float subpixF = subpixD * subpixE;
    const bool lumaMLTZero = lumaMM < 0.0f;
    // the first sample at or beyond the quarter gradient ends the walk of a side
    int kn = 4, kp = 4;
#pragma unroll
    for (int k = 3; k >= 0; --k) {
        if (fabsf(ln[k] - lumaNN * 0.5f) >= gradientScaled) kn = k;
        if (fabsf(lp[k] - lumaNN * 0.5f) >= gradientScaled) kp = k;
    }
    float lumaEndN = ln[0], lumaEndP = lp[0], posNx = pnx[4], posNy = pny[4], posPx = ppx[4], posPy = ppy[4];
#pragma unroll
    for (int k = 3; k >= 0; --k) {
        if (kn <= k) {
            lumaEndN = ln[k];
            posNx = pnx[k];
            posNy = pny[k];
        }
        if (kp <= k) {
            lumaEndP = lp[k];
            posPx = ppx[k];
            posPy = ppy[k];
        }
    }
    if (kn == 4) lumaEndN = ln[3];
    if (kp == 4) lumaEndP = lp[3];
    lumaEndN = lumaEndN - lumaNN * 0.5f;
    lumaEndP = lumaEndP - lumaNN * 0.5f;
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
    float subpixH = subpixG * subpix;
    float pixelOffsetGood = goodSpan ? pixelOffset : 0.0f;
    float pixelOffsetSubpix = gmax(pixelOffsetGood, subpixH);
    if (!horzSpan) posMx += pixelOffsetSubpix * lengthSign;
    else posMy += pixelOffsetSubpix * lengthSign;
    float3 c = sample_rgb(t, posMx, posMy);
    return make_float4(c.x, c.y, c.z, lumaM);
}

// The prepared texel as RGBA16F bits: rgb as stored, the luma rounded to FP16
// in alpha (the temp image of antialias_fxaa_prepare.comp, which the FXAA pass
// copies for unmarked pixels).
__device__ __forceinline__ uint2 prepare_bits(uint2 t) {
    const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&t.x));
    const float b = __low2float(*reinterpret_cast<const __half2*>(&t.y));
    const float l = rg.x * 0.299f + rg.y * 0.587f + b * 0.114f;
    const __half lh = __float2half_rn(l);
    return make_uint2(t.x, (t.y & 0xffffu) | ((uint32_t)__half_as_ushort(lh) << 16));
}

__device__ __forceinline__ uint4 ld_stream(const void* p) {
    uint4 r;
    asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ void st_stream(void* p, uint4 v) {
    asm volatile("st.global.cs.v4.u32 [%0], {%1, %2, %3, %4};" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
                 : "memory");
}

constexpr int kBX = 32, kBY = 8;
#ifndef TAA_FXAA_MIN_BLOCKS
#define TAA_FXAA_MIN_BLOCKS 4  // resident CTAs per SM on the vector path (64 registers, no spills)
#endif

// One pixel as RGBA16F bits: the mask decides between FXAA and the prepared
// texel (antialias_fxaa.comp:39-62).
__device__ __forceinline__ uint2 pixel(const FxaaArgs& a, int x, int y, bool marked, uint2 bits) {
    if (!marked) return prepare_bits(bits);
    return float4_to_half4(
        fxaa_pixel(a.in.p, a.in.pitch, a.in.w, a.in.h, a.rcp_x, a.rcp_y, a.subpix, a.thr, a.thr_min, x, y));
}

// Scalar path: one pixel per thread, any texel-aligned pitch.
__global__ void __launch_bounds__(kBX * kBY) fxaa_kernel(const FxaaArgs a) {
    const int x = blockIdx.x * kBX + threadIdx.x, y = blockIdx.y * kBY + threadIdx.y;
    if (x >= a.in.w || y >= a.in.h) return;
    bool marked = true;
    if (a.seg.p) marked = (__ldg(texel_ptr<uint32_t>(a.seg, x, y)) & 3u) == 1u;
    const uint2 bits = __ldg(texel_ptr<uint2>(a.in, x, y));
    *texel_ptr_w<uint2>(a.out, x, y) = pixel(a, x, y, marked, bits);
}

// Vector path (16-byte aligned rows).
//
// fxaa_stream_kernel writes the prepared texel of every pixel: per warp a row
// segment of kTileW pixels in kPairs rounds of fully coalesced 16-byte
// accesses (lane l of round j moves pixels 2(32j + l) and 2(32j + l) + 1) that
// bypass L1.  It makes no calls and needs few registers, so many warps keep
// the memory system busy.  With a work list (LIST) it also reads the mask in
// the same rounds and appends the marked pixels to the list, one atomic per
// warp; fxaa_list_kernel then antialiases the listed pixels, 32 to a warp.
// Without a list, fxaa_marked_kernel reads the mask again, lists each warp's
// marked pixels in shared memory and antialiases them there.
//
// An edge search is a chain of dependent taps, about 1400 warp instructions
// for one pixel.  Inside a streaming kernel those chains met DRAM latency
// under full load and held warp slots; in a warp of their own segment they
// ran with one or two of 32 lanes busy.  Gathered into full warps after the
// stream they cost little.  Without a mask only the marked kernel runs, over
// every pixel.
constexpr int kPairs = 4;                  // pixel pairs per thread
constexpr int kTileW = 2 * kPairs * kBX;   // 256 pixels per warp row segment
constexpr int kListHead = 4;               // entry count, finished CTAs of the list kernel, 2 words padding
#ifndef TAA_FXAA_STREAM_MIN_BLOCKS
#define TAA_FXAA_STREAM_MIN_BLOCKS 8       // resident CTAs per SM of the streaming kernel (32 registers;
                                           // 6 and 40 registers with the list)
#endif

__device__ __forceinline__ uint2 ld_stream8(const void* p) {
    uint2 r;
    asm volatile("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "l"(p));
    return r;
}

// A warp's exclusive prefix of the lanes' counts n, and the warp total.
__device__ __forceinline__ int warp_prefix(int n, int lane, int* total) {
    int incl = n;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    *total = __shfl_sync(0xffffffffu, incl, 31);
    return incl - n;
}

template <bool LIST>
__global__ void __launch_bounds__(kBX * kBY, LIST ? TAA_FXAA_STREAM_MIN_BLOCKS - 2 : TAA_FXAA_STREAM_MIN_BLOCKS)
    fxaa_stream_kernel(const FxaaArgs a, uint32_t* list) {
    const int W = a.in.w, H = a.in.h;
    const int tx0 = blockIdx.x * kTileW;
    const int y = blockIdx.y * kBY + threadIdx.y;
    const int lane = threadIdx.x;
    if (y >= H) return;  // whole warps leave together
    uint4 t[kPairs];
    uint2 m[kPairs];
#pragma unroll
    for (int j = 0; j < kPairs; ++j) {
        const int x = tx0 + 2 * (j * kBX + lane);
        t[j] = make_uint4(0u, 0u, 0u, 0u);
        m[j] = make_uint2(0u, 0u);
        if (x + 1 < W) {
            t[j] = ld_stream(texel_ptr<uint2>(a.in, x, y));
            if (LIST) m[j] = ld_stream8(texel_ptr<uint32_t>(a.seg, x, y));
        } else if (x < W) {
            const uint2 b = __ldg(texel_ptr<uint2>(a.in, x, y));
            t[j] = make_uint4(b.x, b.y, 0u, 0u);
            if (LIST) m[j].x = __ldg(texel_ptr<uint32_t>(a.seg, x, y));
        }
    }
    uint32_t marked_bits = 0;  // bit 2j + k: pixel tx0 + 2(32j + lane) + k is marked
#pragma unroll
    for (int j = 0; j < kPairs; ++j) {
        const int x = tx0 + 2 * (j * kBX + lane);
        const uint2 o0 = prepare_bits(make_uint2(t[j].x, t[j].y)), o1 = prepare_bits(make_uint2(t[j].z, t[j].w));
        if (x + 1 < W) {
            st_stream(texel_ptr_w<uint2>(a.out, x, y), make_uint4(o0.x, o0.y, o1.x, o1.y));
            marked_bits |= (uint32_t)((m[j].x & 3u) == 1u) << (2 * j);
            marked_bits |= (uint32_t)((m[j].y & 3u) == 1u) << (2 * j + 1);
        } else if (x < W) {
            *texel_ptr_w<uint2>(a.out, x, y) = o0;
            marked_bits |= (uint32_t)((m[j].x & 3u) == 1u) << (2 * j);
        }
    }
    if (LIST) asm volatile("griddepcontrol.launch_dependents;");  // the list kernel may start launching
    if (!LIST || !__any_sync(0xffffffffu, marked_bits)) return;
    int total;
    int pos = warp_prefix(__popc(marked_bits), lane, &total);
    int base = 0;
    if (lane == 0) base = (int)atomicAdd(list, (uint32_t)total);
    pos += __shfl_sync(0xffffffffu, base, 0);
    uint32_t* entries = list + kListHead;
    for (uint32_t b = marked_bits; b; b &= b - 1) {
        const int bit = __ffs(b) - 1;
        const int x = tx0 + 2 * ((bit >> 1) * kBX + lane) + (bit & 1);
        entries[pos++] = (uint32_t)x | ((uint32_t)y << 16);
    }
}

// FXAA on the listed pixels (entries x | y << 16), grid-stride.  Launched as
// a programmatic dependent of the streaming kernel: its launch overlaps that
// kernel's tail and griddepcontrol.wait holds it until the list is complete.
// The last CTA to finish puts the list head back to zero for the next pass
// (every CTA has read the count before it counts itself finished).
__global__ void __launch_bounds__(kBX * kBY, TAA_FXAA_MIN_BLOCKS) fxaa_list_kernel(const FxaaArgs a,
                                                                                  uint32_t* list) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t n = *reinterpret_cast<volatile uint32_t*>(list);
    const uint32_t* entries = list + kListHead;
    for (uint32_t i = blockIdx.x * (kBX * kBY) + threadIdx.y * kBX + threadIdx.x; i < n;
         i += gridDim.x * (kBX * kBY)) {
        const uint32_t e = entries[i];
        const int x = (int)(e & 0xffffu), y = (int)(e >> 16);
        *texel_ptr_w<uint2>(a.out, x, y) = float4_to_half4(
            fxaa_pixel(a.in.p, a.in.pitch, a.in.w, a.in.h, a.rcp_x, a.rcp_y, a.subpix, a.thr, a.thr_min, x, y));
    }
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        if (atomicAdd(list + 1, 1u) == gridDim.x - 1) {
            list[0] = 0u;
            list[1] = 0u;
        }
    }
}

__global__ void __launch_bounds__(kBX * kBY, TAA_FXAA_MIN_BLOCKS) fxaa_marked_kernel(const FxaaArgs a) {
    __shared__ uint16_t s_list[kBY][kTileW];
    const int W = a.in.w, H = a.in.h;
    const int tx0 = blockIdx.x * kTileW;
    const int y = blockIdx.y * kBY + threadIdx.y;
    const int lane = threadIdx.x;
    if (y >= H) return;  // whole warps leave together
    uint2 m[kPairs];
#pragma unroll
    for (int j = 0; j < kPairs; ++j) {
        const int x = tx0 + 2 * (j * kBX + lane);
        m[j] = make_uint2(x < W ? 1u : 0u, x + 1 < W ? 1u : 0u);  // no mask: every pixel
        if (a.seg.p) {
            if (x + 1 < W) m[j] = ld_stream8(texel_ptr<uint32_t>(a.seg, x, y));
            else if (x < W) m[j].x = __ldg(texel_ptr<uint32_t>(a.seg, x, y));
        }
    }
    uint32_t marked_bits = 0;  // bit 2j + k: pixel tx0 + 2(32j + lane) + k is marked
#pragma unroll
    for (int j = 0; j < kPairs; ++j) {
        marked_bits |= (uint32_t)((m[j].x & 3u) == 1u) << (2 * j);
        marked_bits |= (uint32_t)((m[j].y & 3u) == 1u) << (2 * j + 1);
    }
    if (!__any_sync(0xffffffffu, marked_bits)) return;
    int total;
    int pos = warp_prefix(__popc(marked_bits), lane, &total);
    uint16_t* list = s_list[threadIdx.y];
    for (uint32_t b = marked_bits; b; b &= b - 1) {
        const int bit = __ffs(b) - 1;
        list[pos++] = (uint16_t)(2 * ((bit >> 1) * kBX + lane) + (bit & 1));
    }
    __syncwarp();
    for (int i = lane; i < total; i += kBX) {
        const int x = tx0 + list[i];
        *texel_ptr_w<uint2>(a.out, x, y) = float4_to_half4(
            fxaa_pixel(a.in.p, a.in.pitch, W, H, a.rcp_x, a.rcp_y, a.subpix, a.thr, a.thr_min, x, y));
    }
}

bool aligned16(const void* p, size_t pitch) { return ((uintptr_t)p % 16 == 0) && (pitch % 16 == 0); }

// CTAs of the list kernel: the SMs x its resident CTAs on the current device
// (looked up once per device, so that later calls, e.g. under stream capture,
// only launch)
unsigned list_ctas() {
    constexpr int kMaxDevices = 64;
    static unsigned cached[kMaxDevices] = {};
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
    if (dev < kMaxDevices && cached[dev]) return cached[dev];
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fxaa_list_kernel, kBX * kBY, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const unsigned n = (unsigned)(sms * per_sm);
    if (dev < kMaxDevices) cached[dev] = n;
    return n;
}

}  // namespace

cudaError_t launch_fxaa(const Img& in, const Img& segmask, const ImgW& out, const float rcp[2], float subpix,
                        float edge_threshold, float edge_threshold_min, uint32_t* list, cudaStream_t s) {
    FxaaArgs a{in, segmask, out, rcp[0], rcp[1], subpix, edge_threshold, edge_threshold_min};
    const bool vec = aligned16(in.p, in.pitch) && aligned16(out.p, out.pitch) &&
                     (!segmask.p || aligned16(segmask.p, segmask.pitch));
    dim3 block(kBX, kBY);
    if (vec) {
        dim3 grid((in.w + kTileW - 1) / kTileW, (in.h + kBY - 1) / kBY);
        if (segmask.p && list) {
            fxaa_stream_kernel<true><<<grid, block, 0, s>>>(a, list);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(list_ctas());
            cfg.blockDim = block;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            return cudaLaunchKernelEx(&cfg, fxaa_list_kernel, a, list);
        } else if (segmask.p) {
            fxaa_stream_kernel<false><<<grid, block, 0, s>>>(a, nullptr);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
            fxaa_marked_kernel<<<grid, block, 0, s>>>(a);
        } else {
            fxaa_marked_kernel<<<grid, block, 0, s>>>(a);
        }
    } else {
        dim3 grid((in.w + kBX - 1) / kBX, (in.h + kBY - 1) / kBY);
        fxaa_kernel<<<grid, block, 0, s>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace taa_dev
