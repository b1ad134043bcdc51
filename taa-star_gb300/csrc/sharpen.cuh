// sharpen.cuh - the two sharpeners of the reference, per pixel.
#pragma once
#include "common.cuh"

namespace taa_dev {

// Every product and sum below is a separately rounded __fmul_rn / __fadd_rn
// (which the compiler never contracts), so the sharpeners give the shader's
// FP32 bits in any translation unit, with or without -fmad=false.

// ffx_a.h:1455-1457 (defined on FP32 bit patterns).
__device__ __forceinline__ float prx_lo_sqrt(float a) { return __uint_as_float((__float_as_uint(a) >> 1) + 0x1fbc4639u); }
__device__ __forceinline__ float prx_lo_rcp(float a) { return __uint_as_float(0x7ef07ebbu - __float_as_uint(a)); }
__device__ __forceinline__ float prx_med_rcp(float a) {
    float b = __uint_as_float(0x7ef19fffu - __float_as_uint(a));
    return __fmul_rn(b, __fadd_rn(__fmul_rn(-b, a), 2.0f));
}
__device__ __forceinline__ float sat(float x) { return gmin(gmax(x, 0.0f), 1.0f); }

// b * w + d * w + f * w + h * w + e, left to right, every operation rounded.
__device__ __forceinline__ float cas_sum(float b, float d, float f, float h, float e, float w) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(b, w), __fmul_rn(d, w)), __fmul_rn(f, w)), __fmul_rn(h, w)),
                     e);
}

// CasFilter, no-scaling branch, green-coefficient filter (ffx_cas.h:424-537):
// b/d/e/f/h are the cross neighbourhood (north, west, centre, east, south).
__device__ __forceinline__ float3 cas_pixel(float3 b, float3 d, float3 e, float3 f, float3 h, float peak) {
    float mnG = gmin(gmin(d.y, gmin(e.y, f.y)), gmin(b.y, h.y));
    float mxG = gmax(gmax(d.y, gmax(e.y, f.y)), gmax(b.y, h.y));
    float ampG = sat(__fmul_rn(gmin(mnG, __fsub_rn(1.0f, mxG)), prx_lo_rcp(mxG)));
    ampG = prx_lo_sqrt(ampG);
    float wG = __fmul_rn(ampG, peak);
    float rw = prx_med_rcp(__fadd_rn(1.0f, __fmul_rn(4.0f, wG)));
    return make_float3(sat(__fmul_rn(cas_sum(b.x, d.x, f.x, h.x, e.x, wG), rw)),
                       sat(__fmul_rn(cas_sum(b.y, d.y, f.y, h.y, e.y, wG), rw)),
                       sat(__fmul_rn(cas_sum(b.z, d.z, f.z, h.z, e.z, wG), rw)));
}

// shaders/sharpen.comp:24-38 (left, right, top, bottom, centre).
__device__ __forceinline__ float simple_sharpen_channel(float l, float r, float t, float b, float c, float k) {
    const float lap = __fsub_rn(__fsub_rn(__fsub_rn(__fsub_rn(__fmul_rn(4.0f, c), l), r), t), b);
    return gclamp(__fadd_rn(c, __fmul_rn(lap, k)), 0.f, 1.f);
}
__device__ __forceinline__ float3 simple_sharpen_pixel(float3 l, float3 r, float3 t, float3 b, float3 c, float k) {
    return make_float3(simple_sharpen_channel(l.x, r.x, t.x, b.x, c.x, k),
                       simple_sharpen_channel(l.y, r.y, t.y, b.y, c.y, k),
                       simple_sharpen_channel(l.z, r.z, t.z, b.z, c.z, k));
}

}  // namespace taa_dev
