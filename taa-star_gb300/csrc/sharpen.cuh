// sharpen.cuh - the two sharpeners of the reference, per pixel.
#pragma once
#include "common.cuh"

namespace taa_dev {

// ffx_a.h:1455-1457 (defined on FP32 bit patterns).
__device__ __forceinline__ float prx_lo_sqrt(float a) { return __uint_as_float((__float_as_uint(a) >> 1) + 0x1fbc4639u); }
__device__ __forceinline__ float prx_lo_rcp(float a) { return __uint_as_float(0x7ef07ebbu - __float_as_uint(a)); }
__device__ __forceinline__ float prx_med_rcp(float a) {
    float b = __uint_as_float(0x7ef19fffu - __float_as_uint(a));
    return b * (-b * a + 2.0f);
}
__device__ __forceinline__ float sat(float x) { return gmin(gmax(x, 0.0f), 1.0f); }

// CasFilter, no-scaling branch, green-coefficient filter (ffx_cas.h:424-537):
// b/d/e/f/h are the cross neighbourhood (north, west, centre, east, south).
__device__ __forceinline__ float3 cas_pixel(float3 b, float3 d, float3 e, float3 f, float3 h, float peak) {
    float mnG = gmin(gmin(d.y, gmin(e.y, f.y)), gmin(b.y, h.y));
    float mxG = gmax(gmax(d.y, gmax(e.y, f.y)), gmax(b.y, h.y));
    float ampG = sat(gmin(mnG, 1.0f - mxG) * prx_lo_rcp(mxG));
    ampG = prx_lo_sqrt(ampG);
    float wG = ampG * peak;
    float rw = prx_med_rcp(1.0f + 4.0f * wG);
    return make_float3(sat((b.x * wG + d.x * wG + f.x * wG + h.x * wG + e.x) * rw),
                       sat((b.y * wG + d.y * wG + f.y * wG + h.y * wG + e.y) * rw),
                       sat((b.z * wG + d.z * wG + f.z * wG + h.z * wG + e.z) * rw));
}

// shaders/sharpen.comp:24-38 (left, right, top, bottom, centre).
__device__ __forceinline__ float3 simple_sharpen_pixel(float3 l, float3 r, float3 t, float3 b, float3 c, float k) {
    float3 v;
    v.x = c.x + (4.0f * c.x - l.x - r.x - t.x - b.x) * k;
    v.y = c.y + (4.0f * c.y - l.y - r.y - t.y - b.y) * k;
    v.z = c.z + (4.0f * c.z - l.z - r.z - t.z - b.z) * k;
    return make_float3(gclamp(v.x, 0.f, 1.f), gclamp(v.y, 0.f, 1.f), gclamp(v.z, 0.f, 1.f));
}

}  // namespace taa_dev
