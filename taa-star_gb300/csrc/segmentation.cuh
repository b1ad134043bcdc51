// segmentation.cuh - the ray-trace-assist classification of a pixel
// (taa.comp:558-702, calc_segmentation_value), shared by the plain form and
// the tiled forms so that both give the same mask.
//
// The class sits in bits 0-1 (0 keep the TAA result, 1 antialias with FXAA, 2
// ray trace), a history count in bits 16 and up.  Tests in flag order: a
// fixed-width border for FXAA (FXD), everything ray traced (ALL), history
// position off screen (OUT), disocclusion by a mover (DIS), then a weighted sum
// of four edge measures against the threshold - normals (NRM), the Sobel
// magnitude of view-space depth (DPT), a material change (MID), the Sobel
// magnitude of luma (LUM) - and at last the decaying history count (CNT).
//
// The neighbourhood comes through an accessor: material(x, y), normal(x, y),
// lin_depth(x, y) and luma(x, y) at edge-clamped coordinates of the source
// image (the plain form reads global memory, the tiled forms a staged tile),
// prev_material(x, y) and prev_segmask(x, y) at coordinates in range.
// Compiled with -fmad=false like its callers.
#pragma once
#include "common.cuh"

namespace taa_dev {
namespace seg {

struct N3 {
    float x, y, z;
};

// the unit normal of an (azimuth, elevation) pair (.z, .w of the uv/normal image)
__device__ __forceinline__ N3 normal_from(float az, float el) {
    return {cosf(az) * cosf(el), sinf(az) * cosf(el), sinf(el)};
}
// view-space depth of a [0, 1] depth buffer value, near n, far f
__device__ __forceinline__ float lin_depth(float d, float n, float f) { return n * f / (f + d * (n - f)); }
// Y of YCoCg from RGB
__device__ __forceinline__ float luma(float r, float g, float b) { return .25f * r + .5f * g + .25f * b; }

__device__ __forceinline__ float sobel_magnitude(float c00, float c01, float c02, float c10, float c12, float c20,
                                                 float c21, float c22) {
    const float gx = c00 - c20 + 2.0f * c01 - 2.0f * c21 + c02 - c22;
    const float gy = c00 - c02 + 2.0f * c10 - 2.0f * c12 + c20 - c22;
    return sqrtf(gx * gx + gy * gy);
}

template <class Acc>
__device__ __forceinline__ uint32_t classify(const taa_parameters_t& P, int ix, int iy, float hux, float huy, int loW,
                                             int loH, const Acc& acc) {
    const uint32_t fl = P.mRayTraceAugmentFlags;
    auto cx = [&](int v) { return clampi(v, 0, loW - 1); };
    auto cy = [&](int v) { return clampi(v, 0, loH - 1); };
    if (fl & TAA_RTFLAG_FXD) {
        const int b = 100;
        if (ix < b || iy < b || ix >= loW - b || iy >= loH - b) return 1u;
    }
    if (fl & TAA_RTFLAG_ALL) return 2u;
    const bool cnt = (fl & TAA_RTFLAG_CNT) != 0;
    const uint32_t newc = cnt ? ((uint32_t)P.mRayTraceHistoryCount << 16) : 0u;
    if (fl & TAA_RTFLAG_OUT) {
        if (hux < 0.f || huy < 0.f || hux >= 1.f || huy >= 1.f) return 1u;
    }
    const uint32_t mat = acc.material(ix, iy);
    if (fl & TAA_RTFLAG_DIS) {
        const int tx = trunc_index(hux * (float)loW), ty = trunc_index(huy * (float)loH);
        if (tx >= 0 && ty >= 0 && tx < loW && ty < loH) {
            const uint32_t pm = acc.prev_material(tx, ty);
            if (pm != mat && (pm & 0x80000000u) != 0) return 2u | newc;
        }
    }
    float nv = 0.f, dv = 0.f, mv = 0.f, lv = 0.f;
    if (fl & TAA_RTFLAG_NRM) {
        const N3 nC = acc.normal(ix, iy), nL = acc.normal(cx(ix - 1), cy(iy)), nR = acc.normal(cx(ix + 1), cy(iy));
        const N3 nT = acc.normal(cx(ix), cy(iy - 1)), nB = acc.normal(cx(ix), cy(iy + 1));
        auto d3 = [](N3 p, N3 q) { return p.x * q.x + p.y * q.y + p.z * q.z; };
        const float m = gmax(0.f, gmin(gmin(gmin(d3(nC, nL), d3(nC, nR)), d3(nC, nT)), d3(nC, nB)));
        nv = 1.0f - m;
    }
    if (fl & TAA_RTFLAG_DPT) {
        auto L = [&](int dx, int dy) { return acc.lin_depth(cx(ix + dx), cy(iy + dy)); };
        dv = sobel_magnitude(L(-1, -1), L(0, -1), L(1, -1), L(-1, 0), L(1, 0), L(-1, 1), L(0, 1), L(1, 1));
    }
    if (fl & TAA_RTFLAG_MID) {
        if (mat != acc.material(cx(ix - 1), cy(iy)) || mat != acc.material(cx(ix + 1), cy(iy)) ||
            mat != acc.material(cx(ix), cy(iy - 1)) || mat != acc.material(cx(ix), cy(iy + 1)))
            mv = 1.0f;
    }
    if (fl & TAA_RTFLAG_LUM) {
        auto L = [&](int dx, int dy) { return acc.luma(cx(ix + dx), cy(iy + dy)); };
        lv = sobel_magnitude(L(-1, -1), L(0, -1), L(1, -1), L(-1, 0), L(1, 0), L(-1, 1), L(0, 1), L(1, 1));
    }
    const float total =
        nv * P.mRayTraceAugment_WNrm + dv * P.mRayTraceAugment_WDpt + mv * P.mRayTraceAugment_WMId + lv * P.mRayTraceAugment_WLum;
    if (total >= P.mRayTraceAugment_Thresh) return 2u | newc;
    if (cnt) {
        const uint32_t old = (acc.prev_segmask(ix, iy) & 0xffff0000u) >> 16;
        if (old > 0) return 2u | ((old - 1) << 16);
    }
    return 0u;
}

}  // namespace seg
}  // namespace taa_dev
