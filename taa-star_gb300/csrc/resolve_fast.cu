// resolve_fast.cu - the sharpen pass of source/taa.hpp:1111-1139 that runs
// after a resolve (and as taa_sharpen), and the one-launch resolve + sharpen
// of the tiled FP32 form (TAA_FLAG_FUSED_SHARPEN).
//
// The one-launch kernel: one CTA owns a BX x BY tile of output pixels.  It
// stages the source colour
// of the tile plus a 1-pixel halo (plus a further pixel when a sharpener is
// fused) in shared memory, converted once per texel to the working colour
// space (tonemap + YCoCg, taa.comp:182-213), and every thread then reads its
// 3x3 neighbourhood from shared memory.  The history gather (16-tap
// Catmull-Rom or bilinear, taa.comp:441-549) goes through the L1 cache.  With
// a fused sharpener the CTA also resolves the 1-pixel ring around its tile
// (recomputing what the neighbour CTA computes, bit for bit), keeps the
// FP16-rounded screen colour of tile+ring in shared memory and applies CAS or
// the simple sharpener to the tile from there, so the unsharpened image never
// goes to HBM.
//
// This translation unit is compiled with -fmad=false: every operation rounds
// as the FP32 oracle's does, with fused multiply-adds only where the oracle
// has them (moments, Catmull-Rom accumulation) or where fusing provably
// cannot change a result (products by powers of two), so the tiled form gives
// the oracle's bits.
#include "common.cuh"
#include "sharpen.cuh"
#include "kernels.h"
#include "../../include/taa_gb300.h"

namespace taa_dev {

bool fast_path_supported(const taa_uniforms_t& U, int in_w, int in_h, int out_w, int out_h, bool rt_augment_ok,
                         bool extra_modes_ok) {
    if (in_w != out_w || in_h != out_h) return false;
    if (U.mUpsampling || U.mBypassHistoryUpdate) return false;
    if (U.splitScreen && U.splitX < out_w - 1) return false;
    const taa_parameters_t& P = U.param[0];
    if (P.mPassThrough || (P.mRayTraceAugment && !rt_augment_ok)) return false;
    if (!extra_modes_ok && (P.mAddNoise || P.mDynamicAntiGhosting || P.mVelocitySampleMode == 1)) return false;
    bool jitter_zero = U.mJitterNdc[0] * 0.5f * P.mUnjitterFactor == 0.f &&
                       U.mJitterNdc[1] * 0.5f * P.mUnjitterFactor == 0.f;
    if ((P.mUnjitterNeighbourhood || P.mUnjitterCurrentSample) && !jitter_zero) return false;
    if (P.mInterpolationMode < 0 || P.mInterpolationMode > 2) return false;
    return true;
}

bool up_path_supported(const taa_uniforms_t& U, int in_w, int in_h, int out_w, int out_h) {
    if (!U.mUpsampling || in_w > out_w || in_h > out_h || (in_w == out_w && in_h == out_h)) return false;
    if (U.mBypassHistoryUpdate || (U.splitScreen && U.splitX < out_w - 1)) return false;
    const taa_parameters_t& P = U.param[0];
    if (P.mPassThrough || P.mRayTraceAugment || P.mDynamicAntiGhosting || P.mVelocitySampleMode != 0) return false;
    if (P.mInterpolationMode < 0 || P.mInterpolationMode > 2) return false;
    const bool jitter_zero = U.mJitterNdc[0] * 0.5f * P.mUnjitterFactor == 0.f &&
                             U.mJitterNdc[1] * 0.5f * P.mUnjitterFactor == 0.f;
    return !P.mUnjitterNeighbourhood || jitter_zero;
}

namespace {

constexpr int kTileX = 32;

struct C3 { float x, y, z; };
__device__ __forceinline__ C3 c3(float4 v) { return {v.x, v.y, v.z}; }

// Working-space conversion of one source texel (taa.comp:204).
__device__ __forceinline__ float4 to_working(float4 c, bool tonemap, bool ycocg) {
    if (tonemap) {
        float l = 1.0f + gmax(gmax(c.x, c.y), c.z);
        c.x = c.x / l;
        c.y = c.y / l;
        c.z = c.z / l;
    }
    if (ycocg) {
        // the products by powers of two are exact, so a fused form rounds like
        // the separate multiply and add of the oracle
        float y = __fmaf_rn(.25f, c.z, __fmaf_rn(.25f, c.x, .5f * c.y));
        float co = __fmaf_rn(-.5f, c.z, .5f * c.x);
        float cg = __fmaf_rn(-.25f, c.z, __fmaf_rn(-.25f, c.x, .5f * c.y));
        return make_float4(y, co, cg, 0.f);
    }
    return make_float4(c.x, c.y, c.z, 0.f);
}

// History sample in the oracle's FP32 order (the Catmull-Rom accumulation is
// its fused multiply-add chain).  The alpha channel carries the dynamic
// anti-ghosting mask, which these forms do not read.
template <int INTERP, int HF, bool WANT_ALPHA = false>
__device__ __forceinline__ float4 sample_history(const Img& h, float u, float v) {
    if (INTERP == 2) {
        // 16-tap Catmull-Rom, separable rows (taa.comp:441-514)
        float itx = u * (float)h.w, ity = v * (float)h.h;
        float bx = floorf(itx - 0.5f), by = floorf(ity - 0.5f);
        float fx = itx - (bx + 0.5f), fy = ity - (by + 0.5f);
        float wx[4], wy[4];
        {
            float f2 = fx * fx, f3 = f2 * fx;
            wx[0] = -0.5f * f3 + f2 - 0.5f * fx;
            wx[1] = 1.5f * f3 - 2.5f * f2 + 1.0f;
            wx[2] = -1.5f * f3 + 2.0f * f2 + 0.5f * fx;
            wx[3] = 0.5f * f3 - 0.5f * f2;
        }
        {
            float f2 = fy * fy, f3 = f2 * fy;
            wy[0] = -0.5f * f3 + f2 - 0.5f * fy;
            wy[1] = 1.5f * f3 - 2.5f * f2 + 1.0f;
            wy[2] = -1.5f * f3 + 2.0f * f2 + 0.5f * fy;
            wy[3] = 0.5f * f3 - 0.5f * f2;
        }
        int kx = trunc_index(bx), ky = trunc_index(by);
        int xs[4], ys[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            xs[i] = clampi(kx - 1 + i, 0, h.w - 1);
            ys[i] = clampi(ky - 1 + i, 0, h.h - 1);
        }
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!h.p) return acc;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const char* rowp = h.p + (size_t)ys[j] * h.pitch;
            float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                float4 s;
                if (HF == 0) s = __ldg(reinterpret_cast<const float4*>(rowp) + xs[i]);
                else s = half4_to_float4(__ldg(reinterpret_cast<const uint2*>(rowp) + xs[i]));
                r.x = __fmaf_rn(wx[i], s.x, r.x);
                r.y = __fmaf_rn(wx[i], s.y, r.y);
                r.z = __fmaf_rn(wx[i], s.z, r.z);
                if (WANT_ALPHA) r.w = __fmaf_rn(wx[i], s.w, r.w);
            }
            acc.x = __fmaf_rn(wy[j], r.x, acc.x);
            acc.y = __fmaf_rn(wy[j], r.y, acc.y);
            acc.z = __fmaf_rn(wy[j], r.z, acc.z);
            if (WANT_ALPHA) acc.w = __fmaf_rn(wy[j], r.w, acc.w);
        }
        return acc;
    } else {
        // exact-weight bilinear (taa.comp:546); the "b-spline" mode takes four of these
        auto bil = [&](float uu, float vv) {
            float px = uu * (float)h.w - 0.5f, py = vv * (float)h.h - 0.5f;
            float fx0 = floorf(px), fy0 = floorf(py);
            float fx = px - fx0, fy = py - fy0;
            if (!(fx == fx)) fx = 0.f;
            if (!(fy == fy)) fy = 0.f;
            int x0 = trunc_index(fx0), y0 = trunc_index(fy0);
            int xa = clampi(x0, 0, h.w - 1), xb = clampi(x0 + 1 < x0 ? x0 : x0 + 1, 0, h.w - 1);
            int ya = clampi(y0, 0, h.h - 1), yb = clampi(y0 + 1 < y0 ? y0 : y0 + 1, 0, h.h - 1);
            float4 A = fetch_history<HF>(h, xa, ya), B = fetch_history<HF>(h, xb, ya);
            float4 C = fetch_history<HF>(h, xa, yb), D = fetch_history<HF>(h, xb, yb);
            float gx = 1.0f - fx, gy = 1.0f - fy;
            float4 t = make_float4(A.x * gx + B.x * fx, A.y * gx + B.y * fx, A.z * gx + B.z * fx, A.w * gx + B.w * fx);
            float4 b = make_float4(C.x * gx + D.x * fx, C.y * gx + D.y * fx, C.z * gx + D.z * fx, C.w * gx + D.w * fx);
            return make_float4(t.x * gy + b.x * fy, t.y * gy + b.y * fy, t.z * gy + b.z * fy, t.w * gy + b.w * fy);
        };
        if (INTERP == 0) return bil(u, v);
        // taa.comp:517-543
        float it[2] = {u * (float)h.w, v * (float)h.h};
        float inv[2] = {1.0f / (float)h.w, 1.0f / (float)h.h};
        float s0[2], s1[2], t0[2], t1[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            float tc = floorf(it[k] - 0.5f) + 0.5f;
            float f = it[k] - tc, f2 = f * f, f3 = f2 * f;
            float w0 = f2 - 0.5f * (f3 + f);
            float w1 = 1.5f * f3 - 2.5f * f2 + 1.0f;
            float w3 = 0.5f * (f3 - f2);
            float w2 = 1.0f - w0 - w1 - w3;
            s0[k] = w0 + w1;
            s1[k] = w2 + w3;
            t0[k] = (tc - 1.0f + w1 / (w0 + w1)) * inv[k];
            t1[k] = (tc + 1.0f + w3 / (w2 + w3)) * inv[k];
        }
        float4 A = bil(t0[0], t0[1]), B = bil(t1[0], t0[1]), C = bil(t0[0], t1[1]), D = bil(t1[0], t1[1]);
        return make_float4((A.x * s0[0] + B.x * s1[0]) * s0[1] + (C.x * s0[0] + D.x * s1[0]) * s1[1],
                           (A.y * s0[0] + B.y * s1[0]) * s0[1] + (C.y * s0[0] + D.y * s1[0]) * s1[1],
                           (A.z * s0[0] + B.z * s1[0]) * s0[1] + (C.z * s0[0] + D.z * s1[0]) * s1[1],
                           (A.w * s0[0] + B.w * s1[0]) * s0[1] + (C.w * s0[0] + D.w * s1[0]) * s1[1]);
    }
}

// Resolve of one pixel from the staged neighbourhood.  `nb` points at the
// centre texel in the staging array of row stride `ns`.
template <int HF, int MC, int INTERP>
__device__ __forceinline__ void resolve_pixel(const taa_uniforms_t& U, const taa_parameters_t& P, const FrameArgs& a,
                                              int x, int y, const float4* nb, int ns, float4& to_hist,
                                              float4& to_screen) {
    const float N = 9.0f, rN = 1.0f / 9.0f;
    C3 c0 = c3(nb[0]);
    C3 c1 = c3(nb[-ns - 1]), c2 = c3(nb[-ns]), c3_ = c3(nb[-ns + 1]);
    C3 c4 = c3(nb[-1]), c5 = c3(nb[1]);
    C3 c6 = c3(nb[ns - 1]), c7 = c3(nb[ns]), c8 = c3(nb[ns + 1]);
    C3 mn, mx, ct = c0;  // ct: clip-towards colour (the mean for variance clipping)
    if (P.mVarianceClipping) {
        C3 m1{c0.x + c1.x + c2.x + c3_.x + c4.x + c5.x + c6.x + c7.x + c8.x,
              c0.y + c1.y + c2.y + c3_.y + c4.y + c5.y + c6.y + c7.y + c8.y,
              c0.z + c1.z + c2.z + c3_.z + c4.z + c5.z + c6.z + c7.z + c8.z};
        auto sq = [&](float p0, float p1, float p2, float p3, float p4, float p5, float p6, float p7, float p8) {
            float m = __fmul_rn(p0, p0);
            m = __fmaf_rn(p1, p1, m); m = __fmaf_rn(p2, p2, m); m = __fmaf_rn(p3, p3, m);
            m = __fmaf_rn(p4, p4, m); m = __fmaf_rn(p5, p5, m); m = __fmaf_rn(p6, p6, m);
            m = __fmaf_rn(p7, p7, m); m = __fmaf_rn(p8, p8, m);
            return m;
        };
        C3 m2{sq(c0.x, c1.x, c2.x, c3_.x, c4.x, c5.x, c6.x, c7.x, c8.x),
              sq(c0.y, c1.y, c2.y, c3_.y, c4.y, c5.y, c6.y, c7.y, c8.y),
              sq(c0.z, c1.z, c2.z, c3_.z, c4.z, c5.z, c6.z, c7.z, c8.z)};
        C3 mean{div_const_rn(m1.x, N, rN), div_const_rn(m1.y, N, rN), div_const_rn(m1.z, N, rN)};
        float vx = __fmaf_rn(-mean.x, mean.x, div_const_rn(m2.x, N, rN));
        float vy = __fmaf_rn(-mean.y, mean.y, div_const_rn(m2.y, N, rN));
        float vz = __fmaf_rn(-mean.z, mean.z, div_const_rn(m2.z, N, rN));
        float g = P.mVarClipGamma;
        float sx = g * sqrtf(gmax(0.f, vx)), sy = g * sqrtf(gmax(0.f, vy)), sz = g * sqrtf(gmax(0.f, vz));
        mn = {mean.x - sx, mean.y - sy, mean.z - sz};
        mx = {mean.x + sx, mean.y + sy, mean.z + sz};
        ct = mean;
    } else if (P.mShapedNeighbourhood) {
        auto mn9 = [](float a0, float a1, float a2, float a3, float a4, float a5, float a6, float a7, float a8) {
            return gmin(gmin(gmin(gmin(gmin(gmin(gmin(gmin(a0, a1), a2), a3), a4), a5), a6), a7), a8);
        };
        auto mx9 = [](float a0, float a1, float a2, float a3, float a4, float a5, float a6, float a7, float a8) {
            return gmax(gmax(gmax(gmax(gmax(gmax(gmax(gmax(a0, a1), a2), a3), a4), a5), a6), a7), a8);
        };
        auto mn5 = [](float a0, float a2, float a4, float a5, float a7) { return gmin(gmin(gmin(gmin(a0, a2), a4), a5), a7); };
        auto mx5 = [](float a0, float a2, float a4, float a5, float a7) { return gmax(gmax(gmax(gmax(a0, a2), a4), a5), a7); };
        mn = {(mn9(c0.x, c1.x, c2.x, c3_.x, c4.x, c5.x, c6.x, c7.x, c8.x) + mn5(c0.x, c2.x, c4.x, c5.x, c7.x)) * 0.5f,
              (mn9(c0.y, c1.y, c2.y, c3_.y, c4.y, c5.y, c6.y, c7.y, c8.y) + mn5(c0.y, c2.y, c4.y, c5.y, c7.y)) * 0.5f,
              (mn9(c0.z, c1.z, c2.z, c3_.z, c4.z, c5.z, c6.z, c7.z, c8.z) + mn5(c0.z, c2.z, c4.z, c5.z, c7.z)) * 0.5f};
        mx = {(mx9(c0.x, c1.x, c2.x, c3_.x, c4.x, c5.x, c6.x, c7.x, c8.x) + mx5(c0.x, c2.x, c4.x, c5.x, c7.x)) * 0.5f,
              (mx9(c0.y, c1.y, c2.y, c3_.y, c4.y, c5.y, c6.y, c7.y, c8.y) + mx5(c0.y, c2.y, c4.y, c5.y, c7.y)) * 0.5f,
              (mx9(c0.z, c1.z, c2.z, c3_.z, c4.z, c5.z, c6.z, c7.z, c8.z) + mx5(c0.z, c2.z, c4.z, c5.z, c7.z)) * 0.5f};
    } else {
        mn = {gmin(gmin(gmin(gmin(gmin(gmin(gmin(gmin(c0.x, c1.x), c2.x), c3_.x), c4.x), c5.x), c6.x), c7.x), c8.x),
              gmin(gmin(gmin(gmin(gmin(gmin(gmin(gmin(c0.y, c1.y), c2.y), c3_.y), c4.y), c5.y), c6.y), c7.y), c8.y),
              gmin(gmin(gmin(gmin(gmin(gmin(gmin(gmin(c0.z, c1.z), c2.z), c3_.z), c4.z), c5.z), c6.z), c7.z), c8.z)};
        mx = {gmax(gmax(gmax(gmax(gmax(gmax(gmax(gmax(c0.x, c1.x), c2.x), c3_.x), c4.x), c5.x), c6.x), c7.x), c8.x),
              gmax(gmax(gmax(gmax(gmax(gmax(gmax(gmax(c0.y, c1.y), c2.y), c3_.y), c4.y), c5.y), c6.y), c7.y), c8.y),
              gmax(gmax(gmax(gmax(gmax(gmax(gmax(gmax(c0.z, c1.z), c2.z), c3_.z), c4.z), c5.z), c6.z), c7.z), c8.z)};
    }
    if (P.mUseYCoCg && P.mShrinkChromaAxis) {
        C3 hs{0.5f * (mx.x - mn.x), 0.25f * (mx.y - mn.y), 0.25f * (mx.z - mn.z)};
        C3 ce{(mn.x + mx.x) * 0.5f, (mn.y + mx.y) * 0.5f, (mn.z + mx.z) * 0.5f};
        mn = {ce.x - hs.x, ce.y - hs.y, ce.z - hs.z};
        mx = {ce.x + hs.x, ce.y + hs.y, ce.z + hs.z};
        if (ct.x < mn.x || ct.y < mn.y || ct.z < mn.z || ct.x > mx.x || ct.y > mx.y || ct.z > mx.z) ct = ce;
    }

    // history position (taa.comp:391-438); uv = (x + 0.5) / size correctly rounded
    float u = div_const_rn((float)x + 0.5f, (float)a.out_w, a.inv_out_w);
    float v = div_const_rn((float)y + 0.5f, (float)a.out_h, a.inv_out_h);
    float depth = __ldg(texel_ptr<float>(a.depth, x, y));
    float4 vs = fetch_velocity<MC>(a.velocity, x, y);
    float hu, hv, ehd;
    bool can = !(P.mUseVelocityVectors == 0 || (P.mUseVelocityVectors == 1 && vs.w < 0.5f));
    if (can) {
        if (P.mVelocitySampleMode == 2) {
            int best_dx = -1, best_dy = -1;
            float dc = fetch_r32f(a.depth, x - 1, y - 1);
#pragma unroll
            for (int k = 1; k < 9; ++k) {
                int dx = k % 3 - 1, dy = k / 3 - 1;
                float d = fetch_r32f(a.depth, x + dx, y + dy);
                if (d < dc) { best_dx = dx; best_dy = dy; dc = d; }
            }
            vs = fetch_velocity<MC>(a.velocity, x + best_dx, y + best_dy);
        }
        hu = u - vs.x;
        hv = v - vs.y;
        ehd = depth - vs.z;
    } else {
        float cs0 = u * 2.0f - 1.0f, cs1 = v * 2.0f - 1.0f;
        const float* A = U.mInverseViewProjMatrix;
        const float* B = U.mHistoryViewProjMatrix;
        float ws[4], hs[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) ws[i] = A[i] * cs0 + A[4 + i] * cs1 + A[8 + i] * depth + A[12 + i];
#pragma unroll
        for (int i = 0; i < 4; ++i) hs[i] = B[i] * ws[0] + B[4 + i] * ws[1] + B[8 + i] * ws[2] + B[12 + i] * ws[3];
        hu = (hs[0] / hs[3]) * 0.5f + 0.5f;
        hv = (hs[1] / hs[3]) * 0.5f + 0.5f;
        ehd = hs[2] / hs[3];
    }

    float4 hraw = sample_history<INTERP, HF>(a.history, hu, hv);
    C3 hc{hraw.x, hraw.y, hraw.z};
    if (P.mUseYCoCg) {
        hc = {.25f * hraw.x + .5f * hraw.y + .25f * hraw.z, .5f * hraw.x - .5f * hraw.z,
              -.25f * hraw.x + .5f * hraw.y - .25f * hraw.z};
    }

    bool rejected = false;
    if (P.mRejectOutside && (hu < 0.f || hv < 0.f || hu >= 1.f || hv >= 1.f)) rejected = true;
    if (P.mDepthCulling) {
        int tx = clampi(trunc_index(hu * (float)a.color.w), 0, a.color.w - 1);
        int ty = clampi(trunc_index(hv * (float)a.color.h), 0, a.color.h - 1);
        float hd = a.history_depth.p ? __ldg(texel_ptr<float>(a.history_depth, tx, ty)) : 0.f;
        if (fabsf(hd - ehd) > 0.1f * (1.0f - hd)) rejected = true;
    }

    C3 orig = hc;
    switch (P.mColorClampingOrClipping) {
        case 1:
            hc = {gmin(gmax(hc.x, mn.x), mx.x), gmin(gmax(hc.y, mn.y), mx.y), gmin(gmax(hc.z, mn.z), mx.z)};
            break;
        case 2: {
            C3 p{0.5f * (mx.x + mn.x), 0.5f * (mx.y + mn.y), 0.5f * (mx.z + mn.z)};
            C3 e{0.5f * (mx.x - mn.x) + 1e-7f, 0.5f * (mx.y - mn.y) + 1e-7f, 0.5f * (mx.z - mn.z) + 1e-7f};
            C3 d{hc.x - p.x, hc.y - p.y, hc.z - p.z};
            float ma = gmax(fabsf(d.x / e.x), gmax(fabsf(d.y / e.y), fabsf(d.z / e.z)));
            if (ma > 1.0f) hc = {p.x + d.x / ma, p.y + d.y / ma, p.z + d.z / ma};
            break;
        }
        case 3: {
            C3 r{hc.x - ct.x, hc.y - ct.y, hc.z - ct.z};
            C3 rmax{mx.x - ct.x, mx.y - ct.y, mx.z - ct.z}, rmin{mn.x - ct.x, mn.y - ct.y, mn.z - ct.z};
            const float eps = 1e-7f;
            auto sc = [&](float s) { r = {r.x * s, r.y * s, r.z * s}; };
            if (r.x > rmax.x + eps) sc(rmax.x / r.x);
            if (r.y > rmax.y + eps) sc(rmax.y / r.y);
            if (r.z > rmax.z + eps) sc(rmax.z / r.z);
            if (r.x < rmin.x - eps) sc(rmin.x / r.x);
            if (r.y < rmin.y - eps) sc(rmin.y / r.y);
            if (r.z < rmin.z - eps) sc(rmin.z / r.z);
            hc = {ct.x + r.x, ct.y + r.y, ct.z + r.z};
            break;
        }
        default: break;
    }

    float alpha = P.mAlpha;
    if (rejected) {
        alpha = P.mRejectionAlpha;
    } else {
        if (P.mVelBasedAlpha) {
            float du = u - hu, dv = v - hv;
            float speed = sqrtf(du * du + dv * dv);
            float t = gclamp(speed * P.mVelBasedAlphaFactor, 0.f, 1.f);
            alpha = gmax(alpha, alpha * (1.0f - t) + P.mVelBasedAlphaMax * t);
        }
        auto lum = [&](C3 c) { return P.mUseYCoCg ? c.x : .25f * c.x + .5f * c.y + .25f * c.z; };
        if (P.mLumaWeightingLottes) {
            float lc = lum(c0), lh = lum(hc);
            float w = 1.0f - fabsf(lc - lh) / gmax(gmax(lc, lh), 0.2f);
            float ww = w * w;
            alpha = P.mMaxAlpha * (1.0f - ww) + P.mMinAlpha * ww;
        }
        if (P.mReduceBlendNearClamp) {
            float lmn = lum(mn), lmx = lum(mx), lh = lum(orig);
            float dist = 2.0f * fabsf(gmin(lh - lmn, lmx - lh)) / (lmx - lmn);
            if (lmx - lmn < 0.001f) dist = 1.0f;
            alpha = alpha * gclamp(4.0f * dist, 0.f, 1.f);
        }
    }
    if (U.mResetHistory) alpha = 1.0f;
    float t = 1.0f - alpha;
    C3 o{hc.x * t + c0.x * alpha, hc.y * t + c0.y * alpha, hc.z * t + c0.z * alpha};
    if (P.mUseYCoCg) {
        float tmp = o.x - o.z;
        o = {tmp + o.y, o.x + o.z, tmp - o.y};
    }
    to_hist = make_float4(o.x, o.y, o.z, 0.f);
    if (P.mToneMapLumaKaris) {
        float l = 1.0f - gmax(gmax(o.x, o.y), o.z);
        o = {o.x / l, o.y / l, o.z / l};
    }
    to_screen = make_float4(o.x, o.y, o.z, 1.0f);
}

// BY rows of kTileX pixels per CTA; SHARPEN 0 none, 1 simple, 2 CAS.
template <int HF, int MC, int INTERP, int SHARPEN, int BY>
__global__ void __launch_bounds__(kTileX * BY) resolve_tiled_kernel(const taa_uniforms_t U, const FrameArgs a) {
    constexpr int BX = kTileX;
    constexpr int NT = BX * BY;
    constexpr int HO = SHARPEN ? 1 : 0;
    constexpr int RX = BX + 2 * HO, RY = BY + 2 * HO;  // resolved region
    constexpr int SX = RX + 2, SY = RY + 2;            // staged colour
    __shared__ float4 s_col[SY * SX];
    __shared__ float3 s_out[SHARPEN ? RY * RX : 1];

    const taa_parameters_t& P = U.param[0];
    const int tid = threadIdx.y * BX + threadIdx.x;
    const int x0 = blockIdx.x * BX - HO, y0 = blockIdx.y * BY - HO;
    const int W = a.out_w, H = a.out_h;
    const bool tonemap = P.mToneMapLumaKaris != 0, ycocg = P.mUseYCoCg != 0;

    for (int i = tid; i < SX * SY; i += NT) {
        int sy = i / SX, sx = i - sy * SX;
        int gx = clampi(x0 - 1 + sx, 0, W - 1), gy = clampi(y0 - 1 + sy, 0, H - 1);
        float4 c = half4_to_float4(__ldg(texel_ptr<uint2>(a.color, gx, gy)));
        s_col[i] = to_working(c, tonemap, ycocg);
    }
    __syncthreads();

    for (int i = tid; i < RX * RY; i += NT) {
        int ry = i / RX, rx = i - ry * RX;
        int x = x0 + rx, y = y0 + ry;
        if (x < 0 || y < 0 || x >= W || y >= H) continue;
        float4 to_hist, to_screen;
        resolve_pixel<HF, MC, INTERP>(U, P, a, x, y, &s_col[(ry + 1) * SX + rx + 1], SX, to_hist, to_screen);
        bool interior = rx >= HO && rx < HO + BX && ry >= HO && ry < HO + BY;
        if (interior) {
            store_history<HF>(a.history_out, x, y, to_hist);
            if (a.result.p) store_rgba16f(a.result, x, y, to_screen);
        }
        if (SHARPEN) {
            // what the reference's sharpen pass reads back from the RGBA16F result image
            float4 q = half4_to_float4(float4_to_half4(to_screen));
            s_out[i] = make_float3(q.x, q.y, q.z);
        }
    }
    if (SHARPEN) {
        __syncthreads();
        int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
        if (x < W && y < H && a.sharpened.p) {
            auto at = [&](int dx, int dy) {
                int xx = clampi(x + dx, 0, W - 1) - x0, yy = clampi(y + dy, 0, H - 1) - y0;
                return s_out[yy * RX + xx];
            };
            float3 r;
            if (SHARPEN == 2)
                r = cas_pixel(at(0, -1), at(-1, 0), at(0, 0), at(1, 0), at(0, 1), __uint_as_float(a.cas_peak_bits));
            else
                r = simple_sharpen_pixel(at(-1, 0), at(1, 0), at(0, -1), at(0, 1), at(0, 0), a.sharpen_factor);
            store_rgba16f(a.sharpened, x, y, make_float4(r.x, r.y, r.z, 1.0f));
        }
    }
}

// Sharpen of an RGBA16F image (result -> sharpened), streaming: each warp
// takes a strip of 30 output columns and kSharpenRows rows.  Lane l loads
// column x0 - 1 + l of the strip's rows and of the rows above and below it
// (edge-clamped coordinates, as the per-tap clamp of sharpen.comp and CAS
// reads them), every load issued before the first use; the left and right
// neighbours come from the adjacent lanes by shuffles, and lanes 1..30 store.
// Launched after a resolve as a programmatic dependent: griddepcontrol.wait
// holds the loads until the resolve's result image is complete (without that
// launch attribute the wait returns at once).
#ifndef TAA_SHARPEN_ROWS
#define TAA_SHARPEN_ROWS 8  // rows per warp strip (a tuning constant)
#endif
constexpr int kSharpenRows = TAA_SHARPEN_ROWS, kSharpenCols = 30;
template <int SHARPEN>
__global__ void __launch_bounds__(256) sharpen_kernel(const FrameArgs a) {
    constexpr int R = kSharpenRows;
    const int W = a.out_w, H = a.out_h;
    const int lane = threadIdx.x & 31;
    const int strips_x = (W + kSharpenCols - 1) / kSharpenCols;
    const int warp = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int sy = warp / strips_x, sx = warp - sy * strips_x;
    const int y0 = sy * R;
    if (y0 >= H) return;  // the same for every lane of the warp
    const int x = sx * kSharpenCols - 1 + lane;
    const int cx = clampi(x, 0, W - 1);
    const Img src{a.result.p, a.result.pitch, W, H};
    asm volatile("griddepcontrol.wait;" ::: "memory");
    uint2 t[R + 2];
#pragma unroll
    for (int r = 0; r < R + 2; ++r) t[r] = __ldg(texel_ptr<uint2>(src, cx, clampi(y0 - 1 + r, 0, H - 1)));
    const bool col_out = lane >= 1 && lane <= kSharpenCols && x < W;
    auto rgb = [](uint2 v) {
        const float4 c = half4_to_float4(v);
        return make_float3(c.x, c.y, c.z);
    };
#pragma unroll
    for (int r = 1; r <= R; ++r) {
        const uint2 c = t[r];
        uint2 lf, rt;
        lf.x = __shfl_up_sync(0xffffffffu, c.x, 1);
        lf.y = __shfl_up_sync(0xffffffffu, c.y, 1);
        rt.x = __shfl_down_sync(0xffffffffu, c.x, 1);
        rt.y = __shfl_down_sync(0xffffffffu, c.y, 1);
        const int y = y0 + r - 1;
        if (col_out && y < H) {
            float3 o;
            if (SHARPEN == 2)
                o = cas_pixel(rgb(t[r - 1]), rgb(lf), rgb(c), rgb(rt), rgb(t[r + 1]), __uint_as_float(a.cas_peak_bits));
            else
                o = simple_sharpen_pixel(rgb(lf), rgb(rt), rgb(t[r - 1]), rgb(t[r + 1]), rgb(c), a.sharpen_factor);
            store_rgba16f(a.sharpened, x, y, make_float4(o.x, o.y, o.z, 1.0f));
        }
    }
}

template <int HF, int MC, int INTERP, int SHARPEN>
cudaError_t launch_tiled(const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    constexpr int BY = SHARPEN ? 16 : 8;
    dim3 block(kTileX, BY);
    dim3 grid((a.out_w + kTileX - 1) / kTileX, (a.out_h + BY - 1) / BY);
    resolve_tiled_kernel<HF, MC, INTERP, SHARPEN, BY><<<grid, block, 0, s>>>(U, a);
    return cudaGetLastError();
}

template <int HF, int MC, int INTERP>
cudaError_t dispatch_sharpen(const FastKey& k, const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    switch (k.sharpen) {
        case 0: return launch_tiled<HF, MC, INTERP, 0>(U, a, s);
        case 1: return launch_tiled<HF, MC, INTERP, 1>(U, a, s);
        default: return launch_tiled<HF, MC, INTERP, 2>(U, a, s);
    }
}
template <int HF, int MC>
cudaError_t dispatch_interp(const FastKey& k, const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    switch (k.interp) {
        case 0: return dispatch_sharpen<HF, MC, 0>(k, U, a, s);
        case 1: return dispatch_sharpen<HF, MC, 1>(k, U, a, s);
        default: return dispatch_sharpen<HF, MC, 2>(k, U, a, s);
    }
}

}  // namespace

cudaError_t launch_resolve_fast(const FastKey& k, const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    if (k.history_fmt == 0) {
        return k.motion_ch == 4 ? dispatch_interp<0, 4>(k, U, a, s) : dispatch_interp<0, 2>(k, U, a, s);
    }
    return k.motion_ch == 4 ? dispatch_interp<1, 4>(k, U, a, s) : dispatch_interp<1, 2>(k, U, a, s);
}

cudaError_t launch_sharpen(int sharpener, const FrameArgs& a, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    const long long warps = (long long)((a.out_w + kSharpenCols - 1) / kSharpenCols) *
                            ((a.out_h + kSharpenRows - 1) / kSharpenRows);
    cfg.gridDim = dim3((unsigned)((warps + 7) / 8));
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return sharpener == 2 ? cudaLaunchKernelEx(&cfg, sharpen_kernel<2>, a) : cudaLaunchKernelEx(&cfg, sharpen_kernel<1>, a);
}

}  // namespace taa_dev
