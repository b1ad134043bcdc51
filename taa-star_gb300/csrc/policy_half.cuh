// policy_half.cuh - the arithmetic policy of the FP16 resolve form: the CTA
// pipeline of tiled_skeleton.cuh with packed-half2 neighbourhood and clip
// arithmetic.
//
//  * staging: each source texel is converted once to YCoCg in half2
//    arithmetic and kept as two half2 words, (Y, Co) and (Cg, 0);
//  * box: the 3x3 mean and variance (taa.comp:266-277) in half2, in two
//    passes - mean = c_0 + sum(c_k - c_0)/9, then var = sum(c_k - mean)^2/9 -
//    so no FP16 sum cancels (the shader's one-pass m2/9 - mean^2 would lose
//    all precision in FP16); min/max boxes use half2 min/max;
//  * clip: the clip-towards-centre decision (taa.comp:323-345) is taken in
//    half2 with an approximate reciprocal; the box half-width is held at
//    least at the smallest normal FP16 value (6.1e-5, instead of the shader's
//    1e-7, which FP16 cannot hold as a normal number);
//  * the history filter, the clipped history value, the current colour and
//    the blend stay in FP32, so an alpha near 0.1 does not drift over long
//    sequences.
//  * GUARD (TAA_FLAG_FP16_GUARD): a pixel whose clip engages on a box that
//    is ill-conditioned for FP16 is finished in FP32 from its source texels.
// Its error contract is against the FP64 oracle, frame by frame (relative L2
// and PSNR), not bit parity.  resolve_half.cu and resolve_half_guard.cu
// instantiate the two variants (compiled without -fmad=false).
#pragma once
#include <cuda_fp16.h>

#include "history_filter.cuh"
#include "kernels.h"
#include "policy_f32.cuh"

namespace taa_dev {
namespace half_form {

using tiled::C3;

__device__ __forceinline__ __half2 u2h(uint32_t v) { return *reinterpret_cast<__half2*>(&v); }
__device__ __forceinline__ uint32_t h2u(__half2 v) { return *reinterpret_cast<uint32_t*>(&v); }

// Width ratio of a box's widest to its tightest channel above which the
// guarded variant finishes a clipped pixel in FP32 (a tuning constant, by
// measurement on the benchmark scenes: at 256 single frames stay below 1e-3
// relative L2 against FP64 but a 64-frame C2 chain reaches 1.1e-3; at 16
// single frames measure below 1e-4).
#ifndef TAA_FP16_EXACT_RATIO
#define TAA_FP16_EXACT_RATIO 16.0f
#endif

template <bool GUARD> struct HalfPol : tiled::HistoryFilter {
    using Staged = uint2;  // (Y, Co), (Cg, 0) as half2 - or (R, G), (B, 0)
    struct Box {
        __half2 c0a, c0b, lo_a, lo_b, hi_a, hi_b, ct_a, ct_b;
        C3 cur;  // the current colour in FP32 for the blend
    };
    // the blend takes the current colour in FP32 from the source texel
    static constexpr bool kExactCentre = true;
    static __device__ __forceinline__ C3 centre(const Box& b, const uint2*) { return b.cur; }
    static __device__ __forceinline__ void centre_colour(Box& b, const Img& color, int cx, int cy, bool tonemap,
                                                         bool ycocg) {
        float4 c = half4_to_float4(__ldg(texel_ptr<uint2>(color, cx, cy)));
        if (tonemap) {
            float l = 1.0f + gmax(gmax(c.x, c.y), c.z);
            c.x = c.x / l;
            c.y = c.y / l;
            c.z = c.z / l;
        }
        if (ycocg)
            b.cur = {.25f * c.x + .5f * c.y + .25f * c.z, .5f * c.x - .5f * c.z, -.25f * c.x + .5f * c.y - .25f * c.z};
        else
            b.cur = {c.x, c.y, c.z};
    }

    static __device__ __forceinline__ uint2 stage(uint2 raw, bool tonemap, bool ycocg) {
        __half2 rg = u2h(raw.x), ba = u2h(raw.y);
        if (tonemap) {
            float4 c = half4_to_float4(raw);
            float l = 1.0f + gmax(gmax(c.x, c.y), c.z);
            rg = __floats2half2_rn(c.x / l, c.y / l);
            ba = __floats2half2_rn(c.z / l, 0.f);
        }
        if (ycocg) {
            const __half2 r2 = __low2half2(rg), g2 = __high2half2(rg), b2 = __low2half2(ba);
            __half2 ya = __hfma2(r2, __floats2half2_rn(.25f, .5f), __hmul2(g2, __floats2half2_rn(.5f, 0.f)));
            ya = __hfma2(b2, __floats2half2_rn(.25f, -.5f), ya);
            __half2 yb = __hfma2(r2, __floats2half2_rn(-.25f, 0.f), __hmul2(g2, __floats2half2_rn(.5f, 0.f)));
            yb = __hfma2(b2, __floats2half2_rn(-.25f, 0.f), yb);
            return make_uint2(h2u(ya), h2u(yb));
        }
        return make_uint2(h2u(rg), h2u(__halves2half2(__low2half(ba), __float2half_rn(0.f))));
    }

    template <bool HOT>
    static __device__ __forceinline__ void box(const uint2* nb, int ns, const tiled::Mode<HOT>& M, float g, Box& b,
                                               f2 /*unused*/) {
        const int off[8] = {-ns - 1, -ns, -ns + 1, -1, 1, ns - 1, ns, ns + 1};
        const uint2 cc = nb[0];
        const __half2 c0a = u2h(cc.x), c0b = u2h(cc.y);
        b.c0a = c0a;
        b.c0b = c0b;
        b.ct_a = c0a;
        b.ct_b = c0b;
        if (M.variance()) {
            // two passes about the centre, then about the mean: the squared
            // deviations are summed without cancellation
            uint2 t[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) t[k] = nb[off[k]];
            __half2 s1a = __float2half2_rn(0.f), s1b = s1a;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                s1a = __hadd2(s1a, __hsub2(u2h(t[k].x), c0a));
                s1b = __hadd2(s1b, __hsub2(u2h(t[k].y), c0b));
            }
            const __half2 ninth = __float2half2_rn(1.0f / 9.0f);
            const __half2 ma = __hfma2(s1a, ninth, c0a), mb = __hfma2(s1b, ninth, c0b);
            __half2 da = __hsub2(c0a, ma), db = __hsub2(c0b, mb);
            __half2 s2a = __hmul2(da, da), s2b = __hmul2(db, db);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                da = __hsub2(u2h(t[k].x), ma);
                db = __hsub2(u2h(t[k].y), mb);
                s2a = __hfma2(da, da, s2a);
                s2b = __hfma2(db, db, s2b);
            }
            const __half2 gg = __float2half2_rn(g);
            __half2 sa = __hmul2(gg, h2sqrt(__hmul2(s2a, ninth))), sb = __hmul2(gg, h2sqrt(__hmul2(s2b, ninth)));
            b.lo_a = __hsub2(ma, sa);
            b.hi_a = __hadd2(ma, sa);
            b.lo_b = __hsub2(mb, sb);
            b.hi_b = __hadd2(mb, sb);
            b.ct_a = ma;
            b.ct_b = mb;
        } else {
            __half2 la = c0a, lb = c0b, ha = c0a, hb = c0b;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                uint2 t = nb[off[k]];
                la = __hmin2(la, u2h(t.x));
                lb = __hmin2(lb, u2h(t.y));
                ha = __hmax2(ha, u2h(t.x));
                hb = __hmax2(hb, u2h(t.y));
            }
            if (M.shaped()) {
                // the cross: centre, up, left, right, down (taa.comp:282-285)
                __half2 pa = c0a, pb = c0b, qa = c0a, qb = c0b;
                const int cross[4] = {-ns, -1, 1, ns};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    uint2 t = nb[cross[k]];
                    pa = __hmin2(pa, u2h(t.x));
                    pb = __hmin2(pb, u2h(t.y));
                    qa = __hmax2(qa, u2h(t.x));
                    qb = __hmax2(qb, u2h(t.y));
                }
                const __half2 h = __float2half2_rn(0.5f);
                la = __hmul2(__hadd2(la, pa), h);
                lb = __hmul2(__hadd2(lb, pb), h);
                ha = __hmul2(__hadd2(ha, qa), h);
                hb = __hmul2(__hadd2(hb, qb), h);
            }
            b.lo_a = la;
            b.lo_b = lb;
            b.hi_a = ha;
            b.hi_b = hb;
        }
        if (M.shrink()) {
            const __half2 h = __float2half2_rn(0.5f);
            __half2 cea = __hmul2(__hadd2(b.lo_a, b.hi_a), h), ceb = __hmul2(__hadd2(b.lo_b, b.hi_b), h);
            __half2 hsa = __hmul2(__hsub2(b.hi_a, b.lo_a), __floats2half2_rn(0.5f, 0.25f));
            __half2 hsb = __hmul2(__hsub2(b.hi_b, b.lo_b), __floats2half2_rn(0.25f, 0.25f));
            b.lo_a = __hsub2(cea, hsa);
            b.hi_a = __hadd2(cea, hsa);
            b.lo_b = __hsub2(ceb, hsb);
            b.hi_b = __hadd2(ceb, hsb);
            float2 ta = __half22float2(b.ct_a), tb = __half22float2(b.ct_b);
            float2 la = __half22float2(b.lo_a), lb = __half22float2(b.lo_b), ha = __half22float2(b.hi_a),
                   hb = __half22float2(b.hi_b);
            if (ta.x < la.x || ta.y < la.y || tb.x < lb.x || ta.x > ha.x || ta.y > ha.y || tb.x > hb.x) {
                b.ct_a = cea;
                b.ct_b = ceb;
            }
        }
    }

    static __device__ __forceinline__ void reproject(const taa_uniforms_t& U, float u, float v, float depth, float& hu,
                                                     float& hv, float& ehd) {
        float cs0 = u * 2.0f - 1.0f, cs1 = v * 2.0f - 1.0f;
        const float* A = U.mInverseViewProjMatrix;
        const float* B = U.mHistoryViewProjMatrix;
        float ws[4], hs[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) ws[i] = A[i] * cs0 + A[4 + i] * cs1 + A[8 + i] * depth + A[12 + i];
#pragma unroll
        for (int i = 0; i < 4; ++i) hs[i] = B[i] * ws[0] + B[4 + i] * ws[1] + B[8 + i] * ws[2] + B[12 + i] * ws[3];
        float r = 1.0f / hs[3];
        hu = (hs[0] * r) * 0.5f + 0.5f;
        hv = (hs[1] * r) * 0.5f + 0.5f;
        ehd = hs[2] * r;
    }

    // Where an ill-conditioned clip is finished in FP32 (exact_finish): the
    // frame, the pixel and whether the source is tonemapped.
    struct At {
        const FrameArgs* a;
        int x, y;
        bool tm;
    };

    template <bool HOT>
    static __device__ __forceinline__ float4 finish(const taa_uniforms_t& U, const taa_parameters_t& P,
                                                    const tiled::Mode<HOT>& M, const Box& b, const C3& c0, float4 hraw, float u,
                                                    float v, float hu, float hv, bool rejected) {
        return finish_at<HOT>(U, P, M, b, c0, hraw, u, v, hu, hv, rejected, nullptr);
    }
    template <bool HOT>
    static __device__ __forceinline__ float4 finish_at(const taa_uniforms_t& U, const taa_parameters_t& P,
                                                       const tiled::Mode<HOT>& M, const Box& b, const C3& c0,
                                                       float4 hraw, float u, float v, float hu, float hv, bool rejected,
                                                       const At* at) {
        const bool yc = M.ycocg();
        C3 hc{hraw.x, hraw.y, hraw.z};
        if (yc)
            hc = {.25f * hraw.x + .5f * hraw.y + .25f * hraw.z, .5f * hraw.x - .5f * hraw.z,
                  -.25f * hraw.x + .5f * hraw.y - .25f * hraw.z};
        const C3 orig = hc;
        const int clip = M.clip();
        if (clip == 2) {
            // decision in half2, clipped value in FP32
            const __half2 h = __float2half2_rn(0.5f), emin = __float2half2_rn(6.103515625e-05f);
            __half2 pa = __hmul2(__hadd2(b.hi_a, b.lo_a), h), pb = __hmul2(__hadd2(b.hi_b, b.lo_b), h);
            __half2 ea = __hmax2(__hmul2(__hsub2(b.hi_a, b.lo_a), h), emin);
            __half2 eb = __hmax2(__hmul2(__hsub2(b.hi_b, b.lo_b), h), emin);
            __half2 qa = __floats2half2_rn(hc.x, hc.y), qb = __floats2half2_rn(hc.z, 0.f);
            __half2 ua = __habs2(__hmul2(__hsub2(qa, pa), h2rcp(ea)));
            __half2 ub = __habs2(__hmul2(__hsub2(qb, pb), h2rcp(eb)));
            __half2 mm = __hmax2(ua, __lowhigh2highlow(ua));
            __half m = __hmax(__low2half(mm), __low2half(ub));
            if constexpr (GUARD) {
                if (at && __hgt(m, __float2half_rn(1.0f))) {
                    // the clip engages: with a box this ill-conditioned, finish in FP32
                    const float2 ef = __half22float2(ea);
                    const float ez = __low2float(eb);
                    if (gmin(gmin(ef.x, ef.y), ez) * kExactRatio < gmax(gmax(ef.x, ef.y), ez))
                        return exact_finish<HOT>(U, *at->a, P, M, hraw, u, v, hu, hv, rejected, at->x, at->y, at->tm);
                }
            }
            if (__hgt(m, __float2half_rn(1.0f))) {
                float2 pf = __half22float2(pa);
                float pz = __low2float(pb);
                float r = __fdividef(1.0f, __half2float(m));
                hc = {pf.x + (hc.x - pf.x) * r, pf.y + (hc.y - pf.y) * r, pz + (hc.z - pz) * r};
            }
        } else if (clip == 1 || clip == 3) {
            float2 la = __half22float2(b.lo_a), lb = __half22float2(b.lo_b), ha = __half22float2(b.hi_a),
                   hb = __half22float2(b.hi_b), ta = __half22float2(b.ct_a), tb = __half22float2(b.ct_b);
            C3 mn{la.x, la.y, lb.x}, mx{ha.x, ha.y, hb.x}, ct{ta.x, ta.y, tb.x};
            if (clip == 1) {
                hc = {gmin(gmax(hc.x, mn.x), mx.x), gmin(gmax(hc.y, mn.y), mx.y), gmin(gmax(hc.z, mn.z), mx.z)};
            } else {
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
            }
        }
        float alpha = P.mAlpha;
        if (rejected) {
            alpha = P.mRejectionAlpha;
        } else {
            if (M.vel_alpha()) {
                float du = u - hu, dv = v - hv;
                float t = gclamp(sqrtf(du * du + dv * dv) * P.mVelBasedAlphaFactor, 0.f, 1.f);
                alpha = gmax(alpha, alpha * (1.0f - t) + P.mVelBasedAlphaMax * t);
            }
            auto lum = [&](C3 c) { return yc ? c.x : .25f * c.x + .5f * c.y + .25f * c.z; };
            if (M.lottes()) {
                float lc = lum(c0), lh = lum(hc);
                float w = 1.0f - fabsf(lc - lh) / gmax(gmax(lc, lh), 0.2f);
                float ww = w * w;
                alpha = P.mMaxAlpha * (1.0f - ww) + P.mMinAlpha * ww;
            }
            if (M.near_clamp()) {
                float2 la = __half22float2(b.lo_a), ha = __half22float2(b.hi_a);
                float2 lb = __half22float2(b.lo_b), hb = __half22float2(b.hi_b);
                float lmn = lum(C3{la.x, la.y, lb.x}), lmx = lum(C3{ha.x, ha.y, hb.x}), lh = lum(orig);
                float dist = 2.0f * fabsf(gmin(lh - lmn, lmx - lh)) / (lmx - lmn);
                if (lmx - lmn < 0.001f) dist = 1.0f;
                alpha = alpha * gclamp(4.0f * dist, 0.f, 1.f);
            }
        }
        if (U.mResetHistory) alpha = 1.0f;
        float t = 1.0f - alpha;
        C3 o{hc.x * t + c0.x * alpha, hc.y * t + c0.y * alpha, hc.z * t + c0.z * alpha};
        if (yc) {
            float tmp = o.x - o.z;
            o = {tmp + o.y, o.x + o.z, tmp - o.y};
        }
        if (M.noise()) {  // taa.comp:903-906
            const float4 n = taa_noise(U, P, u, v);
            o = {o.x + n.x, o.y + n.y, o.z + n.z};
        }
        return make_float4(o.x, o.y, o.z, 0.f);
    }

    static __device__ __forceinline__ float4 un_tonemap(float4 o) {
        float l = 1.0f - gmax(gmax(o.x, o.y), o.z);
        return make_float4(o.x / l, o.y / l, o.z / l, o.w);
    }

    // The clip of taa.comp:323-369 multiplies the error of the box's tightest
    // channel by the displacement in the widest one (|d|/ma, taa.comp:340).
    // Next to a firefly the luma box spans the spike while the chroma box stays
    // a few FP16 ulps wide, and the clipped value moves by O(1).  A pixel whose
    // clip engages on such a box - its tightest channel kExactRatio times
    // narrower than its widest - is finished in FP32 from the source texels
    // instead (exact_finish).
    static constexpr bool kExactFallback = GUARD;
    static constexpr bool kDebug = false;  // a debug binding runs the tiled FP32 form
    static constexpr float kExactRatio = TAA_FP16_EXACT_RATIO;
    // The pixel as the FP32 form resolves it: its 3x3 source texels staged in
    // FP32, the FP32 box and the FP32 rectification and blend.
    template <bool HOT>
    static __device__ __noinline__ float4 exact_finish(const taa_uniforms_t& U, const FrameArgs& a,
                                                       const taa_parameters_t& P, const tiled::Mode<HOT>& M,
                                                       float4 hraw, float u, float v, float hu, float hv,
                                                       bool rejected, int x, int y, bool tm) {
        const bool yc = M.ycocg();
        const int W = a.color.w, H = a.color.h;
        float4 nb[9];
#pragma unroll
        for (int k = 0; k < 9; ++k)
            nb[k] = tiled::ExactF32::stage(
                __ldg(texel_ptr<uint2>(a.color, clampi(x + k % 3 - 1, 0, W - 1), clampi(y + k / 3 - 1, 0, H - 1))),
                tm, yc);
        tiled::ExactF32::Box eb;
        tiled::ExactF32::box<HOT>(&nb[4], 3, M, P.mVarClipGamma, eb, f2{a.neg_zero2});
        return tiled::ExactF32::finish<HOT>(U, P, M, eb, C3{nb[4].x, nb[4].y, nb[4].z}, hraw, u, v, hu, hv, rejected);
    }
};

}  // namespace half_form
}  // namespace taa_dev
