// resolve_fast16.cu - the FP16 form in the benchmark mode: the strip body
// (strip_body.cuh) with the neighbourhood and clip arithmetic in packed half2
// and the history and blend in FP32.
//
//  * staging: each source texel is converted once to YCoCg and stored as two
//    half2 words, (Y, Co) and (Cg, 0) - 8 bytes, half the shared-memory
//    traffic of the FP32 staging;
//  * box: the 3x3 mean and variance (taa.comp:266-277) in half2, about the
//    pixel's own centre texel: d = t - c, mean = c + sum(d)/9, var =
//    sum(d^2)/9 - (sum(d)/9)^2.  In FP16 the shader's one-pass
//    m2/9 - mean^2 cancels to nothing on a flat neighbourhood; about the
//    centre the squared terms are small there, and where they are large (a
//    firefly at the centre) the variance is large too;
//  * clip: the ratio of the history's distance from the box centre to the
//    box half extent (taa.comp:323-345) in half2 with the approximate half2
//    reciprocal; the half extent is held at least at the smallest normal
//    FP16 value, 6.1e-5 (the shader's 1e-7 is not a normal FP16 number);
//  * guard: a clip that engages on a box whose tightest half extent is
//    TAA_FP16_STRIP_GUARD_RATIO times narrower than its widest (the tight
//    chroma box next to a firefly, where the clip multiplies the box's FP16
//    error by up to the ratio), or on a box that is not finite, is decided
//    again in FP32 from the pixel's nine source texels;
//  * the history filter, the clipped history value, the current colour (read
//    again from the source texel in FP32) and the blend stay in FP32, so an
//    alpha near 0.1 does not drift over long sequences.
// Contract: frame relative L2 within 1e-3 of the FP64 oracle (tests/).
#include <cuda_fp16.h>

#include <cstring>

#include "strip_body.cuh"

// Ratio of a box's widest to its tightest half extent above which a clip that
// engages is decided in FP32 (a tuning constant, chosen by measurement on the
// benchmark sequences).
#ifndef TAA_FP16_STRIP_GUARD_RATIO
#define TAA_FP16_STRIP_GUARD_RATIO 16.0f
#endif

namespace taa_dev {
namespace fast32 {

__device__ __forceinline__ __half2 u2h(uint32_t v) { return *reinterpret_cast<__half2*>(&v); }
__device__ __forceinline__ uint32_t h2u(__half2 v) { return *reinterpret_cast<uint32_t*>(&v); }

struct HalfPol {
    using Staged = uint2;  // (Y, Co), (Cg, 0) as half2
    static __device__ __forceinline__ uint2 stage(uint2 raw) {
        const float3 c = ycocg(raw);
        return make_uint2(h2u(__floats2half2_rn(c.x, c.y)), h2u(__floats2half2_rn(c.z, 0.f)));
    }

    // The FP32 box and clip ratio of pixel (x, y) from its nine source texels
    // (the guard): the same arithmetic as TAA_FORM_FAST's box.
    static __device__ __noinline__ void box_f32(const Args& a, int x, int y, const float hc[3], float m[3],
                                                float& ma) {
        float s1[3] = {0.f, 0.f, 0.f}, s2[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                const float3 t = ycocg(__ldg(at<uint2>(a.color, a.color_pitch, clampi(x + dx, 0, a.W - 1),
                                                       clampi(y + dy, 0, a.H - 1))));
                const float tv[3] = {t.x, t.y, t.z};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    s1[c] += tv[c];
                    s2[c] = fmaf(tv[c], tv[c], s2[c]);
                }
            }
        ma = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            m[c] = s1[c] * (1.0f / 9.0f);
            const float var = fmaf(-m[c], m[c], s2[c] * (1.0f / 9.0f));
            const float e = fmaf(a.gamma, sqrt_approx(fmaxf(var, 0.f)), 1e-7f);
            ma = fmaxf(ma, fabsf(hc[c] - m[c]) * rcp_approx(e));
        }
    }

    static __device__ __forceinline__ void finish(const Args& a, const uint2* sp, int x, int ya, const float3 h[NPX],
                                                  unsigned rej, bool landed) {
        const __half2 ninth = __float2half2_rn(1.0f / 9.0f), zero = __float2half2_rn(0.f);
        const __half2 gam = __float2half2_rn(a.gamma), eps = __float2half2_rn(6.103515625e-05f);
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            const int y = ya + k;
            if (!(x < a.W && y < a.H && landed)) continue;
            // box about the centre texel, in half2
            const uint2 cc = sp[(k + 1) * SX + 1];
            const __half2 ca = u2h(cc.x), cb = u2h(cc.y);
            __half2 s1a = zero, s1b = zero, s2a = zero, s2b = zero;
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const uint2 t = sp[(k + r) * SX + c];
                    const __half2 da = __hsub2(u2h(t.x), ca), db = __hsub2(u2h(t.y), cb);
                    s1a = __hadd2(s1a, da);
                    s1b = __hadd2(s1b, db);
                    s2a = __hfma2(da, da, s2a);
                    s2b = __hfma2(db, db, s2b);
                }
            const __half2 qa = __hmul2(s1a, ninth), qb = __hmul2(s1b, ninth);
            const __half2 ma_ = __hadd2(ca, qa), mb_ = __hadd2(cb, qb);
            const __half2 va = __hmax2(__hfma2(__hneg2(qa), qa, __hmul2(s2a, ninth)), zero);
            const __half2 vb = __hmax2(__hfma2(__hneg2(qb), qb, __hmul2(s2b, ninth)), zero);
            const __half2 ea = __hfma2(gam, h2sqrt(va), eps), eb = __hfma2(gam, h2sqrt(vb), eps);
            // the clip decision in half2
            float hc[3];
            hist_ycocg(h[k], hc);
            const __half2 da = __habs2(__hsub2(__floats2half2_rn(hc[0], hc[1]), ma_));
            const __half2 db = __habs2(__hsub2(__floats2half2_rn(hc[2], 0.f), mb_));
            const __half2 ra = __hmul2(da, h2rcp(ea)), rb = __hmul2(db, h2rcp(eb));
            float ma = fmaxf(fmaxf(__low2float(ra), __high2float(ra)), __low2float(rb));
            const float2 mf = __half22float2(ma_);
            float m[3] = {mf.x, mf.y, __low2float(mb_)};
            // the guard: an engaged clip on an ill-conditioned or non-finite box, in FP32
            const float e0 = __low2float(ea), e1 = __high2float(ea), e2 = __low2float(eb);
            const float emin = fminf(e0, fminf(e1, e2)), emax = fmaxf(e0, fmaxf(e1, e2));
            if (!(ma <= 1.0f) && !(emax <= TAA_FP16_STRIP_GUARD_RATIO * emin && ma < 65504.f)) box_f32(a, x, y, hc, m, ma);
            // the current colour in FP32 from its source texel
            const float3 cur3 = ycocg(__ldg(at<uint2>(a.color, a.color_pitch, x, y)));
            const float cur[3] = {cur3.x, cur3.y, cur3.z};
            const float alpha = a.reset ? 1.0f : ((rej >> k) & 1u ? a.rejection_alpha : a.alpha);
            clip_blend_store(a, x, y, hc, m, ma, cur, alpha);
        }
    }
};

}  // namespace fast32

cudaError_t launch_resolve_half_strips(int motion_ch, const taa_uniforms_t& U, const FrameArgs& f, cudaStream_t s) {
    using namespace fast32;
    const Args a = make_args(U, f);
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int tma_ok = a.hist && f.history.w >= WW && f.history.h >= WH &&
                       encode_history_map(f.history, TAA_FAST_TMA2D ? 2 : 0, WW, WH, &map);
    const dim3 grid((a.W + TX - 1) / TX, (a.H + TY - 1) / TY);
    if (U.param[0].mInterpolationMode == 2) {
        if (motion_ch == 4) resolve_strips<HalfPol, 2, 4><<<grid, NT, 0, s>>>(a, map, tma_ok);
        else resolve_strips<HalfPol, 2, 2><<<grid, NT, 0, s>>>(a, map, tma_ok);
    } else {
        if (motion_ch == 4) resolve_strips<HalfPol, 0, 4><<<grid, NT, 0, s>>>(a, map, tma_ok);
        else resolve_strips<HalfPol, 0, 2><<<grid, NT, 0, s>>>(a, map, tma_ok);
    }
    return cudaGetLastError();
}

}  // namespace taa_dev
