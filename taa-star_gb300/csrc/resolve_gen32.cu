// resolve_gen32.cu - TAA_FORM_FAST for the rest of the parameter block's
// rectification modes on the strip body (strip_body.cuh): YCoCg or RGB, the
// variance box (taa.comp:266-277) or the 3x3 minimum/maximum box (288-291),
// clamp (taa.comp:831) or the clip toward the box centre (clipAabb,
// taa.comp:323-345), any use of the velocity (for every pixel, for movers,
// or reprojection through the matrices).  The benchmark mode (YCoCg,
// variance, clip, velocity for every pixel) runs F32Pol and the reference's
// default mode (RGB, min/max, clamp) ClampRgbPol; this unit covers the other
// combinations with one policy template, one view, RGBA32F history.
#include <cstring>

#include "strip_body.cuh"

namespace taa_dev {
namespace fast32 {

template <bool YC, bool VAR, int RECT>  // RECT 1 clamp, 2 clip toward the centre
struct GenPol {
    using Staged = float4;
    struct Ctx {
        const Reproj* rp;
    };
    static constexpr bool kReproject = true;
    // (Y, Co, Cg, Cg^2) or (R, G, B, B^2): the fourth lane feeds the third
    // channel's second moment
    static __device__ __forceinline__ float4 stage(uint2 raw) {
        if constexpr (YC) {
            return F32Pol::stage(raw);
        } else {
            const float4 c = half4_to_float4(raw);
            return make_float4(c.x, c.y, c.z, c.z * c.z);
        }
    }
    static __device__ __forceinline__ void finish(const Args& a, const float4* sp, int x, int ya, const float3 h[NPX],
                                                  unsigned rej, bool landed, const PixelInfo& px, Ctx& ctx) {
        const Reproj& md = *ctx.rp;
        // a colour's luma in the working space (taa.comp:855-893)
        auto lum = [](const float c[3]) { return YC ? c[0] : 0.25f * c[0] + 0.5f * c[1] + 0.25f * c[2]; };
        Row r0, r1;
        RowMinMax q0, q1;
        if constexpr (VAR) {
            r0 = row_sums(sp);
            r1 = row_sums(sp + SX);
        } else {
            q0 = row_minmax(sp);
            q1 = row_minmax(sp + SX);
        }
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            float lo[3], hi[3];  // the box: clamp bounds (min/max, or mean -+ gamma sigma)
            float p[3], e[3];    // its centre and half extent + 1e-7 (the clip's)
            if constexpr (VAR) {
                const Row r2 = row_sums(sp + (k + 2) * SX);
                const Row s = add(add(r0, r1), r2);
                r0 = r1;
                r1 = r2;
                const f2 n = dup(1.0f / 9.0f);
                const f2 mean = mulp(s.a, n), c2 = mulp(s.c, n);
                const f2 var = fmap(neg2(mean), mean, mulp(s.q, n));
                const float m[3] = {f2lo(mean), f2hi(mean), f2lo(c2)};
                const float v[3] = {f2lo(var), f2hi(var), fmaf(-f2lo(c2), f2lo(c2), f2hi(c2))};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float sg = a.gamma * sqrt_approx(fmaxf(v[c], 0.f));
                    lo[c] = m[c] - sg;
                    hi[c] = m[c] + sg;
                    p[c] = m[c];
                    e[c] = sg + 1e-7f;
                }
            } else {
                const RowMinMax q2 = row_minmax(sp + (k + 2) * SX);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    lo[c] = fminf(q0.mn[c], fminf(q1.mn[c], q2.mn[c]));
                    hi[c] = fmaxf(q0.mx[c], fmaxf(q1.mx[c], q2.mx[c]));
                    p[c] = 0.5f * (hi[c] + lo[c]);
                    e[c] = fmaf(0.5f, hi[c] - lo[c], 1e-7f);
                }
                q0 = q1;
                q1 = q2;
            }
            if (YC && md.shrink) {  // taa.comp:297-311: chroma half extents halved about the box centre
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float half = (c == 0 ? 0.5f : 0.25f) * (hi[c] - lo[c]), ce = (lo[c] + hi[c]) * 0.5f;
                    lo[c] = ce - half;
                    hi[c] = ce + half;
                    p[c] = ce;
                    e[c] = half + 1e-7f;
                }
            }
            const int y = ya + k;
            if (!(x < a.W && y < a.H && landed)) continue;
            float hc[3];
            if constexpr (YC) {
                hist_ycocg(h[k], hc);
            } else {
                hc[0] = h[k].x;
                hc[1] = h[k].y;
                hc[2] = h[k].z;
            }
            const float orig[3] = {hc[0], hc[1], hc[2]};
            if constexpr (RECT == 1) {
#pragma unroll
                for (int c = 0; c < 3; ++c) hc[c] = fminf(fmaxf(hc[c], lo[c]), hi[c]);
            } else {
                float ma = 0.f;
#pragma unroll
                for (int c = 0; c < 3; ++c) ma = fmaxf(ma, fabsf(hc[c] - p[c]) * rcp_approx(e[c]));
                const float sc = ma > 1.0f ? rcp_approx(ma) : 1.0f;
#pragma unroll
                for (int c = 0; c < 3; ++c) hc[c] = fmaf(hc[c] - p[c], sc, p[c]);
            }
            const float4 c0 = lds128(&sp[(k + 1) * SX + 1]);
            const float cur[3] = {c0.x, c0.y, c0.z};
            float alpha = a.alpha;
            if ((rej >> k) & 1u) {
                alpha = a.rejection_alpha;
            } else {
                if (md.vel_alpha) {  // taa.comp:856-860
                    const float du = px.u - px.hu[k], dv = px.v[k] - px.hv[k];
                    const float t = fminf(fmaxf(sqrt_approx(du * du + dv * dv) * md.vel_alpha_factor, 0.f), 1.f);
                    alpha = fmaxf(alpha, fmaf(t, md.vel_alpha_max - alpha, alpha));
                }
                if (md.lottes) {  // taa.comp:863-870
                    const float lc = lum(cur), lh = lum(hc);
                    const float wl = 1.0f - fabsf(lc - lh) * rcp_approx(fmaxf(fmaxf(lc, lh), 0.2f));
                    alpha = fmaf(wl * wl, md.min_alpha - md.max_alpha, md.max_alpha);
                }
                if (md.near_clamp) {  // taa.comp:873-892
                    const float lmn = lum(lo), lmx = lum(hi), lh = lum(orig);
                    float dist = 2.0f * fabsf(fminf(lh - lmn, lmx - lh)) * rcp_approx(lmx - lmn);
                    if (lmx - lmn < 0.001f) dist = 1.0f;
                    alpha *= fminf(fmaxf(4.0f * dist, 0.f), 1.f);
                }
            }
            if (a.reset) alpha = 1.0f;
            float o[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) o[c] = fmaf(alpha, cur[c] - hc[c], hc[c]);
            if constexpr (YC) {
                const float tmp = o[0] - o[2];
                store_out(a, x, y, make_float4(tmp + o[1], o[0] + o[2], tmp - o[1], 0.f));
            } else {
                store_out(a, x, y, make_float4(o[0], o[1], o[2], 0.f));
            }
        }
    }
};

}  // namespace fast32

// The parameter modes this unit runs: clamp or clip toward the centre on the
// variance or min/max box, YCoCg (with or without chroma-axis shrinking) or
// RGB, any velocity use with simple sampling, the velocity-based alpha, the
// luma weighting and the near-clamp reduction of the blend weight; no
// tonemap, shaped neighbourhood, noise, anti-ghosting or ray-trace assist.
bool fast32_gen_mode(const taa_parameters_t& P) {
    return !P.mToneMapLumaKaris && !P.mShapedNeighbourhood &&
           (P.mColorClampingOrClipping == 1 || P.mColorClampingOrClipping == 2) && P.mUseVelocityVectors >= 0 &&
           P.mUseVelocityVectors <= 2 && P.mVelocitySampleMode == 0 && !P.mAddNoise && !P.mDynamicAntiGhosting &&
           !P.mRayTraceAugment && (P.mInterpolationMode == 0 || P.mInterpolationMode == 2);
}

bool fast32_gen_supported(const taa_uniforms_t& U, int history_fmt, int in_w, int in_h, int out_w, int out_h) {
    return history_fmt == 0 && fast32_gen_mode(U.param[0]) && fast_path_supported(U, in_w, in_h, out_w, out_h);
}

cudaError_t launch_resolve_fast32_gen(int motion_ch, const taa_uniforms_t& U, const FrameArgs& f, cudaStream_t s) {
    using namespace fast32;
    const taa_parameters_t& P = U.param[0];
    const Args a = make_args(U, f);
    const Reproj rp = make_reproj(U);
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int tma_ok = a.hist && f.history.w >= WW && f.history.h >= WH && encode_history_map(f.history, 2, WW, WH, &map);
    const dim3 grid((a.W + TX - 1) / TX, (a.H + TY - 1) / TY);
    const bool cr = P.mInterpolationMode == 2, m4 = motion_ch == 4;
    auto go = [&](auto pol) {
        using Pol = decltype(pol);
        if (cr) {
            if (m4) resolve_strips_reproj<Pol, 2, 4><<<grid, NT, 0, s>>>(a, map, tma_ok, rp);
            else resolve_strips_reproj<Pol, 2, 2><<<grid, NT, 0, s>>>(a, map, tma_ok, rp);
        } else {
            if (m4) resolve_strips_reproj<Pol, 0, 4><<<grid, NT, 0, s>>>(a, map, tma_ok, rp);
            else resolve_strips_reproj<Pol, 0, 2><<<grid, NT, 0, s>>>(a, map, tma_ok, rp);
        }
        return cudaGetLastError();
    };
    const bool yc = P.mUseYCoCg != 0, var = P.mVarianceClipping != 0, clamp = P.mColorClampingOrClipping == 1;
    if (yc) {
        if (var) return clamp ? go(GenPol<true, true, 1>{}) : go(GenPol<true, true, 2>{});
        return clamp ? go(GenPol<true, false, 1>{}) : go(GenPol<true, false, 2>{});
    }
    if (var) return clamp ? go(GenPol<false, true, 1>{}) : go(GenPol<false, true, 2>{});
    return clamp ? go(GenPol<false, false, 1>{}) : go(GenPol<false, false, 2>{});
}

}  // namespace taa_dev
