// policy_f32.cuh - the exact FP32 arithmetic policy of the tiled resolve
// forms (see tiled_skeleton.cuh): the oracle's FP32 operations in its order.
//
// Units that include this are compiled with -fmad=false: every operation
// rounds as the FP32 oracle's does, with fused multiply-adds only where the
// oracle has them (the second-moment chain, the Catmull-Rom accumulation) or
// where fusing provably cannot change a result (products by powers of two),
// so the tiled form gives the oracle's bits - the same bits as the plain form.
// Independent channel and axis chains run as packed f32x2 pairs (f32x2.cuh),
// which round lane by lane exactly as the scalar operations.
#pragma once
#include "f32x2.cuh"
#include "history_filter.cuh"

namespace taa_dev {
namespace tiled {

struct ExactF32 : HistoryFilter {
    using Staged = float4;
    struct Box {
        C3 mn, mx, ct;
    };
    // the current colour for the blend: the staged centre texel, read again
    // when it is needed rather than held in registers across the window wait
    static __device__ __forceinline__ C3 centre(const Box&, const float4* staged_centre) {
        const float4 t = *staged_centre;
        return C3{t.x, t.y, t.z};
    }
    // the staged centre texel already is the exact current colour
    static constexpr bool kExactCentre = false;
    // the FP32 box needs no fallback
    static constexpr bool kExactFallback = false;
    // debug outputs (taa.comp:912-942): the box bounds and what finish records
    static constexpr bool kDebug = true;
    template <class B> static __device__ __forceinline__ void box_bounds(const B& b, float3& mn, float3& mx) {
        mn = make_float3(b.mn.x, b.mn.y, b.mn.z);
        mx = make_float3(b.mx.x, b.mx.y, b.mx.z);
    }
    static __device__ __forceinline__ void centre_colour(Box&, const Img&, int, int, bool, bool) {}

    // working-space conversion of one source texel (taa.comp:182-213)
    static __device__ __forceinline__ float4 stage(uint2 raw, bool tonemap, bool ycocg) {
        float4 c = half4_to_float4(raw);
        if (tonemap) {
            float l = 1.0f + gmax(gmax(c.x, c.y), c.z);
            c.x = c.x / l;
            c.y = c.y / l;
            c.z = c.z / l;
        }
        if (ycocg) {
            // products by powers of two are exact: fusing rounds like the oracle's mul + add
            float y = __fmaf_rn(.25f, c.z, __fmaf_rn(.25f, c.x, .5f * c.y));
            float co = __fmaf_rn(-.5f, c.z, .5f * c.x);
            float cg = __fmaf_rn(-.25f, c.z, __fmaf_rn(-.25f, c.x, .5f * c.y));
            return make_float4(y, co, cg, 0.f);
        }
        return make_float4(c.x, c.y, c.z, 0.f);
    }

    // taa.comp:259-319 on the staged neighbourhood (nb points at the centre)
    template <bool HOT>
    static __device__ __forceinline__ void box(const float4* nb, int ns, const Mode<HOT>& M, float g, Box& b,
                                               f2 z) {
        auto ld = [&](int o) { float4 t = nb[o]; return C3{t.x, t.y, t.z}; };
        const C3 c0 = ld(0), c1 = ld(-ns - 1), c2 = ld(-ns), c3 = ld(-ns + 1), c4 = ld(-1), c5 = ld(1),
                 c6 = ld(ns - 1), c7 = ld(ns), c8 = ld(ns + 1);
        b.ct = c0;
        if (M.variance()) {
            // per channel: m1 = p0 + ... + p8 in tap order, m2 = p0^2 then FMAs,
            // mean = m1 / 9, var = m2 / 9 - mean^2 (one FMA); the channels run
            // two at a time as (Y, Co) and (Cg, 0) pairs
            const int off[9] = {0, -ns - 1, -ns, -ns + 1, -1, 1, ns - 1, ns, ns + 1};
            f2 pa, pb, m1a, m1b, m2a, m2b;
            load_pairs(&nb[0], m1a, m1b);
            m2a = mul2(m1a, m1a, z);
            m2b = mul2(m1b, m1b, z);
#pragma unroll
            for (int k = 1; k < 9; ++k) {
                load_pairs(&nb[off[k]], pa, pb);
                m1a = add2(m1a, pa);
                m1b = add2(m1b, pb);
                m2a = fma2(pa, pa, m2a);
                m2b = fma2(pb, pb, m2b);
            }
            const f2 nN = dup(-9.0f), rN = dup(1.0f / 9.0f);
            const f2 mean_a = div_const_rn2(m1a, nN, rN, z), mean_b = div_const_rn2(m1b, nN, rN, z);
            const f2 var_a = fma2(neg2(mean_a), mean_a, div_const_rn2(m2a, nN, rN, z));
            const f2 var_b = fma2(neg2(mean_b), mean_b, div_const_rn2(m2b, nN, rN, z));
            const f2 gg = dup(g);
            const f2 s_a = mul2(gg, pk(sqrtf(gmax(0.f, f2lo(var_a))), sqrtf(gmax(0.f, f2hi(var_a)))), z);
            const f2 s_b = mul2(gg, pk(sqrtf(gmax(0.f, f2lo(var_b))), 0.f), z);
            const f2 lo_a = sub2(mean_a, s_a), hi_a = add2(mean_a, s_a);
            const f2 lo_b = sub2(mean_b, s_b), hi_b = add2(mean_b, s_b);
            b.mn = {f2lo(lo_a), f2hi(lo_a), f2lo(lo_b)};
            b.mx = {f2lo(hi_a), f2hi(hi_a), f2lo(hi_b)};
            b.ct = {f2lo(mean_a), f2hi(mean_a), f2lo(mean_b)};
        } else {
            auto mn9 = [](float a0, float a1, float a2, float a3, float a4, float a5, float a6, float a7, float a8) {
                return gmin(gmin(gmin(gmin(gmin(gmin(gmin(gmin(a0, a1), a2), a3), a4), a5), a6), a7), a8);
            };
            auto mx9 = [](float a0, float a1, float a2, float a3, float a4, float a5, float a6, float a7, float a8) {
                return gmax(gmax(gmax(gmax(gmax(gmax(gmax(gmax(a0, a1), a2), a3), a4), a5), a6), a7), a8);
            };
            b.mn = {mn9(c0.x, c1.x, c2.x, c3.x, c4.x, c5.x, c6.x, c7.x, c8.x),
                    mn9(c0.y, c1.y, c2.y, c3.y, c4.y, c5.y, c6.y, c7.y, c8.y),
                    mn9(c0.z, c1.z, c2.z, c3.z, c4.z, c5.z, c6.z, c7.z, c8.z)};
            b.mx = {mx9(c0.x, c1.x, c2.x, c3.x, c4.x, c5.x, c6.x, c7.x, c8.x),
                    mx9(c0.y, c1.y, c2.y, c3.y, c4.y, c5.y, c6.y, c7.y, c8.y),
                    mx9(c0.z, c1.z, c2.z, c3.z, c4.z, c5.z, c6.z, c7.z, c8.z)};
            if (M.shaped()) {
                auto mn5 = [](float a0, float a2, float a4, float a5, float a7) { return gmin(gmin(gmin(gmin(a0, a2), a4), a5), a7); };
                auto mx5 = [](float a0, float a2, float a4, float a5, float a7) { return gmax(gmax(gmax(gmax(a0, a2), a4), a5), a7); };
                b.mn = {(b.mn.x + mn5(c0.x, c2.x, c4.x, c5.x, c7.x)) * 0.5f, (b.mn.y + mn5(c0.y, c2.y, c4.y, c5.y, c7.y)) * 0.5f,
                        (b.mn.z + mn5(c0.z, c2.z, c4.z, c5.z, c7.z)) * 0.5f};
                b.mx = {(b.mx.x + mx5(c0.x, c2.x, c4.x, c5.x, c7.x)) * 0.5f, (b.mx.y + mx5(c0.y, c2.y, c4.y, c5.y, c7.y)) * 0.5f,
                        (b.mx.z + mx5(c0.z, c2.z, c4.z, c5.z, c7.z)) * 0.5f};
            }
        }
        if (M.shrink()) {
            C3 hs{0.5f * (b.mx.x - b.mn.x), 0.25f * (b.mx.y - b.mn.y), 0.25f * (b.mx.z - b.mn.z)};
            C3 ce{(b.mn.x + b.mx.x) * 0.5f, (b.mn.y + b.mx.y) * 0.5f, (b.mn.z + b.mx.z) * 0.5f};
            b.mn = {ce.x - hs.x, ce.y - hs.y, ce.z - hs.z};
            b.mx = {ce.x + hs.x, ce.y + hs.y, ce.z + hs.z};
            const C3& t = b.ct;
            if (t.x < b.mn.x || t.y < b.mn.y || t.z < b.mn.z || t.x > b.mx.x || t.y > b.mx.y || t.z > b.mx.z) b.ct = ce;
        }
    }

    // taa.comp:426-430
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
        hu = (hs[0] / hs[3]) * 0.5f + 0.5f;
        hv = (hs[1] / hs[3]) * 0.5f + 0.5f;
        ehd = hs[2] / hs[3];
    }

    // taa.comp:441-514: the x and y axes of the Catmull-Rom weights as pairs
    static __device__ __forceinline__ void catmullrom_taps(float u, float v, int w, int h, Taps& t, f2 z) {
        const f2 it = mul2(pk(u, v), pk((float)w, (float)h), z);
        const f2 half = dup(0.5f);
        const f2 bf = pk(floorf(f2lo(it) - 0.5f), floorf(f2hi(it) - 0.5f));
        const f2 f = sub2(it, add2(bf, half));
        const f2 f2_ = mul2(f, f, z), f3 = mul2(f2_, f, z);
        const f2 hf = mul2(half, f, z);
        const f2 w0 = sub2(add2(mul2(dup(-0.5f), f3, z), f2_), hf);
        const f2 w1 = add2(sub2(mul2(dup(1.5f), f3, z), mul2(dup(2.5f), f2_, z)), dup(1.0f));
        const f2 w2 = add2(add2(mul2(dup(-1.5f), f3, z), mul2(dup(2.0f), f2_, z)), hf);
        const f2 w3 = sub2(mul2(half, f3, z), mul2(half, f2_, z));
        t.wx[0] = f2lo(w0); t.wy[0] = f2hi(w0);
        t.wx[1] = f2lo(w1); t.wy[1] = f2hi(w1);
        t.wx[2] = f2lo(w2); t.wy[2] = f2hi(w2);
        t.wx[3] = f2lo(w3); t.wy[3] = f2hi(w3);
        t.ux = trunc_index(f2lo(bf)) - 1;
        t.uy = trunc_index(f2hi(bf)) - 1;
    }

    // the window filter with each tap as two pairs (x, y), (z, w): a row sums
    // its four taps, then the rows are summed, both with one FMA per step
    template <int INTERP, int HF, bool W4 = false, class Taps_, class HT>
    static __device__ __forceinline__ float4 filter_window(const Taps_& h, const HT* base, int stride) {
        if constexpr (INTERP == 2 && HF == 0) {
            const Taps& t = h.t[0];
            const f2 zero = dup(0.f);
            f2 wxd[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) wxd[i] = dup(t.wx[i]);
            f2 acc_xy = zero, acc_zw = zero;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                f2 r_xy = zero, r_zw = zero;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    f2 s_xy, s_zw;
                    load_pairs(&base[j * stride + i], s_xy, s_zw);
                    r_xy = fma2(wxd[i], s_xy, r_xy);
                    r_zw = fma2(wxd[i], s_zw, r_zw);
                }
                const f2 wyd = dup(t.wy[j]);
                acc_xy = fma2(wyd, r_xy, acc_xy);
                acc_zw = fma2(wyd, r_zw, acc_zw);
            }
            return make_float4(f2lo(acc_xy), f2hi(acc_xy), f2lo(acc_zw), W4 ? f2hi(acc_zw) : 0.f);
        } else {
            return HistoryFilter::filter_window<INTERP, HF, W4>(h, base, stride);
        }
    }

    // taa.comp:825-900: rectification and blend; returns the RGB result.  UP:
    // the upsampling form's blend, mix(history, current, alpha * beta) with
    // beta = 1 on rejection and reset (beta 0: no source sample in the texel).
    template <bool HOT, bool UP = false>
    static __device__ __forceinline__ float4 finish(const taa_uniforms_t& U, const taa_parameters_t& P,
                                                    const Mode<HOT>& M, const Box& b, const C3& c0, float4 hraw, float u,
                                                    float v, float hu, float hv, bool rejected, float beta = 1.0f,
                                                    FinishOut* fo = nullptr) {
        const bool yc = M.ycocg();
        C3 hc{hraw.x, hraw.y, hraw.z};
        if (yc)
            hc = {.25f * hraw.x + .5f * hraw.y + .25f * hraw.z, .5f * hraw.x - .5f * hraw.z,
                  -.25f * hraw.x + .5f * hraw.y - .25f * hraw.z};
        const C3 orig = hc;
        const C3 &mn = b.mn, &mx = b.mx, &ct = b.ct;
        switch (M.clip()) {
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
        if (fo) fo->rdiff = make_float3(hc.x - orig.x, hc.y - orig.y, hc.z - orig.z);
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
                float lmn = lum(mn), lmx = lum(mx), lh = lum(orig);
                float dist = 2.0f * fabsf(gmin(lh - lmn, lmx - lh)) / (lmx - lmn);
                if (lmx - lmn < 0.001f) dist = 1.0f;
                alpha = alpha * gclamp(4.0f * dist, 0.f, 1.f);
            }
        }
        if (U.mResetHistory) alpha = 1.0f;
        if (fo) fo->alpha = alpha;
        if constexpr (UP) {
            if (rejected || U.mResetHistory) beta = 1.0f;
            alpha = alpha * beta;
        }
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
};


}  // namespace tiled
}  // namespace taa_dev
