// resolve_tiled.cu - the tiled FP32 resolve form: the CTA pipeline of
// tiled_skeleton.cuh with the oracle's FP32 arithmetic.
//
// This unit is compiled with -fmad=false: every operation rounds as the FP32
// oracle's does, with fused multiply-adds only where the oracle has them (the
// second-moment chain, the Catmull-Rom accumulation) or where fusing provably
// cannot change a result (products by powers of two), so the tiled form gives
// the oracle's bits - the same bits as the plain form.
#include "tiled_skeleton.cuh"
#include "kernels.h"

namespace taa_dev {
namespace {

using tiled::C3;
using tiled::Taps;

struct ExactF32 {
    using Staged = float4;
    struct Box {
        C3 c0, mn, mx, ct;
    };
    // the staged centre texel already is the exact current colour
    static constexpr bool kExactCentre = false;
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
    static __device__ __forceinline__ void box(const float4* nb, int ns, const tiled::Mode<HOT>& M, float g, Box& b) {
        auto ld = [&](int o) { float4 t = nb[o]; return C3{t.x, t.y, t.z}; };
        const C3 c0 = ld(0), c1 = ld(-ns - 1), c2 = ld(-ns), c3 = ld(-ns + 1), c4 = ld(-1), c5 = ld(1),
                 c6 = ld(ns - 1), c7 = ld(ns), c8 = ld(ns + 1);
        b.c0 = c0;
        b.ct = c0;
        if (M.variance()) {
            const float N = 9.0f, rN = 1.0f / 9.0f;
            auto ch = [&](float p0, float p1, float p2, float p3, float p4, float p5, float p6, float p7, float p8,
                          float& lo, float& hi, float& mean) {
                float m1 = p0 + p1 + p2 + p3 + p4 + p5 + p6 + p7 + p8;
                float m2 = __fmul_rn(p0, p0);
                m2 = __fmaf_rn(p1, p1, m2); m2 = __fmaf_rn(p2, p2, m2); m2 = __fmaf_rn(p3, p3, m2);
                m2 = __fmaf_rn(p4, p4, m2); m2 = __fmaf_rn(p5, p5, m2); m2 = __fmaf_rn(p6, p6, m2);
                m2 = __fmaf_rn(p7, p7, m2); m2 = __fmaf_rn(p8, p8, m2);
                mean = div_const_rn(m1, N, rN);
                float var = __fmaf_rn(-mean, mean, div_const_rn(m2, N, rN));
                float s = g * sqrtf(gmax(0.f, var));
                lo = mean - s;
                hi = mean + s;
            };
            ch(c0.x, c1.x, c2.x, c3.x, c4.x, c5.x, c6.x, c7.x, c8.x, b.mn.x, b.mx.x, b.ct.x);
            ch(c0.y, c1.y, c2.y, c3.y, c4.y, c5.y, c6.y, c7.y, c8.y, b.mn.y, b.mx.y, b.ct.y);
            ch(c0.z, c1.z, c2.z, c3.z, c4.z, c5.z, c6.z, c7.z, c8.z, b.mn.z, b.mx.z, b.ct.z);
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

    // taa.comp:441-514 as the 16-tap form
    static __device__ __forceinline__ void catmullrom_taps(float u, float v, int w, int h, Taps& t) {
        float itx = u * (float)w, ity = v * (float)h;
        float bx = floorf(itx - 0.5f), by = floorf(ity - 0.5f);
        float fx = itx - (bx + 0.5f), fy = ity - (by + 0.5f);
        {
            float f2 = fx * fx, f3 = f2 * fx;
            t.wx[0] = -0.5f * f3 + f2 - 0.5f * fx;
            t.wx[1] = 1.5f * f3 - 2.5f * f2 + 1.0f;
            t.wx[2] = -1.5f * f3 + 2.0f * f2 + 0.5f * fx;
            t.wx[3] = 0.5f * f3 - 0.5f * f2;
        }
        {
            float f2 = fy * fy, f3 = f2 * fy;
            t.wy[0] = -0.5f * f3 + f2 - 0.5f * fy;
            t.wy[1] = 1.5f * f3 - 2.5f * f2 + 1.0f;
            t.wy[2] = -1.5f * f3 + 2.0f * f2 + 0.5f * fy;
            t.wy[3] = 0.5f * f3 - 0.5f * f2;
        }
        int kx = trunc_index(bx), ky = trunc_index(by);
        t.ux = kx - 1;
        t.uy = ky - 1;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            t.xs[i] = clampi(kx - 1 + i, 0, w - 1);
            t.ys[i] = clampi(ky - 1 + i, 0, h - 1);
        }
    }
    // exact-weight bilinear (taa.comp:546)
    static __device__ __forceinline__ void bilinear_taps(float u, float v, int w, int h, Taps& t) {
        float px = u * (float)w - 0.5f, py = v * (float)h - 0.5f;
        float fx0 = floorf(px), fy0 = floorf(py);
        float fx = px - fx0, fy = py - fy0;
        if (!(fx == fx)) fx = 0.f;
        if (!(fy == fy)) fy = 0.f;
        int x0 = trunc_index(fx0), y0 = trunc_index(fy0);
        t.ux = x0;
        t.uy = y0;
        t.xs[0] = clampi(x0, 0, w - 1);
        t.xs[1] = clampi(x0 + 1 < x0 ? x0 : x0 + 1, 0, w - 1);
        t.ys[0] = clampi(y0, 0, h - 1);
        t.ys[1] = clampi(y0 + 1 < y0 ? y0 : y0 + 1, 0, h - 1);
        t.wx[0] = 1.0f - fx;
        t.wx[1] = fx;
        t.wy[0] = 1.0f - fy;
        t.wy[1] = fy;
    }
    // taa.comp:517-537: positions and combination weights of the four bilinear taps
    static __device__ __forceinline__ void bspline_positions(float u, float v, int w, int h, float s0[2], float s1[2],
                                                             float t0[2], float t1[2]) {
        float it[2] = {u * (float)w, v * (float)h};
        float inv[2] = {1.0f / (float)w, 1.0f / (float)h};
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
    }

    template <class F>
    static __device__ __forceinline__ float4 bil(const Taps& t, F&& texel) {
        float4 A = texel(t.xs[0], t.ys[0]), B = texel(t.xs[1], t.ys[0]);
        float4 C = texel(t.xs[0], t.ys[1]), D = texel(t.xs[1], t.ys[1]);
        float gx = t.wx[0], fx = t.wx[1], gy = t.wy[0], fy = t.wy[1];
        float4 tt = make_float4(A.x * gx + B.x * fx, A.y * gx + B.y * fx, A.z * gx + B.z * fx, 0.f);
        float4 bb = make_float4(C.x * gx + D.x * fx, C.y * gx + D.y * fx, C.z * gx + D.z * fx, 0.f);
        return make_float4(tt.x * gy + bb.x * fy, tt.y * gy + bb.y * fy, tt.z * gy + bb.z * fy, 0.f);
    }

    // the same filter reading 4x4 (or 2x2) consecutive window entries
    template <int INTERP, int HF, class HT>
    static __device__ __forceinline__ float4 filter_window(const tiled::HistoryTaps<ExactF32, INTERP>& h, const HT* base,
                                                           int stride) {
        const Taps& t = h.t[0];
        auto at = [&](int i, int j) { return tiled::to_f4<HF>(base[j * stride + i]); };
        if (INTERP == 2) {
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float rx = 0.f, ry = 0.f, rz = 0.f;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    float4 s = at(i, j);
                    rx = __fmaf_rn(t.wx[i], s.x, rx);
                    ry = __fmaf_rn(t.wx[i], s.y, ry);
                    rz = __fmaf_rn(t.wx[i], s.z, rz);
                }
                acc.x = __fmaf_rn(t.wy[j], rx, acc.x);
                acc.y = __fmaf_rn(t.wy[j], ry, acc.y);
                acc.z = __fmaf_rn(t.wy[j], rz, acc.z);
            }
            return acc;
        }
        float4 A = at(0, 0), B = at(1, 0), C = at(0, 1), D = at(1, 1);
        float gx = t.wx[0], fx = t.wx[1], gy = t.wy[0], fy = t.wy[1];
        float4 tt = make_float4(A.x * gx + B.x * fx, A.y * gx + B.y * fx, A.z * gx + B.z * fx, 0.f);
        float4 bb = make_float4(C.x * gx + D.x * fx, C.y * gx + D.y * fx, C.z * gx + D.z * fx, 0.f);
        return make_float4(tt.x * gy + bb.x * fy, tt.y * gy + bb.y * fy, tt.z * gy + bb.z * fy, 0.f);
    }

    template <int INTERP, class F>
    static __device__ __forceinline__ float4 filter(const tiled::HistoryTaps<ExactF32, INTERP>& h, F&& texel) {
        if (INTERP == 2) {
            const Taps& t = h.t[0];
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float rx = 0.f, ry = 0.f, rz = 0.f;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    float4 s = texel(t.xs[i], t.ys[j]);
                    rx = __fmaf_rn(t.wx[i], s.x, rx);
                    ry = __fmaf_rn(t.wx[i], s.y, ry);
                    rz = __fmaf_rn(t.wx[i], s.z, rz);
                }
                acc.x = __fmaf_rn(t.wy[j], rx, acc.x);
                acc.y = __fmaf_rn(t.wy[j], ry, acc.y);
                acc.z = __fmaf_rn(t.wy[j], rz, acc.z);
            }
            return acc;
        }
        if (INTERP == 0) return bil(h.t[0], texel);
        float4 A = bil(h.t[0], texel), B = bil(h.t[1], texel), C = bil(h.t[2], texel), D = bil(h.t[3], texel);
        const float *s0 = h.s0, *s1 = h.s1;
        return make_float4((A.x * s0[0] + B.x * s1[0]) * s0[1] + (C.x * s0[0] + D.x * s1[0]) * s1[1],
                           (A.y * s0[0] + B.y * s1[0]) * s0[1] + (C.y * s0[0] + D.y * s1[0]) * s1[1],
                           (A.z * s0[0] + B.z * s1[0]) * s0[1] + (C.z * s0[0] + D.z * s1[0]) * s1[1], 0.f);
    }

    // taa.comp:825-900: rectification and blend; returns the RGB result
    template <bool HOT>
    static __device__ __forceinline__ float4 finish(const taa_uniforms_t& U, const taa_parameters_t& P,
                                                    const tiled::Mode<HOT>& M, const Box& b, float4 hraw, float u,
                                                    float v, float hu, float hv, bool rejected) {
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
                float lc = lum(b.c0), lh = lum(hc);
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
        float t = 1.0f - alpha;
        const C3& c0 = b.c0;
        C3 o{hc.x * t + c0.x * alpha, hc.y * t + c0.y * alpha, hc.z * t + c0.z * alpha};
        if (yc) {
            float tmp = o.x - o.z;
            o = {tmp + o.y, o.x + o.z, tmp - o.y};
        }
        return make_float4(o.x, o.y, o.z, 0.f);
    }

    static __device__ __forceinline__ float4 un_tonemap(float4 o) {
        float l = 1.0f - gmax(gmax(o.x, o.y), o.z);
        return make_float4(o.x / l, o.y / l, o.z / l, o.w);
    }
};

}  // namespace

cudaError_t launch_resolve_tiled(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U,
                                 const FrameArgs& a, cudaStream_t s) {
    return tiled::launch_form<ExactF32>(history_fmt, motion_ch, interp, U, a, s);
}

}  // namespace taa_dev
