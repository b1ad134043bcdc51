// history_filter.cuh - the history sample of taa.comp (sample_history_rgba,
// taa.comp:441-549) on explicit texel taps, shared by the tiled forms.
//
// Catmull-Rom is evaluated as its 16-tap form (taa.comp:469-495), which the
// shader's 9-tap bilinear trick equals under an exact sampler; bilinear is one
// exact-weight 2x2 set; the "b-spline" is four 2x2 sets at the shader's
// positions combined with its weights.  Rounding follows the compilation unit:
// resolve_tiled.cu compiles this with -fmad=false and explicit FMAs where the
// oracle has them (the Catmull-Rom accumulation), so it gives the oracle's bits.
#pragma once
#include "tiled_skeleton.cuh"

namespace taa_dev {
namespace tiled {

struct HistoryFilter {
    // taa.comp:441-514: weights and the first (unclamped) tap of the 4x4 footprint
    static __device__ __forceinline__ void catmullrom_taps(float u, float v, int w, int h, Taps& t, f2 /*z*/) {
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
        t.ux = trunc_index(bx) - 1;
        t.uy = trunc_index(by) - 1;
    }
    // exact-weight bilinear (taa.comp:546)
    static __device__ __forceinline__ void bilinear_taps(float u, float v, int w, int h, Taps& t) {
        float px = u * (float)w - 0.5f, py = v * (float)h - 0.5f;
        float fx0 = floorf(px), fy0 = floorf(py);
        float fx = px - fx0, fy = py - fy0;
        if (!(fx == fx)) fx = 0.f;
        if (!(fy == fy)) fy = 0.f;
        t.ux = trunc_index(fx0);
        t.uy = trunc_index(fy0);
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

    // one exact-weight 2x2 set read through texel(x, y) at clamped coordinates;
    // W4: the fourth channel too (the history's dynamic mask), else 0
    template <bool W4 = false, class F>
    static __device__ __forceinline__ float4 bil(const Taps& t, int w, int h, F&& texel) {
        const int xa = t.xs(0, w), xb = t.xs(1, w), ya = t.ys(0, h), yb = t.ys(1, h);
        float4 A = texel(xa, ya), B = texel(xb, ya);
        float4 C = texel(xa, yb), D = texel(xb, yb);
        return bil_weights<W4>(t, A, B, C, D);
    }
    template <bool W4>
    static __device__ __forceinline__ float4 bil_weights(const Taps& t, float4 A, float4 B, float4 C, float4 D) {
        float gx = t.wx[0], fx = t.wx[1], gy = t.wy[0], fy = t.wy[1];
        float4 tt = make_float4(A.x * gx + B.x * fx, A.y * gx + B.y * fx, A.z * gx + B.z * fx,
                                W4 ? A.w * gx + B.w * fx : 0.f);
        float4 bb = make_float4(C.x * gx + D.x * fx, C.y * gx + D.y * fx, C.z * gx + D.z * fx,
                                W4 ? C.w * gx + D.w * fx : 0.f);
        return make_float4(tt.x * gy + bb.x * fy, tt.y * gy + bb.y * fy, tt.z * gy + bb.z * fy,
                           W4 ? tt.w * gy + bb.w * fy : 0.f);
    }

    // The Catmull-Rom accumulation: rows of four taps, then the rows (W4: the
    // fourth channel too).
    template <bool W4 = false, class F>
    static __device__ __forceinline__ float4 catmullrom_sum(const Taps& t, F&& at) {
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float rx = 0.f, ry = 0.f, rz = 0.f, rw = 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                float4 s = at(i, j);
                rx = __fmaf_rn(t.wx[i], s.x, rx);
                ry = __fmaf_rn(t.wx[i], s.y, ry);
                rz = __fmaf_rn(t.wx[i], s.z, rz);
                if (W4) rw = __fmaf_rn(t.wx[i], s.w, rw);
            }
            acc.x = __fmaf_rn(t.wy[j], rx, acc.x);
            acc.y = __fmaf_rn(t.wy[j], ry, acc.y);
            acc.z = __fmaf_rn(t.wy[j], rz, acc.z);
            if (W4) acc.w = __fmaf_rn(t.wy[j], rw, acc.w);
        }
        return acc;
    }

    // the filter reading 4x4 (or 2x2) consecutive window entries from `base`
    template <int INTERP, int HF, bool W4 = false, class Taps_, class HT>
    static __device__ __forceinline__ float4 filter_window(const Taps_& h, const HT* base, int stride) {
        const Taps& t = h.t[0];
        auto at = [&](int i, int j) { return to_f4<HF>(base[j * stride + i]); };
        if (INTERP == 2) return catmullrom_sum<W4>(t, at);
        return bil_weights<W4>(t, at(0, 0), at(1, 0), at(0, 1), at(1, 1));
    }

    // the filter reading texel(x, y) at clamped coordinates of a w x h image
    template <int INTERP, bool W4 = false, class Taps_, class F>
    static __device__ __forceinline__ float4 filter(const Taps_& h, int w, int hh, F&& texel) {
        if (INTERP == 2) {
            const Taps& t = h.t[0];
            int xs[4], ys[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                xs[k] = t.xs(k, w);
                ys[k] = t.ys(k, hh);
            }
            return catmullrom_sum<W4>(t, [&](int i, int j) { return texel(xs[i], ys[j]); });
        }
        if (INTERP == 0) return bil<W4>(h.t[0], w, hh, texel);
        float4 A = bil<W4>(h.t[0], w, hh, texel), B = bil<W4>(h.t[1], w, hh, texel),
               C = bil<W4>(h.t[2], w, hh, texel), D = bil<W4>(h.t[3], w, hh, texel);
        const float *s0 = h.s0, *s1 = h.s1;
        return make_float4((A.x * s0[0] + B.x * s1[0]) * s0[1] + (C.x * s0[0] + D.x * s1[0]) * s1[1],
                           (A.y * s0[0] + B.y * s1[0]) * s0[1] + (C.y * s0[0] + D.y * s1[0]) * s1[1],
                           (A.z * s0[0] + B.z * s1[0]) * s0[1] + (C.z * s0[0] + D.z * s1[0]) * s1[1],
                           W4 ? (A.w * s0[0] + B.w * s1[0]) * s0[1] + (C.w * s0[0] + D.w * s1[0]) * s1[1] : 0.f);
    }
};

}  // namespace tiled
}  // namespace taa_dev
