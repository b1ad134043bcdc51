// taa_oracle.cpp - CPU restatement of shaders/taa.comp (test infrastructure).
//
// THIS IS THE ORACLE: only tests, the smoke check and the benchmark's CPU
// baseline use it, as the checker.  Sampler semantics and the FP32/FP64 split
// are described in taa_oracle.hpp.  Each function cites the shader lines it
// follows.  Build with -ffp-contract=off so the FP32 instance rounds every
// operation as written.
#include "taa_oracle.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace taa_oracle {
namespace {

// ---------------------------------------------------------------- vectors
template <class R> struct V2 { R x, y; };
template <class R> struct V3 { R x, y, z; };
template <class R> struct V4 { R x, y, z, w; };

template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> operator/(V3<R> a, V3<R> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline V3<R> operator+(V3<R> a, R s) { return {a.x + s, a.y + s, a.z + s}; }
template <class R> inline V3<R> splat3(R s) { return {s, s, s}; }
template <class R> inline V3<R> rgb(V4<R> v) { return {v.x, v.y, v.z}; }

// GLSL min/max/clamp on finite values (max(x,y) = x < y ? y : x).
template <class R> inline R gmax(R a, R b) { return a < b ? b : a; }
template <class R> inline R gmin(R a, R b) { return b < a ? b : a; }
template <class R> inline R gclamp(R x, R lo, R hi) { return gmin(gmax(x, lo), hi); }
template <class R> inline V3<R> vmin(V3<R> a, V3<R> b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
template <class R> inline V3<R> vmax(V3<R> a, V3<R> b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
template <class R> inline V3<R> vabs(V3<R> a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
template <class R> inline V3<R> vsqrt(V3<R> a) { return {std::sqrt(a.x), std::sqrt(a.y), std::sqrt(a.z)}; }
template <class R> inline V3<R> vfma(V3<R> a, V3<R> b, V3<R> c) {
    return {std::fma(a.x, b.x, c.x), std::fma(a.y, b.y, c.y), std::fma(a.z, b.z, c.z)};
}
// mix(x, y, a) = x*(1-a) + y*a (GLSL spec).
template <class R> inline R gmix(R x, R y, R a) { return x * (R(1) - a) + y * a; }
template <class R> inline V3<R> vmix(V3<R> x, V3<R> y, R a) {
    R t = R(1) - a;
    return {x.x * t + y.x * a, x.y * t + y.y * a, x.z * t + y.z * a};
}
template <class R> inline R fract(R x) { return x - std::floor(x); }

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Float-to-int truncation as ivec2(float) does, made total: NaN and values
// below 0 give 0 or a negative index that the caller clamps; huge values are
// held below INT_MAX.
template <class R> inline int trunc_index(R t) {
    if (!(t > R(-1e9))) return -1000000000;
    if (t > R(1e9)) return 1000000000;
    return (int)t;
}

// --------------------------------------------------------------- sampler
template <class R> V4<R> fetch(const ImageF& t, int x, int y) {
    if (!t.p) return {R(0), R(0), R(0), R(0)};
    x = clampi(x, 0, t.w - 1);
    y = clampi(y, 0, t.h - 1);
    const float* q = t.p + ((size_t)y * t.w + x) * t.ch;
    V4<R> r{R(q[0]), R(0), R(0), R(0)};
    if (t.ch > 1) r.y = R(q[1]);
    if (t.ch > 2) r.z = R(q[2]);
    if (t.ch > 3) r.w = R(q[3]);
    return r;
}

// Exact-weight bilinear, clamp to edge, texel centres at k+0.5.
template <class R> V4<R> bilinear(const ImageF& t, V2<R> uv) {
    if (!t.p) return {R(0), R(0), R(0), R(0)};
    R px = uv.x * R(t.w) - R(0.5);
    R py = uv.y * R(t.h) - R(0.5);
    R fx0 = std::floor(px), fy0 = std::floor(py);
    R fx = px - fx0, fy = py - fy0;
    int x0 = trunc_index(fx0), y0 = trunc_index(fy0);
    if (!(fx == fx)) fx = R(0);
    if (!(fy == fy)) fy = R(0);
    int xa = clampi(x0, 0, t.w - 1), xb = clampi(x0 + 1 < x0 ? x0 : x0 + 1, 0, t.w - 1);
    int ya = clampi(y0, 0, t.h - 1), yb = clampi(y0 + 1 < y0 ? y0 : y0 + 1, 0, t.h - 1);
    V4<R> a = fetch<R>(t, xa, ya), b = fetch<R>(t, xb, ya);
    V4<R> c = fetch<R>(t, xa, yb), d = fetch<R>(t, xb, yb);
    R gx = R(1) - fx, gy = R(1) - fy;
    V4<R> top{a.x * gx + b.x * fx, a.y * gx + b.y * fx, a.z * gx + b.z * fx, a.w * gx + b.w * fx};
    V4<R> bot{c.x * gx + d.x * fx, c.y * gx + d.y * fx, c.z * gx + d.z * fx, c.w * gx + d.w * fx};
    return {top.x * gy + bot.x * fy, top.y * gy + bot.y * fy, top.z * gy + bot.z * fy, top.w * gy + bot.w * fy};
}

// --------------------------------------------------------------- resolver
template <class R> struct Resolver {
    const taa_uniforms_t& U;
    const ResolveInputs& in;
    const ResolveOutputs& out;
    int loW, loH, hiW, hiH;
    bool same;  // source and target sizes equal: hi-res centres are lo-res centres

    // per-invocation state (the shader's globals)
    const taa_parameters_t* P = nullptr;

    Resolver(const taa_uniforms_t& u, const ResolveInputs& i, const ResolveOutputs& o)
        : U(u), in(i), out(o), loW(i.color.w), loH(i.color.h), hiW(i.out_w), hiH(i.out_h),
          same(i.color.w == i.out_w && i.color.h == i.out_h) {}

    // taa.comp:158-179
    V3<R> rgb_to_ycocg(V3<R> c) const {
        return {R(.25) * c.x + R(.5) * c.y + R(.25) * c.z,
                R(.5) * c.x - R(.5) * c.z,
                R(-.25) * c.x + R(.5) * c.y - R(.25) * c.z};
    }
    V3<R> ycocg_to_rgb(V3<R> c) const {
        R tmp = c.x - c.z;
        return {tmp + c.y, c.x + c.z, tmp - c.y};
    }
    V3<R> maybe_rgb_to_ycocg(V3<R> c) const { return P->mUseYCoCg ? rgb_to_ycocg(c) : c; }
    V3<R> maybe_ycocg_to_rgb(V3<R> c) const { return P->mUseYCoCg ? ycocg_to_rgb(c) : c; }
    R luminance(V3<R> c) const { return P->mUseYCoCg ? c.x : rgb_to_ycocg(c).x; }

    // taa.comp:182-197
    V3<R> tonemap_rgb(V3<R> hdr) const {
        if (P->mToneMapLumaKaris) {
            R luma = gmax(gmax(hdr.x, hdr.y), hdr.z);
            return hdr / (R(1.0) + luma);
        }
        return hdr;
    }
    V3<R> un_tonemap_rgb(V3<R> ldr) const {
        if (P->mToneMapLumaKaris) {
            R luma = gmax(gmax(ldr.x, ldr.y), ldr.z);
            return ldr / (R(1.0) - luma);
        }
        return ldr;
    }

    // JITTER_UV, taa.comp:47
    V2<R> jitter_uv() const {
        return {R(U.mJitterNdc[0]) * R(0.5) * R(P->mUnjitterFactor),
                R(U.mJitterNdc[1]) * R(0.5) * R(P->mUnjitterFactor)};
    }

    // texture(uCurrentFrame, offset + vec2(iuv + d + 0.5) * invsize), taa.comp:199-220
    V3<R> color_tap(int ix, int iy, V2<R> offset) const {
        if (offset.x == R(0) && offset.y == R(0)) return rgb(fetch<R>(in.color, ix, iy));
        R invx = R(1) / R(loW), invy = R(1) / R(loH);
        V2<R> uv{offset.x + (R(ix) + R(0.5)) * invx, offset.y + (R(iy) + R(0.5)) * invy};
        return rgb(bilinear<R>(in.color, uv));
    }
    V3<R> load_color(int ix, int iy, V2<R> offset) const {
        return maybe_rgb_to_ycocg(tonemap_rgb(color_tap(ix, iy, offset)));
    }

    // taa.comp:216-220
    V3<R> getCurrentColor(int ix, int iy) const {
        V2<R> off = P->mUnjitterCurrentSample ? jitter_uv() : V2<R>{R(0), R(0)};
        return load_color(ix, iy, off);
    }

    // taa.comp:222-257
    V3<R> getCurrentUpsampledColor(int tx, int ty, R& beta) const {
        V2<R> scale{R(hiW) / R(loW), R(hiH) / R(loH)};
        V2<R> ju = jitter_uv();
        V2<R> texelJitter{ju.x * R(loW) * R(-1), ju.y * R(loH) * R(-1)};
        V2<R> foundTc{R(-1), R(-1)};
        const R almostOne = R(0.999999);
        const R ox[4] = {R(0), almostOne, R(0), almostOne};
        const R oy[4] = {R(0), R(0), almostOne, almostOne};
        for (int k = 0; k < 4; ++k) {
            V2<R> s{std::floor(R(loW) * (R(tx) + ox[k]) / R(hiW)) + R(0.5) + texelJitter.x,
                    std::floor(R(loH) * (R(ty) + oy[k]) / R(hiH)) + R(0.5) + texelJitter.y};
            if (trunc_index(s.x * scale.x) == tx && trunc_index(s.y * scale.y) == ty) foundTc = s;
        }
        if (foundTc.x >= R(0.0)) {
            beta = R(1.0);
            // (floor(foundTc) + 0.5) / loRes is a source texel centre
            return maybe_rgb_to_ycocg(tonemap_rgb(rgb(fetch<R>(
                in.color, trunc_index(std::floor(foundTc.x)), trunc_index(std::floor(foundTc.y))))));
        }
        beta = R(0.0);
        return {R(0), R(0), R(0)};
    }

    // taa.comp:259-319
    void getColorAndAabb(int ix, int iy, V3<R>& centerCol, V3<R>& minCol, V3<R>& maxCol,
                         V3<R>& cliptowards) const {
        const R N = R(9.0);
        V2<R> off = P->mUnjitterNeighbourhood ? jitter_uv() : V2<R>{R(0), R(0)};
        centerCol = load_color(ix, iy, off);
        V3<R> c1 = load_color(ix - 1, iy - 1, off);
        V3<R> c2 = load_color(ix + 0, iy - 1, off);
        V3<R> c3 = load_color(ix + 1, iy - 1, off);
        V3<R> c4 = load_color(ix - 1, iy + 0, off);
        V3<R> c5 = load_color(ix + 1, iy + 0, off);
        V3<R> c6 = load_color(ix - 1, iy + 1, off);
        V3<R> c7 = load_color(ix + 0, iy + 1, off);
        V3<R> c8 = load_color(ix + 1, iy + 1, off);

        if (P->mVarianceClipping) {
            V3<R> m1 = centerCol + c1 + c2 + c3 + c4 + c5 + c6 + c7 + c8;
            // second moment as a fused chain in source order
            V3<R> m2 = centerCol * centerCol;
            m2 = vfma(c1, c1, m2); m2 = vfma(c2, c2, m2); m2 = vfma(c3, c3, m2);
            m2 = vfma(c4, c4, m2); m2 = vfma(c5, c5, m2); m2 = vfma(c6, c6, m2);
            m2 = vfma(c7, c7, m2); m2 = vfma(c8, c8, m2);
            V3<R> mean = m1 / N;
            V3<R> var = vfma(V3<R>{-mean.x, -mean.y, -mean.z}, mean, m2 / N);
            V3<R> sigma = vsqrt(vmax(splat3(R(0)), var));
            R g = R(P->mVarClipGamma);
            minCol = mean - g * sigma;
            maxCol = mean + g * sigma;
            cliptowards = mean;
        } else if (P->mShapedNeighbourhood) {
            V3<R> mn3 = vmin(vmin(vmin(vmin(vmin(vmin(vmin(vmin(centerCol, c1), c2), c3), c4), c5), c6), c7), c8);
            V3<R> mx3 = vmax(vmax(vmax(vmax(vmax(vmax(vmax(vmax(centerCol, c1), c2), c3), c4), c5), c6), c7), c8);
            V3<R> mn5 = vmin(vmin(vmin(vmin(centerCol, c2), c4), c5), c7);
            V3<R> mx5 = vmax(vmax(vmax(vmax(centerCol, c2), c4), c5), c7);
            minCol = (mn3 + mn5) * R(0.5);
            maxCol = (mx3 + mx5) * R(0.5);
            cliptowards = centerCol;
        } else {
            minCol = vmin(vmin(vmin(vmin(vmin(vmin(vmin(vmin(centerCol, c1), c2), c3), c4), c5), c6), c7), c8);
            maxCol = vmax(vmax(vmax(vmax(vmax(vmax(vmax(vmax(centerCol, c1), c2), c3), c4), c5), c6), c7), c8);
            cliptowards = centerCol;
        }

        if (P->mUseYCoCg && P->mShrinkChromaAxis) {
            const V3<R> scaleYCoCg{R(1.0), R(0.5), R(0.5)};
            V3<R> halfSize = (R(0.5) * scaleYCoCg) * (maxCol - minCol);
            V3<R> center = (minCol + maxCol) * R(0.5);
            minCol = center - halfSize;
            maxCol = center + halfSize;
            bool out = cliptowards.x < minCol.x || cliptowards.y < minCol.y || cliptowards.z < minCol.z ||
                       cliptowards.x > maxCol.x || cliptowards.y > maxCol.y || cliptowards.z > maxCol.z;
            if (out) cliptowards = center;
        }
    }

    // taa.comp:323-345 with p = (0,0,0,1), q = (hist, 1)
    V3<R> clipAabb(V3<R> aabbMin, V3<R> aabbMax, V3<R> q) const {
        const R eps = R(1e-7f);
        V3<R> pClip = R(0.5) * (aabbMax + aabbMin);
        V3<R> eClip = R(0.5) * (aabbMax - aabbMin) + eps;
        V3<R> vClip = q - pClip;  // .w = 1 - 1 = 0
        V3<R> vUnit = vClip / eClip;
        V3<R> aUnit = vabs(vUnit);
        R maUnit = gmax(aUnit.x, gmax(aUnit.y, aUnit.z));
        if (maUnit > R(1.0)) return pClip + vClip / maUnit;
        return q;
    }

    // taa.comp:348-369 with p = (colClipTowards, 1), q = (hist, 1); .w of r stays 0
    V3<R> clipAabbSlow(V3<R> aabbMin, V3<R> aabbMax, V3<R> p, V3<R> q) const {
        V3<R> r = q - p;
        V3<R> rmax = aabbMax - p;
        V3<R> rmin = aabbMin - p;
        const R eps = R(1e-7f);
        if (r.x > rmax.x + eps) r = r * (rmax.x / r.x);
        if (r.y > rmax.y + eps) r = r * (rmax.y / r.y);
        if (r.z > rmax.z + eps) r = r * (rmax.z / r.z);
        if (r.x < rmin.x - eps) r = r * (rmin.x / r.x);
        if (r.y < rmin.y - eps) r = r * (rmin.y / r.y);
        if (r.z < rmin.z - eps) r = r * (rmin.z / r.z);
        return p + r;
    }

    // SAMPLE_TEX(tex, currentUv + toUv * d) for a lo-res-sized texture.
    V4<R> sample_at(const ImageF& t, int ix, int iy, V2<R> uv, int dx, int dy) const {
        if (same) return fetch<R>(t, ix + dx, iy + dy);
        V2<R> toUv{R(1) / R(t.w), R(1) / R(t.h)};
        return bilinear<R>(t, V2<R>{uv.x + toUv.x * R(dx), uv.y + toUv.y * R(dy)});
    }

    // taa.comp:391-438
    void getHistoryPosition(int ix, int iy, V2<R> currentUv, R currentDepth, V2<R>& historyUv,
                            R& historyDepth, R& speed) const {
        V4<R> vs = sample_at(in.velocity, ix, iy, currentUv, 0, 0);
        bool canUse = true;
        if (P->mUseVelocityVectors == 0 || (P->mUseVelocityVectors == 1 && vs.w < R(0.5))) canUse = false;
        if (canUse) {
            if (P->mVelocitySampleMode == 1) {
                // 3x3 longest; the reference keeps the last tap (taa.comp:412)
                V2<R> maxVel{vs.x, vs.y};
                const int ox[8] = {1, -1, -1, 0, -1, 0, 1, 1};
                const int oy[8] = {-1, 0, -1, -1, 1, 1, 0, 1};
                V2<R> sam{R(0), R(0)};
                for (int k = 0; k < 8; ++k) {
                    V4<R> s = sample_at(in.velocity, ix, iy, currentUv, ox[k], oy[k]);
                    sam = {s.x, s.y};
                    if (sam.x * sam.x + sam.y * sam.y > maxVel.x * maxVel.x + maxVel.y * maxVel.y) maxVel = sam;
                }
                vs.x = sam.x;
                vs.y = sam.y;
            } else if (P->mVelocitySampleMode == 2) {
                // findClosestUvAndZ_3x3, taa.comp:371-389
                const int ox[9] = {-1, 0, 1, -1, 0, 1, -1, 0, 1};
                const int oy[9] = {-1, -1, -1, 0, 0, 0, 1, 1, 1};
                int best = 0;
                R dClosest = sample_at(in.depth, ix, iy, currentUv, ox[0], oy[0]).x;
                for (int k = 1; k < 9; ++k) {
                    R d = sample_at(in.depth, ix, iy, currentUv, ox[k], oy[k]).x;
                    if (d < dClosest) { best = k; dClosest = d; }
                }
                if (same) {
                    vs = fetch<R>(in.velocity, ix + ox[best], iy + oy[best]);
                } else {
                    V2<R> toUv{R(1) / R(in.depth.w), R(1) / R(in.depth.h)};
                    vs = bilinear<R>(in.velocity, V2<R>{currentUv.x + toUv.x * R(ox[best]),
                                                        currentUv.y + toUv.y * R(oy[best])});
                }
            }
            historyUv = {currentUv.x - vs.x, currentUv.y - vs.y};
            historyDepth = currentDepth - vs.z;
        } else {
            R cs[4] = {currentUv.x * R(2.0) - R(1.0), currentUv.y * R(2.0) - R(1.0), currentDepth, R(1)};
            R ws[4], hs[4];
            const float* A = U.mInverseViewProjMatrix;
            const float* B = U.mHistoryViewProjMatrix;
            for (int i = 0; i < 4; ++i)
                ws[i] = R(A[0 * 4 + i]) * cs[0] + R(A[1 * 4 + i]) * cs[1] + R(A[2 * 4 + i]) * cs[2] + R(A[3 * 4 + i]) * cs[3];
            for (int i = 0; i < 4; ++i)
                hs[i] = R(B[0 * 4 + i]) * ws[0] + R(B[1 * 4 + i]) * ws[1] + R(B[2 * 4 + i]) * ws[2] + R(B[3 * 4 + i]) * ws[3];
            historyUv = {(hs[0] / hs[3]) * R(0.5) + R(0.5), (hs[1] / hs[3]) * R(0.5) + R(0.5)};
            historyDepth = hs[2] / hs[3];
        }
        V2<R> velUv{currentUv.x - historyUv.x, currentUv.y - historyUv.y};
        speed = std::sqrt(velUv.x * velUv.x + velUv.y * velUv.y);
    }

    // taa.comp:441-514, evaluated as the equivalent 16-tap form with edge clamp.
    V4<R> history_catmullrom(V2<R> uv) const {
        const ImageF& t = in.history;
        R sx = R(t.w), sy = R(t.h);
        R itx = uv.x * sx, ity = uv.y * sy;
        R tcx = std::floor(itx - R(0.5)) + R(0.5), tcy = std::floor(ity - R(0.5)) + R(0.5);
        R fx = itx - tcx, fy = ity - tcy;
        R wx[4], wy[4];
        auto weights = [](R f, R* w) {
            R f2 = f * f, f3 = f2 * f;
            w[0] = R(-0.5) * f3 + f2 - R(0.5) * f;
            w[1] = R(1.5) * f3 - R(2.5) * f2 + R(1.0);
            w[2] = R(-1.5) * f3 + R(2.0) * f2 + R(0.5) * f;
            w[3] = R(0.5) * f3 - R(0.5) * f2;
        };
        weights(fx, wx);
        weights(fy, wy);
        int kx = trunc_index(std::floor(itx - R(0.5)));
        int ky = trunc_index(std::floor(ity - R(0.5)));
        // rows first, then columns, each a fused multiply-add chain from zero
        V4<R> acc{R(0), R(0), R(0), R(0)};
        for (int j = 0; j < 4; ++j) {
            V4<R> row{R(0), R(0), R(0), R(0)};
            int yy = ky - 1 + j;
            for (int i = 0; i < 4; ++i) {
                V4<R> s = fetch<R>(t, kx - 1 + i, yy);
                row.x = std::fma(wx[i], s.x, row.x);
                row.y = std::fma(wx[i], s.y, row.y);
                row.z = std::fma(wx[i], s.z, row.z);
                row.w = std::fma(wx[i], s.w, row.w);
            }
            acc.x = std::fma(wy[j], row.x, acc.x);
            acc.y = std::fma(wy[j], row.y, acc.y);
            acc.z = std::fma(wy[j], row.z, acc.z);
            acc.w = std::fma(wy[j], row.w, acc.w);
        }
        return acc;
    }

    // taa.comp:517-543, literally: four exact bilinear taps.
    V4<R> history_bspline(V2<R> uv) const {
        const ImageF& t = in.history;
        R sx = R(t.w), sy = R(t.h);
        R ix = R(1) / sx, iy = R(1) / sy;
        R itx = uv.x * sx, ity = uv.y * sy;
        R tc[2] = {std::floor(itx - R(0.5)) + R(0.5), std::floor(ity - R(0.5)) + R(0.5)};
        R f[2] = {itx - tc[0], ity - tc[1]};
        R s0[2], s1[2], t0[2], t1[2];
        for (int a = 0; a < 2; ++a) {
            R ff = f[a], f2 = ff * ff, f3 = f2 * ff;
            R w0 = f2 - R(0.5) * (f3 + ff);
            R w1 = R(1.5) * f3 - R(2.5) * f2 + R(1.0);
            R w3 = R(0.5) * (f3 - f2);
            R w2 = R(1.0) - w0 - w1 - w3;
            s0[a] = w0 + w1;
            s1[a] = w2 + w3;
            R f0 = w1 / (w0 + w1);
            R f1 = w3 / (w2 + w3);
            R inv = a == 0 ? ix : iy;
            t0[a] = (tc[a] - R(1) + f0) * inv;
            t1[a] = (tc[a] + R(1) + f1) * inv;
        }
        V4<R> A = bilinear<R>(t, {t0[0], t0[1]}), B = bilinear<R>(t, {t1[0], t0[1]});
        V4<R> C = bilinear<R>(t, {t0[0], t1[1]}), D = bilinear<R>(t, {t1[0], t1[1]});
        V4<R> r;
        r.x = (A.x * s0[0] + B.x * s1[0]) * s0[1] + (C.x * s0[0] + D.x * s1[0]) * s1[1];
        r.y = (A.y * s0[0] + B.y * s1[0]) * s0[1] + (C.y * s0[0] + D.y * s1[0]) * s1[1];
        r.z = (A.z * s0[0] + B.z * s1[0]) * s0[1] + (C.z * s0[0] + D.z * s1[0]) * s1[1];
        r.w = (A.w * s0[0] + B.w * s1[0]) * s0[1] + (C.w * s0[0] + D.w * s1[0]) * s1[1];
        return r;
    }

    // taa.comp:545-549
    V4<R> sample_history_rgba(V2<R> uv) const {
        if (P->mInterpolationMode == 0) return bilinear<R>(in.history, uv);
        if (P->mInterpolationMode == 1) return history_bspline(uv);
        return history_catmullrom(uv);
    }

    // taa.comp:551-556
    V4<R> noise(V2<R> uv) const {
        V2<R> seed{uv.x + R(U.mSinTime[0]) + R(0.6959174), uv.y + R(U.mSinTime[0]) + R(0.6959174)};
        R s = std::sin(seed.x * R(12.9898) + seed.y * R(78.233));
        R n[4] = {fract(s * R(43758.5453)), fract(s * R(28001.8384)), fract(s * R(50849.4141)),
                  fract(s * R(12996.89))};
        R f = R(P->mNoiseFactor);
        return {(n[0] * R(2.0) - R(1.0)) * f, (n[1] * R(2.0) - R(1.0)) * f, (n[2] * R(2.0) - R(1.0)) * f,
                (n[3] * R(2.0) - R(1.0)) * f};
    }

    // taa.comp:559-580
    R linearize_depth(R d) const {
        R n = R(U.mCamNearPlane), f = R(U.mCamFarPlane);
        return n * f / (f + d * (n - f));
    }
    R sample_linear_depth(int x, int y) const { return linearize_depth(fetch<R>(in.depth, x, y).x); }
    R sample_luminance(int x, int y) const { return rgb_to_ycocg(rgb(fetch<R>(in.color, x, y))).x; }
    V3<R> sample_normal(int x, int y) const {
        V4<R> un = fetch<R>(in.uvnrm, x, y);
        return {std::cos(un.z) * std::cos(un.w), std::sin(un.z) * std::cos(un.w), std::sin(un.w)};
    }
    static V2<R> sobel(R c00, R c01, R c02, R c10, R c12, R c20, R c21, R c22) {
        return {c00 - c20 + R(2) * c01 - R(2) * c21 + c02 - c22, c00 - c02 + R(2) * c10 - R(2) * c12 + c20 - c22};
    }
    uint32_t load_u(const ImageU& t, int x, int y) const {
        if (!t.p) return 0u;
        return t.p[(size_t)clampi(y, 0, t.h - 1) * t.w + clampi(x, 0, t.w - 1)];
    }

    // taa.comp:589-702
    uint32_t calc_segmentation_value(int ix, int iy, V2<R> historyUv) const {
        const uint32_t flags = P->mRayTraceAugmentFlags;
        auto ctt_x = [&](int v) { return clampi(v, 0, loW - 1); };
        auto ctt_y = [&](int v) { return clampi(v, 0, loH - 1); };
        if (flags & TAA_RTFLAG_FXD) {
            const int b = 100;
            if (ix < b || iy < b || ix >= loW - b || iy >= loH - b) return 1;
        }
        if (flags & TAA_RTFLAG_ALL) return 2;
        bool useHistoryCount = (flags & TAA_RTFLAG_CNT) != 0;
        uint32_t newCountValue = useHistoryCount ? ((uint32_t)P->mRayTraceHistoryCount << 16) : 0u;
        if (flags & TAA_RTFLAG_OUT) {
            if (historyUv.x < R(0) || historyUv.y < R(0) || historyUv.x >= R(1) || historyUv.y >= R(1)) return 1;
        }
        uint32_t matId = load_u(in.material, ix, iy);
        if (flags & TAA_RTFLAG_DIS) {
            int tx = trunc_index(historyUv.x * R(loW)), ty = trunc_index(historyUv.y * R(loH));
            if (tx >= 0 && ty >= 0 && tx < loW && ty < loH) {
                uint32_t prevMatId = load_u(in.prev_material, tx, ty);
                if (prevMatId != matId && (prevMatId & 0x80000000u) != 0) return 2u | newCountValue;
            }
        }
        R nrmValue = R(0), dptValue = R(0), matValue = R(0), lumValue = R(0);
        if (flags & TAA_RTFLAG_NRM) {
            V3<R> nC = sample_normal(ix, iy);
            V3<R> nL = sample_normal(ctt_x(ix - 1), ctt_y(iy));
            V3<R> nR = sample_normal(ctt_x(ix + 1), ctt_y(iy));
            V3<R> nT = sample_normal(ctt_x(ix), ctt_y(iy - 1));
            V3<R> nB = sample_normal(ctt_x(ix), ctt_y(iy + 1));
            auto dot3 = [](V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; };
            R mind = gmax(R(0), gmin(gmin(gmin(dot3(nC, nL), dot3(nC, nR)), dot3(nC, nT)), dot3(nC, nB)));
            nrmValue = R(1.0) - mind;
        }
        auto len2 = [](V2<R> g) { return std::sqrt(g.x * g.x + g.y * g.y); };
        if (flags & TAA_RTFLAG_DPT) {
            auto L = [&](int dx, int dy) { return sample_linear_depth(ctt_x(ix + dx), ctt_y(iy + dy)); };
            dptValue = len2(sobel(L(-1, -1), L(0, -1), L(1, -1), L(-1, 0), L(1, 0), L(-1, 1), L(0, 1), L(1, 1)));
        }
        if (flags & TAA_RTFLAG_MID) {
            if (matId != load_u(in.material, ctt_x(ix - 1), ctt_y(iy)) ||
                matId != load_u(in.material, ctt_x(ix + 1), ctt_y(iy)) ||
                matId != load_u(in.material, ctt_x(ix), ctt_y(iy - 1)) ||
                matId != load_u(in.material, ctt_x(ix), ctt_y(iy + 1)))
                matValue = R(1.0);
        }
        if (flags & TAA_RTFLAG_LUM) {
            auto L = [&](int dx, int dy) { return sample_luminance(ctt_x(ix + dx), ctt_y(iy + dy)); };
            lumValue = len2(sobel(L(-1, -1), L(0, -1), L(1, -1), L(-1, 0), L(1, 0), L(-1, 1), L(0, 1), L(1, 1)));
        }
        R total = nrmValue * R(P->mRayTraceAugment_WNrm) + dptValue * R(P->mRayTraceAugment_WDpt) +
                  matValue * R(P->mRayTraceAugment_WMId) + lumValue * R(P->mRayTraceAugment_WLum);
        if (total >= R(P->mRayTraceAugment_Thresh)) return 2u | newCountValue;
        if (useHistoryCount) {
            uint32_t oldCnt = (load_u(in.prev_segmask, ix, iy) & 0xffff0000u) >> 16;
            if (oldCnt > 0) return 2u | ((oldCnt - 1) << 16);
        }
        return 0u;
    }

    static void put4(double* dst, size_t idx, V4<R> v) {
        if (!dst) return;
        dst[idx * 4 + 0] = double(v.x);
        dst[idx * 4 + 1] = double(v.y);
        dst[idx * 4 + 2] = double(v.z);
        dst[idx * 4 + 3] = double(v.w);
    }

    // taa.comp:708-960
    void pixel(int x, int y) {
        const size_t o = (size_t)y * hiW + x;
        V2<R> uv{(R(x) + R(0.5)) / R(hiW), (R(y) + R(0.5)) / R(hiH)};
        int pidx = (U.splitScreen && x > U.splitX) ? 1 : 0;
        P = &U.param[pidx];
        bool generateSegmentationMask = P->mRayTraceAugment != 0;
        int lx = trunc_index(uv.x * R(loW)), ly = trunc_index(uv.y * R(loH));

        if (P->mPassThrough) {
            V4<R> c = fetch<R>(in.color, lx, ly), h = fetch<R>(in.history, x, y);
            put4(out.screen, o, {c.x, c.y, c.z, R(1)});
            put4(out.history, o, {h.x, h.y, h.z, R(1)});
            put4(out.debug, o, {R(0), R(0), R(0), R(0)});
            return;
        }
        if (U.mBypassHistoryUpdate) {
            V4<R> h = fetch<R>(in.history, x, y);
            put4(out.screen, o, {h.x, h.y, h.z, R(1)});
            put4(out.history, o, {h.x, h.y, h.z, R(1)});
            put4(out.debug, o, {R(0), R(0), R(0), R(0)});
            return;
        }

        bool rejected = false;
        V3<R> currentColor, colMin, colMax, colClipTowards;
        R beta;
        getColorAndAabb(lx, ly, currentColor, colMin, colMax, colClipTowards);
        if (U.mUpsampling) {
            currentColor = getCurrentUpsampledColor(x, y, beta);
        } else {
            currentColor = getCurrentColor(lx, ly);
            beta = R(1.0);
        }
        R depth = fetch<R>(in.depth, lx, ly).x;

        V2<R> historyUv;
        R expectedHistoryDepth, pixelSpeed;
        getHistoryPosition(lx, ly, uv, depth, historyUv, expectedHistoryDepth, pixelSpeed);

        V4<R> historyRaw = sample_history_rgba(historyUv);
        V3<R> historyColor = maybe_rgb_to_ycocg(rgb(historyRaw));
        R alpha = R(P->mAlpha);

        uint32_t segMaskValue = 0;
        if (generateSegmentationMask) {
            segMaskValue = calc_segmentation_value(x, y, historyUv);
            if ((segMaskValue & 3u) != 0) {
                alpha = R(P->mRejectionAlpha);
                rejected = true;
            }
        }

        if (P->mRejectOutside) {
            if (historyUv.x < R(0) || historyUv.y < R(0) || historyUv.x >= R(1) || historyUv.y >= R(1)) {
                alpha = R(P->mRejectionAlpha);
                rejected = true;
            }
        }
        R writeDynamicMask = R(0);
        if (P->mDynamicAntiGhosting) {
            const R eps = R(1e-5f);
            auto mov = [&](int dx, int dy) {
                V4<R> v = sample_at(in.velocity, lx, ly, uv, dx, dy);
                return (std::fabs(v.x) > eps || std::fabs(v.y) > eps) && (std::fabs(v.w) >= R(0.5));
            };
            bool movL = mov(-1, 0), movR = mov(1, 0), movT = mov(0, -1), movB = mov(0, 1), movC = mov(0, 0);
            bool movement = movL || movR || movT || movB || movC;
            if (!movement && historyRaw.w > R(0.0)) rejected = true;
            writeDynamicMask = movC ? R(1.0) : R(0.0);
        }
        if (P->mDepthCulling) {
            int tx = trunc_index(historyUv.x * R(loW)), ty = trunc_index(historyUv.y * R(loH));
            R historyDepth = fetch<R>(in.history_depth, tx, ty).x;
            R depthEpsilon = R(0.1) * (R(1.0) - historyDepth);
            if (std::fabs(historyDepth - expectedHistoryDepth) > depthEpsilon) rejected = true;
        }

        V3<R> origHistColor = historyColor;
        switch (P->mColorClampingOrClipping) {
            case 1: historyColor = vmin(vmax(historyColor, colMin), colMax); break;
            case 2: historyColor = clipAabb(colMin, colMax, historyColor); break;
            case 3: historyColor = clipAabbSlow(colMin, colMax, colClipTowards, historyColor); break;
            default: break;
        }
        V3<R> rectified_diff = historyColor - origHistColor;

        if (rejected) {
            alpha = R(P->mRejectionAlpha);
            beta = R(1.0);
        } else {
            if (P->mVelBasedAlpha) {
                alpha = gmax(alpha, gmix(alpha, R(P->mVelBasedAlphaMax),
                                         gclamp(pixelSpeed * R(P->mVelBasedAlphaFactor), R(0), R(1))));
            }
            if (P->mLumaWeightingLottes) {
                R lumaCurrent = luminance(currentColor);
                R lumaHistory = luminance(historyColor);
                R diff = std::fabs(lumaCurrent - lumaHistory) / gmax(gmax(lumaCurrent, lumaHistory), R(0.2));
                R w = R(1.0) - diff;
                R ww = w * w;
                alpha = gmix(R(P->mMaxAlpha), R(P->mMinAlpha), ww);
            }
            if (P->mReduceBlendNearClamp) {
                R colMin_lum = luminance(colMin);
                R colMax_lum = luminance(colMax);
                R history_lum = luminance(origHistColor);
                R distToClamp = R(2.0) * std::fabs(gmin(history_lum - colMin_lum, colMax_lum - history_lum)) /
                                (colMax_lum - colMin_lum);
                if (colMax_lum - colMin_lum < R(0.001)) distToClamp = R(1.0);
                alpha = alpha * gclamp(R(4) * distToClamp, R(0), R(1));
            }
        }
        if (U.mResetHistory) {
            alpha = R(1.0);
            beta = R(1.0);
        }

        V3<R> antiAliased = maybe_ycocg_to_rgb(vmix(historyColor, currentColor, alpha * beta));
        if (P->mAddNoise) {
            V4<R> n = noise(uv);
            antiAliased = antiAliased + V3<R>{n.x, n.y, n.z};
        }
        V4<R> to_history{antiAliased.x, antiAliased.y, antiAliased.z, writeDynamicMask};
        V3<R> scr = un_tonemap_rgb(antiAliased);
        V4<R> to_screen{scr.x, scr.y, scr.z, R(1.0)};

        if (out.debug) {
            V4<R> g{R(0), R(0), R(0), R(0)};
            switch (P->mDebugMode) {
                case 0: { V3<R> t = colMax - colMin; g = {t.x, t.y, t.z, R(0)}; break; }
                case 1: { V3<R> t = colMax - colMin; R v = t.x * t.y * t.z; g = {v, v, v, R(0)}; break; }
                case 2: {
                    R l = std::sqrt(rectified_diff.x * rectified_diff.x + rectified_diff.y * rectified_diff.y +
                                    rectified_diff.z * rectified_diff.z);
                    g = {rejected ? R(1) : R(0), l, R(0), R(0)};
                    break;
                }
                case 3: g = {alpha, alpha, alpha, R(0)}; break;
                case 4: g = fetch<R>(in.velocity, x, y); break;
                case 5: g = {pixelSpeed, R(0), R(0), R(0)}; break;
                case 6: g = to_screen; break;
                case 7: g = to_history; break;
                case 8:
                    switch (segMaskValue & 3u) {
                        case 0: g = {R(0), R(0), R(1), R(0)}; break;
                        case 1: g = {R(1), R(0), R(0), R(0)}; break;
                        case 2: g = {R(1), R(1), R(0), R(0)}; break;
                        default: break;
                    }
                    break;
                default: break;
            }
            R s = R(P->mDebugScale);
            g = {g.x * (s * R(P->mDebugMask[0])), g.y * (s * R(P->mDebugMask[1])),
                 g.z * (s * R(P->mDebugMask[2])), g.w * (s * R(P->mDebugMask[3]))};
            if (P->mDebugCenter)
                g = {g.x * R(0.5) + R(0.5), g.y * R(0.5) + R(0.5), g.z * R(0.5) + R(0.5), g.w * R(0.5) + R(0.5)};
            put4(out.debug, o, g);
        }
        put4(out.history, o, to_history);
        put4(out.screen, o, to_screen);
        if (generateSegmentationMask && out.segmask) out.segmask[o] = segMaskValue;
    }
};

template <class F> void parallel_rows(int h, int nthreads, F&& f) {
    if (nthreads <= 1 || h < 2) {
        for (int y = 0; y < h; ++y) f(y);
        return;
    }
    nthreads = std::min(nthreads, h);
    std::vector<std::thread> pool;
    pool.reserve(nthreads);
    for (int t = 0; t < nthreads; ++t)
        pool.emplace_back([&, t] {
            for (int y = t; y < h; y += nthreads) f(y);
        });
    for (auto& th : pool) th.join();
}

template <class R> void resolve_t(const taa_uniforms_t& u, const ResolveInputs& in, const ResolveOutputs& out,
                                  int nthreads) {
    parallel_rows(in.out_h, nthreads, [&](int y) {
        Resolver<R> r(u, in, out);
        for (int x = 0; x < in.out_w; ++x) r.pixel(x, y);
    });
}

// ---------------------------------------------------------------- CAS
inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
// ffx_a.h:1455-1457, defined on FP32 bit patterns.
inline float APrxLoSqrtF1(float a) { return bitsf((fbits(a) >> 1) + 0x1fbc4639u); }
inline float APrxLoRcpF1(float a) { return bitsf(0x7ef07ebbu - fbits(a)); }
template <class R> inline R APrxMedRcpF1(R a) {
    R b = R(bitsf(0x7ef19fffu - fbits(float(a))));
    return b * (-b * a + R(2.0));
}
template <class R> inline R ASat(R x) { return gclamp(x, R(0.0), R(1.0)); }

// ffx_cas.h:424-537 (no-scaling branch, without CAS_BETTER_DIAGONALS/CAS_GO_SLOWER/CAS_SLOW,
// as sharpen_cas.comp compiles it); loads clamp to the image.
template <class R> void cas_t(const float* in, int w, int h, uint32_t peak_bits, double* out, int nthreads) {
    const R peak = R(bitsf(peak_bits));
    parallel_rows(h, nthreads, [&](int y) {
        for (int x = 0; x < w; ++x) {
            auto L = [&](int dx, int dy) {
                int xx = clampi(x + dx, 0, w - 1), yy = clampi(y + dy, 0, h - 1);
                const float* q = in + ((size_t)yy * w + xx) * 4;
                return V3<R>{R(q[0]), R(q[1]), R(q[2])};
            };
            V3<R> b = L(0, -1), d = L(-1, 0), e = L(0, 0), f = L(1, 0), hh = L(0, 1);
            auto min3 = [](R a, R bb, R c) { return gmin(a, gmin(bb, c)); };
            auto max3 = [](R a, R bb, R c) { return gmax(a, gmax(bb, c)); };
            R mnG = min3(min3(d.y, e.y, f.y), b.y, hh.y);
            R mxG = max3(max3(d.y, e.y, f.y), b.y, hh.y);
            R rcpMG = R(APrxLoRcpF1(float(mxG)));
            R ampG = ASat(gmin(mnG, R(1.0) - mxG) * rcpMG);
            ampG = R(APrxLoSqrtF1(float(ampG)));
            R wG = ampG * peak;
            R rcpWeight = APrxMedRcpF1(R(1.0) + R(4.0) * wG);
            double* o = out + ((size_t)y * w + x) * 4;
            o[0] = double(ASat((b.x * wG + d.x * wG + f.x * wG + hh.x * wG + e.x) * rcpWeight));
            o[1] = double(ASat((b.y * wG + d.y * wG + f.y * wG + hh.y * wG + e.y) * rcpWeight));
            o[2] = double(ASat((b.z * wG + d.z * wG + f.z * wG + hh.z * wG + e.z) * rcpWeight));
            o[3] = 1.0;
        }
    });
}

// shaders/sharpen.comp:24-38; the border clamp is at size-1.
template <class R> void sharpen_t(const float* in, int w, int h, float factor, double* out, int nthreads) {
    parallel_rows(h, nthreads, [&](int y) {
        for (int x = 0; x < w; ++x) {
            auto L = [&](int dx, int dy) {
                int xx = clampi(x + dx, 0, w - 1), yy = clampi(y + dy, 0, h - 1);
                const float* q = in + ((size_t)yy * w + xx) * 4;
                return V3<R>{R(q[0]), R(q[1]), R(q[2])};
            };
            V3<R> Lf = L(-1, 0), Rt = L(1, 0), T = L(0, -1), B = L(0, 1), C = L(0, 0);
            V3<R> val = C + (R(4.0) * C - Lf - Rt - T - B) * R(factor);
            double* o = out + ((size_t)y * w + x) * 4;
            o[0] = double(gclamp(val.x, R(0), R(1)));
            o[1] = double(gclamp(val.y, R(0), R(1)));
            o[2] = double(gclamp(val.z, R(0), R(1)));
            o[3] = 1.0;
        }
    });
}

// ---------------------------------------------------------------- FXAA
// The FXAA pair of passes source/taa.hpp:1063-1104 dispatches, as one:
//   prepare  shaders/antialias_fxaa_prepare.comp:19-26 - rgb kept, alpha =
//            dot(rgb, (0.299, 0.587, 0.114)), stored in an RGBA16F image;
//   FXAA     shaders/antialias_fxaa.comp:34-64 - FXAA 3.11 quality, preset 12
//            (shaders/Fxaa3_11_mod.h:433-440, PC quality shader 726-1249) on
//            the pixels whose segmentation mask has (mask & 3) == 1, the
//            prepared texel elsewhere.
// Sampler: bilinear, clamp to edge, exact weights, except that a coordinate
// within 1/512 texel of a texel centre reads that texel (an 8-bit sub-texel
// filter rounds such offsets away; without it, rounding of the UV arithmetic
// at 4K would blend neighbours in at weights near 1e-4).
constexpr double kFxaaSnap = 1.0 / 512.0;

template <class R> struct FxaaImage {
    const float* rgba;  // source RGBA (alpha unused), w*h texels
    int w, h;
    // the prepared texel: rgb and the FP16-stored luma
    V4<R> texel(int x, int y) const {
        x = clampi(x, 0, w - 1);
        y = clampi(y, 0, h - 1);
        const float* q = rgba + ((size_t)y * w + x) * 4;
        R r = R(q[0]), g = R(q[1]), b = R(q[2]);
        R l = r * R(0.299) + g * R(0.587) + b * R(0.114);
        return {r, g, b, R(quantize_half(float(l)))};
    }
    // one coordinate of the filter footprint: the lower texel and its weight
    static void axis(R uvc, int size, int& i0, R& f) {
        R p = uvc * R(size) - R(0.5);
        R c = std::floor(p + R(0.5));
        if (std::fabs(p - c) < R(kFxaaSnap)) p = c;
        R p0 = std::floor(p);
        f = p - p0;
        i0 = trunc_index(p0);
        if (!(f == f)) f = R(0);
    }
    V4<R> sample(V2<R> uv) const {
        int x0, y0;
        R fx, fy;
        axis(uv.x, w, x0, fx);
        axis(uv.y, h, y0, fy);
        int x1 = x0 + 1 < x0 ? x0 : x0 + 1, y1 = y0 + 1 < y0 ? y0 : y0 + 1;
        V4<R> a = texel(x0, y0), b = texel(x1, y0), c = texel(x0, y1), d = texel(x1, y1);
        R gx = R(1) - fx, gy = R(1) - fy;
        V4<R> top{a.x * gx + b.x * fx, a.y * gx + b.y * fx, a.z * gx + b.z * fx, a.w * gx + b.w * fx};
        V4<R> bot{c.x * gx + d.x * fx, c.y * gx + d.y * fx, c.z * gx + d.z * fx, c.w * gx + d.w * fx};
        return {top.x * gy + bot.x * fy, top.y * gy + bot.y * fy, top.z * gy + bot.z * fy, top.w * gy + bot.w * fy};
    }
    R luma(V2<R> uv) const { return sample(uv).w; }
};

// FxaaPixelShader, quality PC path without gather (Fxaa3_11_mod.h:841-1249;
// the gather variant reads the same texels at a pixel centre).
template <class R> V4<R> fxaa_pixel(const FxaaImage<R>& t, int x, int y, V2<R> rcp, R subpix, R thr, R thr_min) {
    // preset 12: five search steps (Fxaa3_11_mod.h:433-440)
    static const R kStep[5] = {R(1.0), R(1.5), R(2.0), R(4.0), R(12.0)};
    V2<R> posM{(R(x) + R(0.5)) * rcp.x, (R(y) + R(0.5)) * rcp.y};  // antialias_fxaa.comp:43
    // the taps at the pixel centre and at whole-texel offsets from it read texels
    V4<R> rgbyM = t.texel(x, y);
    const R lumaM = rgbyM.w;
    auto off = [&](int dx, int dy) { return t.texel(x + dx, y + dy).w; };
    R lumaS = off(0, 1), lumaE = off(1, 0), lumaN = off(0, -1), lumaW = off(-1, 0);
    // local contrast and the early exit (Fxaa3_11_mod.h:890-910)
    R maxSM = gmax(lumaS, lumaM), minSM = gmin(lumaS, lumaM);
    R maxESM = gmax(lumaE, maxSM), minESM = gmin(lumaE, minSM);
    R maxWN = gmax(lumaN, lumaW), minWN = gmin(lumaN, lumaW);
    R rangeMax = gmax(maxWN, maxESM), rangeMin = gmin(minWN, minESM);
    R rangeMaxScaled = rangeMax * thr;
    R range = rangeMax - rangeMin;
    R rangeMaxClamped = gmax(thr_min, rangeMaxScaled);
    if (range < rangeMaxClamped) return rgbyM;
    R lumaNW = off(-1, -1), lumaSE = off(1, 1), lumaNE = off(1, -1), lumaSW = off(-1, 1);
    // edge orientation (Fxaa3_11_mod.h:923-960)
    R lumaNS = lumaN + lumaS, lumaWE = lumaW + lumaE;
    R subpixRcpRange = R(1.0) / range;
    R subpixNSWE = lumaNS + lumaWE;
    R edgeHorz1 = (R(-2.0) * lumaM) + lumaNS;
    R edgeVert1 = (R(-2.0) * lumaM) + lumaWE;
    R lumaNESE = lumaNE + lumaSE, lumaNWNE = lumaNW + lumaNE;
    R edgeHorz2 = (R(-2.0) * lumaE) + lumaNESE;
    R edgeVert2 = (R(-2.0) * lumaN) + lumaNWNE;
    R lumaNWSW = lumaNW + lumaSW, lumaSWSE = lumaSW + lumaSE;
    R edgeHorz4 = (std::fabs(edgeHorz1) * R(2.0)) + std::fabs(edgeHorz2);
    R edgeVert4 = (std::fabs(edgeVert1) * R(2.0)) + std::fabs(edgeVert2);
    R edgeHorz3 = (R(-2.0) * lumaW) + lumaNWSW;
    R edgeVert3 = (R(-2.0) * lumaS) + lumaSWSE;
    R edgeHorz = std::fabs(edgeHorz3) + edgeHorz4;
    R edgeVert = std::fabs(edgeVert3) + edgeVert4;
    R subpixNWSWNESE = lumaNWSW + lumaNESE;
    R lengthSign = rcp.x;
    const bool horzSpan = edgeHorz >= edgeVert;
    R subpixA = subpixNSWE * R(2.0) + subpixNWSWNESE;
    if (!horzSpan) {
        lumaN = lumaW;
        lumaS = lumaE;
    } else {
        lengthSign = rcp.y;
    }
    R subpixB = (subpixA * R(1.0 / 12.0)) - lumaM;
    // the steeper side and the half-texel step onto the edge (963-990)
    R gradientN = lumaN - lumaM, gradientS = lumaS - lumaM;
    R lumaNN = lumaN + lumaM, lumaSS = lumaS + lumaM;
    const bool pairN = std::fabs(gradientN) >= std::fabs(gradientS);
    R gradient = gmax(std::fabs(gradientN), std::fabs(gradientS));
    if (pairN) lengthSign = -lengthSign;
    R subpixC = gclamp(std::fabs(subpixB) * subpixRcpRange, R(0.0), R(1.0));
    V2<R> posB = posM;
    V2<R> offNP{horzSpan ? rcp.x : R(0.0), horzSpan ? R(0.0) : rcp.y};
    if (!horzSpan) posB.x += lengthSign * R(0.5);
    else posB.y += lengthSign * R(0.5);
    V2<R> posN{posB.x - offNP.x * kStep[0], posB.y - offNP.y * kStep[0]};
    V2<R> posP{posB.x + offNP.x * kStep[0], posB.y + offNP.y * kStep[0]};
    R subpixD = (R(-2.0) * subpixC) + R(3.0);
    R lumaEndN = t.luma(posN);
    R subpixE = subpixC * subpixC;
    R lumaEndP = t.luma(posP);
    if (!pairN) lumaNN = lumaSS;
    R gradientScaled = gradient * R(1.0) / R(4.0);
    R lumaMM = lumaM - lumaNN * R(0.5);
    R subpixF = subpixD * subpixE;
    const bool lumaMLTZero = lumaMM < R(0.0);
    // walk both ends along the edge until the luma leaves the pair's average (993-1190)
    lumaEndN -= lumaNN * R(0.5);
    lumaEndP -= lumaNN * R(0.5);
    bool doneN = std::fabs(lumaEndN) >= gradientScaled;
    bool doneP = std::fabs(lumaEndP) >= gradientScaled;
    if (!doneN) posN = {posN.x - offNP.x * kStep[1], posN.y - offNP.y * kStep[1]};
    bool doneNP = (!doneN) || (!doneP);
    if (!doneP) posP = {posP.x + offNP.x * kStep[1], posP.y + offNP.y * kStep[1]};
    for (int i = 2; i < 5 && doneNP; ++i) {
        if (!doneN) lumaEndN = t.luma(posN);
        if (!doneP) lumaEndP = t.luma(posP);
        if (!doneN) lumaEndN = lumaEndN - lumaNN * R(0.5);
        if (!doneP) lumaEndP = lumaEndP - lumaNN * R(0.5);
        doneN = std::fabs(lumaEndN) >= gradientScaled;
        doneP = std::fabs(lumaEndP) >= gradientScaled;
        if (!doneN) posN = {posN.x - offNP.x * kStep[i], posN.y - offNP.y * kStep[i]};
        doneNP = (!doneN) || (!doneP);
        if (!doneP) posP = {posP.x + offNP.x * kStep[i], posP.y + offNP.y * kStep[i]};
    }
    // the offset across the edge: span position or sub-pixel blend, the larger (1192-1248)
    R dstN = horzSpan ? posM.x - posN.x : posM.y - posN.y;
    R dstP = horzSpan ? posP.x - posM.x : posP.y - posM.y;
    const bool goodSpanN = (lumaEndN < R(0.0)) != lumaMLTZero;
    R spanLength = dstP + dstN;
    const bool goodSpanP = (lumaEndP < R(0.0)) != lumaMLTZero;
    R spanLengthRcp = R(1.0) / spanLength;
    const bool directionN = dstN < dstP;
    R dst = gmin(dstN, dstP);
    const bool goodSpan = directionN ? goodSpanN : goodSpanP;
    R subpixG = subpixF * subpixF;
    R pixelOffset = (dst * (-spanLengthRcp)) + R(0.5);
    R subpixH = subpixG * subpix;
    R pixelOffsetGood = goodSpan ? pixelOffset : R(0.0);
    R pixelOffsetSubpix = gmax(pixelOffsetGood, subpixH);
    if (!horzSpan) posM.x += pixelOffsetSubpix * lengthSign;
    else posM.y += pixelOffsetSubpix * lengthSign;
    V4<R> c = t.sample(posM);
    return {c.x, c.y, c.z, lumaM};
}

template <class R> void fxaa_t(const float* in, const uint32_t* segmask, int w, int h, const float rcp[2],
                               float subpix, float thr, float thr_min, double* out, int nthreads) {
    const FxaaImage<R> t{in, w, h};
    parallel_rows(h, nthreads, [&](int y) {
        for (int x = 0; x < w; ++x) {
            bool marked = !segmask || (segmask[(size_t)y * w + x] & 3u) == 1u;  // antialias_fxaa.comp:39-40
            V4<R> c = marked ? fxaa_pixel<R>(t, x, y, V2<R>{R(rcp[0]), R(rcp[1])}, R(subpix), R(thr), R(thr_min))
                             : t.texel(x, y);
            double* o = out + ((size_t)y * w + x) * 4;
            o[0] = double(c.x);
            o[1] = double(c.y);
            o[2] = double(c.z);
            o[3] = double(c.w);
        }
    });
}

}  // namespace

int resolve(int precision, const taa_uniforms_t& u, const ResolveInputs& in, const ResolveOutputs& out,
            int nthreads) {
    if (!in.color.p || !in.depth.p || !in.velocity.p || in.color.w <= 0 || in.color.h <= 0 || in.out_w <= 0 ||
        in.out_h <= 0)
        return -1;
    if (precision == 64)
        resolve_t<double>(u, in, out, nthreads);
    else
        resolve_t<float>(u, in, out, nthreads);
    return 0;
}

int cas(int precision, const float* in, int w, int h, uint32_t peak_bits, double* out, int nthreads) {
    if (!in || !out || w <= 0 || h <= 0) return -1;
    if (precision == 64)
        cas_t<double>(in, w, h, peak_bits, out, nthreads);
    else
        cas_t<float>(in, w, h, peak_bits, out, nthreads);
    return 0;
}

int sharpen(int precision, const float* in, int w, int h, float factor, double* out, int nthreads) {
    if (!in || !out || w <= 0 || h <= 0) return -1;
    if (precision == 64)
        sharpen_t<double>(in, w, h, factor, out, nthreads);
    else
        sharpen_t<float>(in, w, h, factor, out, nthreads);
    return 0;
}

int fxaa(int precision, const float* in, const uint32_t* segmask, int w, int h, const float rcp_frame[2],
         float subpix, float edge_threshold, float edge_threshold_min, double* out, int nthreads) {
    if (!in || !out || w <= 0 || h <= 0) return -1;
    if (precision == 64)
        fxaa_t<double>(in, segmask, w, h, rcp_frame, subpix, edge_threshold, edge_threshold_min, out, nthreads);
    else
        fxaa_t<float>(in, segmask, w, h, rcp_frame, subpix, edge_threshold, edge_threshold_min, out, nthreads);
    return 0;
}

// shaders/post_process.comp:32-91, one output texel (x, y) inside the image.
// texelFetch clamps to the image (the shader's zoom fetch stays inside for
// source boxes inside the image; outside, Vulkan leaves it undefined).
template <class R>
void post_pixel(const float* in, const float* dbg, int w, int h, const PostParams& pp, int x, int y, double* o) {
    auto put = [&](R r, R g, R b, R a) {
        o[0] = double(r);
        o[1] = double(g);
        o[2] = double(b);
        o[3] = double(a);
    };
    // the split-screen line (43-46)
    if (x == pp.split_x) return put(R(0), R(0), R(0), R(0));
    const int* zs = pp.zoom_src;
    const int* zd = pp.zoom_dst;
    // the border one texel outside the zoomed source box (49-54)
    if (pp.zoom && pp.show_zoom_box) {
        const bool col = (x == zs[0] - 1 || x == zs[0] + zs[2]) && y >= zs[1] - 1 && y <= zs[1] + zs[3];
        const bool row = (y == zs[1] - 1 || y == zs[1] + zs[3]) && x >= zs[0] - 1 && x <= zs[0] + zs[2];
        if (col || row) return put(R(1), R(0), R(0), R(0));
    }
    // the magnified inset: its border, else the texel it maps to in the source box (57-70)
    int fx = x, fy = y;
    if (pp.zoom && x >= zd[0] && y >= zd[1] && x < zd[0] + zd[2] && y < zd[1] + zd[3]) {
        const bool col = (x == zd[0] || x == zd[0] + zd[2] - 1) && y >= zd[1] && y <= zd[1] + zd[3] - 1;
        const bool row = (y == zd[1] || y == zd[1] + zd[3] - 1) && x >= zd[0] && x <= zd[0] + zd[2] - 1;
        if (col || row) return put(R(1), R(1), R(1), R(0));
        const R ux = (R(x - zd[0]) + R(0.5)) / R(zd[2]);
        const R uy = (R(y - zd[1]) + R(0.5)) / R(zd[3]);
        fx = int(R(zs[0]) + ux * R(zs[2]));  // int() truncates toward zero, as GLSL's ivec2(vec2)
        fy = int(R(zs[1]) + uy * R(zs[3]));
    }
    fx = std::min(std::max(fx, 0), w - 1);
    fy = std::min(std::max(fy, 0), h - 1);
    const size_t i = ((size_t)fy * w + fx) * 4;
    // the debug image or the input, by the side of the split (73-89)
    const bool left = pp.split_x < 0 || x < pp.split_x;
    const bool show = left ? pp.show_l != 0 : pp.show_r != 0;
    const float* mask = left ? pp.mask_l : pp.mask_r;
    if (show) {
        R r = R(dbg[i]), g = R(dbg[i + 1]), b = R(dbg[i + 2]);
        const R a = R(dbg[i + 3]);
        if (R(mask[3]) > R(0)) {  // the alpha channel made visible in red and blue
            r = r + a;
            b = b + a;
        }
        return put(r, g, b, R(1));
    }
    put(R(in[i]), R(in[i + 1]), R(in[i + 2]), R(in[i + 3]));
}

int post_process(int precision, const float* in, const float* debug, int w, int h, const PostParams& pp, double* out,
                 int nthreads) {
    if (!in || !out || w <= 0 || h <= 0) return -1;
    if (!debug && (pp.show_l || pp.show_r)) return -1;
    parallel_rows(h, nthreads, [&](int y) {
        for (int x = 0; x < w; ++x) {
            double* o = out + ((size_t)y * w + x) * 4;
            if (precision == 64) post_pixel<double>(in, debug, w, h, pp, x, y, o);
            else post_pixel<float>(in, debug, w, h, pp, x, y, o);
        }
    });
    return 0;
}

// ffx_cas.h:375-394 with ffx_a.h's CPU helpers: ARcpF1(a) = 1/a,
// ALerpF1(a,b,c) = b*c + (-a*c + a), ASatF1 = clamp to [0,1].
void cas_setup(float sharpness, float in_w, float in_h, float out_w, float out_h, uint32_t const0[4],
               uint32_t const1[4]) {
    auto rcp = [](float a) { return 1.0f / a; };
    const0[0] = fbits(in_w * rcp(out_w));
    const0[1] = fbits(in_h * rcp(out_h));
    const0[2] = fbits(0.5f * in_w * rcp(out_w) - 0.5f);
    const0[3] = fbits(0.5f * in_h * rcp(out_h) - 0.5f);
    float s = std::min(1.0f, std::max(0.0f, sharpness));
    float lerp = 5.0f * s + (-8.0f * s + 8.0f);
    float sharp = -rcp(lerp);
    const1[0] = fbits(sharp);
    // AU1_AH2_AF2({sharp, 0}) on the CPU (ffx_a.h:470-545): a truncating
    // float->half conversion indexed by sign+exponent, restated arithmetically:
    // exponent fields below 103 give +-0, 103..112 a subnormal with the implicit
    // bit, 113..142 a normal half, 143 and above (and inf/nan) +-65504.
    auto to_half_trunc = [](float f) -> uint32_t {
        uint32_t u = fbits(f);
        uint32_t sign = (u >> 16) & 0x8000u;
        uint32_t e = (u >> 23) & 0xffu;
        uint32_t m = u & 0x7fffffu;
        if (e < 103u) return sign;
        if (e <= 112u) return sign + (1u << (e - 103u)) + (m >> (126u - e));
        if (e <= 142u) return sign + ((e - 112u) << 10) + (m >> 13);
        return sign + 0x7bffu;
    };
    const1[1] = to_half_trunc(sharp) + (to_half_trunc(0.0f) << 16);
    const1[2] = fbits(8.0f * in_w * rcp(out_w));
    const1[3] = 0;
}

// helper_functions.hpp:9-17
float halton(int i, int b) {
    float f = 1.0f, r = 0.0f;
    while (i > 0) {
        f = f / float(b);
        r = r + f * float(i % b);
        i = i / b;
    }
    return r;
}

// taa.hpp:150-233
void jitter_offset(int dist, uint64_t frame_id, int in_w, int in_h, int fixed_index, int slow_motion,
                   float rotate_degrees, float extra_scale, float out[2], int* num_samples) {
    const float px = 2.0f / float(in_w), py = 2.0f / float(in_h);
    float tab[16][2];
    int n = 0;
    switch (dist) {
        case 0: {
            const float t[4][2] = {{-0.25f, -0.25f}, {0.25f, -0.25f}, {0.25f, 0.25f}, {-0.25f, 0.25f}};
            for (n = 0; n < 4; ++n) { tab[n][0] = px * t[n][0]; tab[n][1] = py * t[n][1]; }
            break;
        }
        case 1: {
            const float t[4][2] = {{-0.25f, -0.25f}, {0.25f, 0.25f}, {0.25f, -0.25f}, {-0.25f, 0.25f}};
            for (n = 0; n < 4; ++n) { tab[n][0] = px * t[n][0]; tab[n][1] = py * t[n][1]; }
            break;
        }
        case 2:
        case 3: {
            int len = dist == 2 ? 8 : 16;
            for (n = 0; n < len; ++n) {
                tab[n][0] = px * (halton(n + 1, 2) - 0.5f);
                tab[n][1] = py * (halton(n + 1, 3) - 0.5f);
            }
            break;
        }
        default: {
            const float e = 1.f / 8.f;
            const float v[4] = {-3.f * e, -1.f * e, 1.f * e, 3.f * e};
            for (int j = 0; j < 4; ++j)
                for (int i = 0; i < 4; ++i) { tab[n][0] = px * v[i]; tab[n][1] = py * v[j]; ++n; }
            break;
        }
    }
    if (slow_motion > 1) frame_id /= (uint64_t)slow_motion;
    if (fixed_index >= 0) frame_id = (uint64_t)fixed_index;
    float x = tab[frame_id % (uint64_t)n][0], y = tab[frame_id % (uint64_t)n][1];
    if (rotate_degrees != 0.f) {
        float rad = rotate_degrees * 0.01745329251994329576923690768489f;
        float s = std::sin(rad), c = std::cos(rad);
        float nx = x * c - y * s, ny = x * s + y * c;
        x = nx;
        y = ny;
    }
    out[0] = x * extra_scale;
    out[1] = y * extra_scale;
    if (num_samples) *num_samples = n;
}

float quantize_half(float x) {
    uint32_t u = fbits(x);
    uint32_t sign = u & 0x80000000u;
    uint32_t a = u & 0x7fffffffu;
    if (a >= 0x7f800000u) return x;  // inf / nan
    // binary16 max finite 65504; values at or above 65520 round to infinity
    if (a >= 0x477ff000u) return bitsf(sign | 0x7f800000u);
    float af = bitsf(a);
    if (af < 6.103515625e-05f) {
        // subnormal half: multiples of 2^-24, round half to even
        float q = std::nearbyint(af * 16777216.0f);
        return bitsf(sign | fbits(q / 16777216.0f));
    }
    // normal: keep 10 mantissa bits, round half to even
    uint32_t lsb = (a >> 13) & 1u;
    uint32_t r = a + 0xfffu + lsb;
    r &= ~0x1fffu;
    return bitsf(sign | r);
}

}  // namespace taa_oracle
