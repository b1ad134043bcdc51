// resolve_plain.cu - the plain FP32 resolve: one thread per output pixel,
// direct global loads, every field of the parameter block honoured.
//
// Follows shaders/taa.comp:708-960 (and its helpers 131-702) with the sampler
// semantics of the project's oracle (texelFetch clamps to the edge; texture()
// at a by-construction texel centre is that texel; elsewhere exact-weight
// bilinear; the 9-tap Catmull-Rom is its 16-tap equivalent).  This
// translation unit is compiled with -fmad=false and uses explicit FMAs only
// where the oracle does (the second-moment chain and the Catmull-Rom
// accumulation), so on the same inputs it rounds like the FP32 oracle
// operation for operation.  It is the reference
// form the tiled and FP16 forms are measured against.
#include "common.cuh"
#include "kernels.h"
#include "segmentation.cuh"

namespace taa_dev {
namespace {

struct V2 { float x, y; };
struct V3 { float x, y, z; };

__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ V3 operator+(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
__device__ __forceinline__ V3 vmin(V3 a, V3 b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
__device__ __forceinline__ V3 vmax(V3 a, V3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
__device__ __forceinline__ V3 vfma(V3 a, V3 b, V3 c) {
    return {__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y), __fmaf_rn(a.z, b.z, c.z)};
}
__device__ __forceinline__ V3 rgb3(float4 v) { return {v.x, v.y, v.z}; }
__device__ __forceinline__ float gmix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ V3 vmix(V3 x, V3 y, float a) {
    float t = 1.0f - a;
    return {x.x * t + y.x * a, x.y * t + y.y * a, x.z * t + y.z * a};
}

// Exact-weight bilinear, clamp to edge (texel centres at k + 0.5).
template <class F>
__device__ __forceinline__ float4 bilinear(int w, int h, V2 uv, F&& tex) {
    return bilinear_uv(w, h, uv.x, uv.y, tex);
}

template <int HF, int MC>
struct PlainResolver {
    const taa_uniforms_t& U;
    const FrameArgs& a;
    const taa_parameters_t* P;
    int loW, loH, hiW, hiH;
    bool same;

    __device__ PlainResolver(const taa_uniforms_t& u, const FrameArgs& args)
        : U(u), a(args), P(nullptr), loW(args.color.w), loH(args.color.h), hiW(args.out_w), hiH(args.out_h),
          same(args.color.w == args.out_w && args.color.h == args.out_h) {}

    __device__ float4 col(int x, int y) const { return fetch_rgba16f(a.color, x, y); }
    __device__ float4 vel(int x, int y) const { return fetch_velocity<MC>(a.velocity, x, y); }
    __device__ float4 dep(int x, int y) const {
        return make_float4(fetch_r32f(a.depth, x, y), 0.f, 0.f, 0.f);
    }
    __device__ float4 his(int x, int y) const { return fetch_history<HF>(a.history, x, y); }

    __device__ V3 rgb_to_ycocg(V3 c) const {
        return {.25f * c.x + .5f * c.y + .25f * c.z, .5f * c.x - .5f * c.z, -.25f * c.x + .5f * c.y - .25f * c.z};
    }
    __device__ V3 ycocg_to_rgb(V3 c) const {
        float tmp = c.x - c.z;
        return {tmp + c.y, c.x + c.z, tmp - c.y};
    }
    __device__ V3 maybe_rgb_to_ycocg(V3 c) const { return P->mUseYCoCg ? rgb_to_ycocg(c) : c; }
    __device__ V3 maybe_ycocg_to_rgb(V3 c) const { return P->mUseYCoCg ? ycocg_to_rgb(c) : c; }
    __device__ float luminance(V3 c) const { return P->mUseYCoCg ? c.x : rgb_to_ycocg(c).x; }
    __device__ V3 tonemap_rgb(V3 hdr) const {
        if (P->mToneMapLumaKaris) return hdr / (1.0f + gmax(gmax(hdr.x, hdr.y), hdr.z));
        return hdr;
    }
    __device__ V3 un_tonemap_rgb(V3 ldr) const {
        if (P->mToneMapLumaKaris) return ldr / (1.0f - gmax(gmax(ldr.x, ldr.y), ldr.z));
        return ldr;
    }
    __device__ V2 jitter_uv() const {
        return {U.mJitterNdc[0] * 0.5f * P->mUnjitterFactor, U.mJitterNdc[1] * 0.5f * P->mUnjitterFactor};
    }
    __device__ V3 color_tap(int ix, int iy, V2 off) const {
        if (off.x == 0.f && off.y == 0.f) return rgb3(col(ix, iy));
        float invx = 1.0f / (float)loW, invy = 1.0f / (float)loH;
        V2 uv{off.x + ((float)ix + 0.5f) * invx, off.y + ((float)iy + 0.5f) * invy};
        return rgb3(bilinear(loW, loH, uv, [&](int x, int y) { return col(x, y); }));
    }
    __device__ V3 load_color(int ix, int iy, V2 off) const {
        return maybe_rgb_to_ycocg(tonemap_rgb(color_tap(ix, iy, off)));
    }

    // taa.comp:222-257
    __device__ V3 upsampled_color(int tx, int ty, float& beta) const {
        int fx, fy;
        if (upsampled_source(U, *P, tx, ty, hiW, hiH, loW, loH, fx, fy)) {
            beta = 1.0f;
            return maybe_rgb_to_ycocg(tonemap_rgb(rgb3(col(fx, fy))));
        }
        beta = 0.0f;
        return {0.f, 0.f, 0.f};
    }

    // taa.comp:259-319
    __device__ void color_and_aabb(int ix, int iy, V3& c0, V3& mn, V3& mx, V3& ct) const {
        const float N = 9.0f;
        V2 off = P->mUnjitterNeighbourhood ? jitter_uv() : V2{0.f, 0.f};
        c0 = load_color(ix, iy, off);
        V3 c1 = load_color(ix - 1, iy - 1, off), c2 = load_color(ix, iy - 1, off), c3 = load_color(ix + 1, iy - 1, off);
        V3 c4 = load_color(ix - 1, iy, off), c5 = load_color(ix + 1, iy, off);
        V3 c6 = load_color(ix - 1, iy + 1, off), c7 = load_color(ix, iy + 1, off), c8 = load_color(ix + 1, iy + 1, off);
        if (P->mVarianceClipping) {
            V3 m1 = c0 + c1 + c2 + c3 + c4 + c5 + c6 + c7 + c8;
            V3 m2 = c0 * c0;
            m2 = vfma(c1, c1, m2); m2 = vfma(c2, c2, m2); m2 = vfma(c3, c3, m2);
            m2 = vfma(c4, c4, m2); m2 = vfma(c5, c5, m2); m2 = vfma(c6, c6, m2);
            m2 = vfma(c7, c7, m2); m2 = vfma(c8, c8, m2);
            V3 mean = m1 / N;
            V3 var = vfma(V3{-mean.x, -mean.y, -mean.z}, mean, m2 / N);
            V3 sg{sqrtf(gmax(0.f, var.x)), sqrtf(gmax(0.f, var.y)), sqrtf(gmax(0.f, var.z))};
            float g = P->mVarClipGamma;
            mn = mean - g * sg;
            mx = mean + g * sg;
            ct = mean;
        } else if (P->mShapedNeighbourhood) {
            V3 mn3 = vmin(vmin(vmin(vmin(vmin(vmin(vmin(vmin(c0, c1), c2), c3), c4), c5), c6), c7), c8);
            V3 mx3 = vmax(vmax(vmax(vmax(vmax(vmax(vmax(vmax(c0, c1), c2), c3), c4), c5), c6), c7), c8);
            V3 mn5 = vmin(vmin(vmin(vmin(c0, c2), c4), c5), c7);
            V3 mx5 = vmax(vmax(vmax(vmax(c0, c2), c4), c5), c7);
            mn = (mn3 + mn5) * 0.5f;
            mx = (mx3 + mx5) * 0.5f;
            ct = c0;
        } else {
            mn = vmin(vmin(vmin(vmin(vmin(vmin(vmin(vmin(c0, c1), c2), c3), c4), c5), c6), c7), c8);
            mx = vmax(vmax(vmax(vmax(vmax(vmax(vmax(vmax(c0, c1), c2), c3), c4), c5), c6), c7), c8);
            ct = c0;
        }
        if (P->mUseYCoCg && P->mShrinkChromaAxis) {
            V3 half_size = V3{0.5f * 1.0f, 0.5f * 0.5f, 0.5f * 0.5f} * (mx - mn);
            V3 center = (mn + mx) * 0.5f;
            mn = center - half_size;
            mx = center + half_size;
            bool out = ct.x < mn.x || ct.y < mn.y || ct.z < mn.z || ct.x > mx.x || ct.y > mx.y || ct.z > mx.z;
            if (out) ct = center;
        }
    }

    // taa.comp:323-345
    __device__ V3 clip_aabb(V3 lo, V3 hi, V3 q) const {
        const float eps = 1e-7f;
        V3 p = 0.5f * (hi + lo);
        V3 e = 0.5f * (hi - lo) + eps;
        V3 v = q - p;
        V3 u = v / e;
        float ma = gmax(fabsf(u.x), gmax(fabsf(u.y), fabsf(u.z)));
        if (ma > 1.0f) return p + v / ma;
        return q;
    }
    // taa.comp:348-369
    __device__ V3 clip_aabb_slow(V3 lo, V3 hi, V3 p, V3 q) const {
        V3 r = q - p, rmax = hi - p, rmin = lo - p;
        const float eps = 1e-7f;
        if (r.x > rmax.x + eps) r = r * (rmax.x / r.x);
        if (r.y > rmax.y + eps) r = r * (rmax.y / r.y);
        if (r.z > rmax.z + eps) r = r * (rmax.z / r.z);
        if (r.x < rmin.x - eps) r = r * (rmin.x / r.x);
        if (r.y < rmin.y - eps) r = r * (rmin.y / r.y);
        if (r.z < rmin.z - eps) r = r * (rmin.z / r.z);
        return p + r;
    }

    template <class F>
    __device__ float4 sample_at(int tw, int th, int ix, int iy, V2 uv, int dx, int dy, F&& tex) const {
        if (same) return tex(ix + dx, iy + dy);
        V2 q{uv.x + (1.0f / (float)tw) * (float)dx, uv.y + (1.0f / (float)th) * (float)dy};
        return bilinear(tw, th, q, tex);
    }
    __device__ float4 vel_at(int ix, int iy, V2 uv, int dx, int dy) const {
        return sample_at(a.velocity.w, a.velocity.h, ix, iy, uv, dx, dy, [&](int x, int y) { return vel(x, y); });
    }
    __device__ float dep_at(int ix, int iy, V2 uv, int dx, int dy) const {
        return sample_at(a.depth.w, a.depth.h, ix, iy, uv, dx, dy, [&](int x, int y) { return dep(x, y); }).x;
    }

    // taa.comp:391-438
    __device__ void history_position(int ix, int iy, V2 cu, float cd, V2& hu, float& hd, float& speed) const {
        float4 vs = vel_at(ix, iy, cu, 0, 0);
        bool can = !(P->mUseVelocityVectors == 0 || (P->mUseVelocityVectors == 1 && vs.w < 0.5f));
        if (can) {
            if (P->mVelocitySampleMode == 1) {
                const int ox[8] = {1, -1, -1, 0, -1, 0, 1, 1};
                const int oy[8] = {-1, 0, -1, -1, 1, 1, 0, 1};
                V2 maxv{vs.x, vs.y}, sam{0.f, 0.f};
                for (int k = 0; k < 8; ++k) {
                    float4 s = vel_at(ix, iy, cu, ox[k], oy[k]);
                    sam = {s.x, s.y};
                    if (sam.x * sam.x + sam.y * sam.y > maxv.x * maxv.x + maxv.y * maxv.y) maxv = sam;
                }
                vs.x = sam.x;  // the reference keeps the last tap (taa.comp:412)
                vs.y = sam.y;
            } else if (P->mVelocitySampleMode == 2) {
                const int ox[9] = {-1, 0, 1, -1, 0, 1, -1, 0, 1};
                const int oy[9] = {-1, -1, -1, 0, 0, 0, 1, 1, 1};
                int best = 0;
                float dc = dep_at(ix, iy, cu, ox[0], oy[0]);
                for (int k = 1; k < 9; ++k) {
                    float d = dep_at(ix, iy, cu, ox[k], oy[k]);
                    if (d < dc) { best = k; dc = d; }
                }
                if (same) {
                    vs = vel(ix + ox[best], iy + oy[best]);
                } else {
                    V2 q{cu.x + (1.0f / (float)a.depth.w) * (float)ox[best],
                         cu.y + (1.0f / (float)a.depth.h) * (float)oy[best]};
                    vs = bilinear(a.velocity.w, a.velocity.h, q, [&](int x, int y) { return vel(x, y); });
                }
            }
            hu = {cu.x - vs.x, cu.y - vs.y};
            hd = cd - vs.z;
        } else {
            float cs[4] = {cu.x * 2.0f - 1.0f, cu.y * 2.0f - 1.0f, cd, 1.0f};
            float ws[4], hs[4];
            const float* A = U.mInverseViewProjMatrix;
            const float* B = U.mHistoryViewProjMatrix;
#pragma unroll
            for (int i = 0; i < 4; ++i) ws[i] = A[i] * cs[0] + A[4 + i] * cs[1] + A[8 + i] * cs[2] + A[12 + i] * cs[3];
#pragma unroll
            for (int i = 0; i < 4; ++i) hs[i] = B[i] * ws[0] + B[4 + i] * ws[1] + B[8 + i] * ws[2] + B[12 + i] * ws[3];
            hu = {(hs[0] / hs[3]) * 0.5f + 0.5f, (hs[1] / hs[3]) * 0.5f + 0.5f};
            hd = hs[2] / hs[3];
        }
        V2 d{cu.x - hu.x, cu.y - hu.y};
        speed = sqrtf(d.x * d.x + d.y * d.y);
    }

    // taa.comp:441-514 as the 16-tap equivalent
    __device__ float4 history_catmullrom(V2 uv) const {
        float sx = (float)a.history.w, sy = (float)a.history.h;
        float itx = uv.x * sx, ity = uv.y * sy;
        float fx = itx - (floorf(itx - 0.5f) + 0.5f), fy = ity - (floorf(ity - 0.5f) + 0.5f);
        float wx[4], wy[4];
        auto weights = [](float f, float* w) {
            float f2 = f * f, f3 = f2 * f;
            w[0] = -0.5f * f3 + f2 - 0.5f * f;
            w[1] = 1.5f * f3 - 2.5f * f2 + 1.0f;
            w[2] = -1.5f * f3 + 2.0f * f2 + 0.5f * f;
            w[3] = 0.5f * f3 - 0.5f * f2;
        };
        weights(fx, wx);
        weights(fy, wy);
        int kx = trunc_index(floorf(itx - 0.5f)), ky = trunc_index(floorf(ity - 0.5f));
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float4 row = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                float4 s = his(kx - 1 + i, ky - 1 + j);
                row.x = __fmaf_rn(wx[i], s.x, row.x);
                row.y = __fmaf_rn(wx[i], s.y, row.y);
                row.z = __fmaf_rn(wx[i], s.z, row.z);
                row.w = __fmaf_rn(wx[i], s.w, row.w);
            }
            acc.x = __fmaf_rn(wy[j], row.x, acc.x);
            acc.y = __fmaf_rn(wy[j], row.y, acc.y);
            acc.z = __fmaf_rn(wy[j], row.z, acc.z);
            acc.w = __fmaf_rn(wy[j], row.w, acc.w);
        }
        return acc;
    }
    // taa.comp:517-543, four exact bilinear taps
    __device__ float4 history_bspline(V2 uv) const {
        float sx = (float)a.history.w, sy = (float)a.history.h;
        float inv[2] = {1.0f / sx, 1.0f / sy};
        float it[2] = {uv.x * sx, uv.y * sy};
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
            float f0 = w1 / (w0 + w1), f1 = w3 / (w2 + w3);
            t0[k] = (tc - 1.0f + f0) * inv[k];
            t1[k] = (tc + 1.0f + f1) * inv[k];
        }
        auto H = [&](int x, int y) { return his(x, y); };
        int w = a.history.w, h = a.history.h;
        float4 A = bilinear(w, h, V2{t0[0], t0[1]}, H), B = bilinear(w, h, V2{t1[0], t0[1]}, H);
        float4 C = bilinear(w, h, V2{t0[0], t1[1]}, H), D = bilinear(w, h, V2{t1[0], t1[1]}, H);
        return make_float4((A.x * s0[0] + B.x * s1[0]) * s0[1] + (C.x * s0[0] + D.x * s1[0]) * s1[1],
                           (A.y * s0[0] + B.y * s1[0]) * s0[1] + (C.y * s0[0] + D.y * s1[0]) * s1[1],
                           (A.z * s0[0] + B.z * s1[0]) * s0[1] + (C.z * s0[0] + D.z * s1[0]) * s1[1],
                           (A.w * s0[0] + B.w * s1[0]) * s0[1] + (C.w * s0[0] + D.w * s1[0]) * s1[1]);
    }
    __device__ float4 sample_history(V2 uv) const {
        if (P->mInterpolationMode == 0)
            return bilinear(a.history.w, a.history.h, uv, [&](int x, int y) { return his(x, y); });
        if (P->mInterpolationMode == 1) return history_bspline(uv);
        return history_catmullrom(uv);
    }

    // taa.comp:551-556
    __device__ float4 noise(V2 uv) const { return taa_noise(U, *P, uv.x, uv.y); }

    // taa.comp:559-702 through segmentation.cuh, reading global memory
    struct SegAccess {
        const PlainResolver& r;
        __device__ uint32_t material(int x, int y) const { return fetch_r32u(r.a.material, x, y); }
        __device__ uint32_t prev_material(int x, int y) const { return fetch_r32u(r.a.prev_material, x, y); }
        __device__ uint32_t prev_segmask(int x, int y) const { return fetch_r32u(r.a.prev_segmask, x, y); }
        __device__ seg::N3 normal(int x, int y) const {
            const float4 u = fetch_rgba32f(r.a.uvnrm, x, y);
            return seg::normal_from(u.z, u.w);
        }
        __device__ float lin_depth(int x, int y) const {
            return seg::lin_depth(fetch_r32f(r.a.depth, x, y), r.U.mCamNearPlane, r.U.mCamFarPlane);
        }
        __device__ float luma(int x, int y) const {
            const float4 c = r.col(x, y);
            return seg::luma(c.x, c.y, c.z);
        }
    };
    __device__ uint32_t segmentation(int ix, int iy, V2 hu) const {
        return seg::classify(*P, ix, iy, hu.x, hu.y, loW, loH, SegAccess{*this});
    }

    // taa.comp:708-960
    __device__ void pixel(int x, int y) {
        V2 uv{((float)x + 0.5f) / (float)hiW, ((float)y + 0.5f) / (float)hiH};
        P = &U.param[(U.splitScreen && x > U.splitX) ? 1 : 0];
        bool gen_seg = P->mRayTraceAugment != 0;
        int lx = trunc_index(uv.x * (float)loW), ly = trunc_index(uv.y * (float)loH);

        if (P->mPassThrough || U.mBypassHistoryUpdate) {
            float4 h = his(x, y);
            float4 s = P->mPassThrough ? col(lx, ly) : h;
            if (a.result.p) store_rgba16f(a.result, x, y, make_float4(s.x, s.y, s.z, 1.f));
            store_history<HF>(a.history_out, x, y, make_float4(h.x, h.y, h.z, 1.f));
            if (a.debug.p) store_rgba16f(a.debug, x, y, make_float4(0.f, 0.f, 0.f, 0.f));
            return;
        }

        bool rejected = false;
        V3 cur, mn, mx, ct;
        float beta;
        color_and_aabb(lx, ly, cur, mn, mx, ct);
        if (U.mUpsampling) {
            cur = upsampled_color(x, y, beta);
        } else {
            V2 off = P->mUnjitterCurrentSample ? jitter_uv() : V2{0.f, 0.f};
            cur = load_color(lx, ly, off);
            beta = 1.0f;
        }
        float depth = fetch_r32f(a.depth, lx, ly);
        V2 hu;
        float ehd, speed;
        history_position(lx, ly, uv, depth, hu, ehd, speed);
        float4 hraw = sample_history(hu);
        V3 hc = maybe_rgb_to_ycocg(rgb3(hraw));
        float alpha = P->mAlpha;

        uint32_t seg = 0;
        if (gen_seg) {
            seg = segmentation(x, y, hu);
            if ((seg & 3u) != 0) { alpha = P->mRejectionAlpha; rejected = true; }
        }
        if (P->mRejectOutside) {
            if (hu.x < 0.f || hu.y < 0.f || hu.x >= 1.f || hu.y >= 1.f) { alpha = P->mRejectionAlpha; rejected = true; }
        }
        float dyn_mask = 0.f;
        if (P->mDynamicAntiGhosting) {
            const float eps = 1e-5f;
            auto mov = [&](int dx, int dy) {
                float4 v = vel_at(lx, ly, uv, dx, dy);
                return (fabsf(v.x) > eps || fabsf(v.y) > eps) && (fabsf(v.w) >= 0.5f);
            };
            bool mL = mov(-1, 0), mR = mov(1, 0), mT = mov(0, -1), mB = mov(0, 1), mC = mov(0, 0);
            if (!(mL || mR || mT || mB || mC) && hraw.w > 0.0f) rejected = true;
            dyn_mask = mC ? 1.0f : 0.0f;
        }
        if (P->mDepthCulling) {
            int tx = trunc_index(hu.x * (float)loW), ty = trunc_index(hu.y * (float)loH);
            float hd = a.history_depth.p ? fetch_r32f(a.history_depth, tx, ty) : 0.f;
            float eps = 0.1f * (1.0f - hd);
            if (fabsf(hd - ehd) > eps) rejected = true;
        }
        V3 orig = hc;
        switch (P->mColorClampingOrClipping) {
            case 1: hc = vmin(vmax(hc, mn), mx); break;
            case 2: hc = clip_aabb(mn, mx, hc); break;
            case 3: hc = clip_aabb_slow(mn, mx, ct, hc); break;
            default: break;
        }
        V3 rdiff = hc - orig;
        if (rejected) {
            alpha = P->mRejectionAlpha;
            beta = 1.0f;
        } else {
            if (P->mVelBasedAlpha)
                alpha = gmax(alpha, gmix(alpha, P->mVelBasedAlphaMax, gclamp(speed * P->mVelBasedAlphaFactor, 0.f, 1.f)));
            if (P->mLumaWeightingLottes) {
                float lc = luminance(cur), lh = luminance(hc);
                float diff = fabsf(lc - lh) / gmax(gmax(lc, lh), 0.2f);
                float w = 1.0f - diff;
                alpha = gmix(P->mMaxAlpha, P->mMinAlpha, w * w);
            }
            if (P->mReduceBlendNearClamp) {
                float lmn = luminance(mn), lmx = luminance(mx), lh = luminance(orig);
                float dist = 2.0f * fabsf(gmin(lh - lmn, lmx - lh)) / (lmx - lmn);
                if (lmx - lmn < 0.001f) dist = 1.0f;
                alpha = alpha * gclamp(4.0f * dist, 0.f, 1.f);
            }
        }
        if (U.mResetHistory) { alpha = 1.0f; beta = 1.0f; }
        V3 aa = maybe_ycocg_to_rgb(vmix(hc, cur, alpha * beta));
        if (P->mAddNoise) {
            float4 n = noise(uv);
            aa = aa + V3{n.x, n.y, n.z};
        }
        float4 to_hist = make_float4(aa.x, aa.y, aa.z, dyn_mask);
        V3 sc = un_tonemap_rgb(aa);
        float4 to_screen = make_float4(sc.x, sc.y, sc.z, 1.0f);

        if (a.debug.p) {
            DebugIn d;
            d.mn = make_float3(mn.x, mn.y, mn.z);
            d.mx = make_float3(mx.x, mx.y, mx.z);
            d.rdiff = make_float3(rdiff.x, rdiff.y, rdiff.z);
            d.rejected = rejected;
            d.alpha = alpha;
            d.speed = speed;
            d.vel = P->mDebugMode == 4 ? vel(x, y) : make_float4(0.f, 0.f, 0.f, 0.f);
            d.to_screen = to_screen;
            d.to_hist = to_hist;
            d.seg = seg;
            store_rgba16f(a.debug, x, y, debug_value(*P, d));
        }
        store_history<HF>(a.history_out, x, y, to_hist);
        if (a.result.p) store_rgba16f(a.result, x, y, to_screen);
        if (gen_seg && a.segmask.p) *texel_ptr_w<uint32_t>(a.segmask, x, y) = seg;
    }
};

template <int HF, int MC>
__global__ void __launch_bounds__(256) resolve_plain_kernel(const taa_uniforms_t U, const FrameArgs a) {
    int x = blockIdx.x * 16 + threadIdx.x;
    int y = blockIdx.y * 16 + threadIdx.y;
    if (x >= a.out_w || y >= a.out_h) return;
    PlainResolver<HF, MC> r(U, a);
    r.pixel(x, y);
}

}  // namespace

cudaError_t launch_resolve_plain(const taa_uniforms_t& U, const FrameArgs& a, int history_format, int motion_channels,
                                 cudaStream_t stream) {
    dim3 block(16, 16);
    dim3 grid((a.out_w + 15) / 16, (a.out_h + 15) / 16);
    if (history_format == 0) {
        if (motion_channels == 4) resolve_plain_kernel<0, 4><<<grid, block, 0, stream>>>(U, a);
        else resolve_plain_kernel<0, 2><<<grid, block, 0, stream>>>(U, a);
    } else {
        if (motion_channels == 4) resolve_plain_kernel<1, 4><<<grid, block, 0, stream>>>(U, a);
        else resolve_plain_kernel<1, 2><<<grid, block, 0, stream>>>(U, a);
    }
    return cudaGetLastError();
}

}  // namespace taa_dev
