// common.cuh - device-side helpers shared by the resolve kernels.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include "../../include/taa_params.h"

namespace taa_dev {

// A pitched device image.
struct Img {
    const char* p;
    size_t pitch;
    int w, h;
};
struct ImgW {
    char* p;
    size_t pitch;
};

// Everything one resolve launch needs besides the uniform block.
struct FrameArgs {
    Img color;          // RGBA16F, source size
    Img depth;          // D32F, source size
    Img history;        // RGBA32F or RGBA16F, target size (p == nullptr reads zeros)
    Img history_depth;  // D32F, source size
    Img velocity;       // RG16F or RGBA16F, source size
    Img material;       // R32UI
    Img prev_material;  // R32UI
    Img prev_segmask;   // R32UI
    Img uvnrm;          // RGBA32F
    ImgW result;        // RGBA16F, target size
    ImgW debug;         // RGBA16F
    ImgW history_out;   // RGBA32F or RGBA16F
    ImgW segmask;       // R32UI
    ImgW sharpened;     // RGBA16F
    int out_w, out_h;
    float inv_out_w, inv_out_h;  // correctly rounded 1/out size
    uint32_t cas_peak_bits;      // CasSetup const1.x
    float sharpen_factor;
    unsigned int* status;        // device status word (bounded waits that gave up set bits)
    uint64_t neg_zero2;          // the FP32 pair (-0.0, -0.0), opaque to the compiler (f32x2.cuh)
};

// A view of a batch, in device memory: its uniform block and images.
struct __align__(16) BatchView {
    taa_uniforms_t U;
    FrameArgs a;
};
// A batch job names a view and one tile of it: view (8 bits), tile row and
// tile column (12 bits each).
__host__ __device__ constexpr uint32_t make_job(int view, int tile_x, int tile_y) {
    return ((uint32_t)view << 24) | ((uint32_t)tile_y << 12) | (uint32_t)tile_x;
}
__host__ __device__ constexpr int job_view(uint32_t j) { return (int)(j >> 24); }
__host__ __device__ constexpr int job_tile_y(uint32_t j) { return (int)((j >> 12) & 0xfffu); }
__host__ __device__ constexpr int job_tile_x(uint32_t j) { return (int)(j & 0xfffu); }

// Bits of the device status word.
constexpr unsigned int kStatusWindowTimeout = 1u;  // a history-window copy did not complete in time

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// GLSL min/max on finite values.
__device__ __forceinline__ float gmax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float gmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

// ivec2(float) made total: truncation toward zero of t held in [-1e9, 1e9]
// (NaN gives -1e9); the caller clamps the index to the image.
__device__ __forceinline__ int trunc_index(float t) {
    return __float2int_rz(fminf(fmaxf(t, -1e9f), 1e9f));
}

template <class T> __device__ __forceinline__ const T* texel_ptr(const Img& im, int x, int y) {
    return reinterpret_cast<const T*>(im.p + (size_t)y * im.pitch) + x;
}

__device__ __forceinline__ float4 half4_to_float4(uint2 v) {
    __half2 a = *reinterpret_cast<__half2*>(&v.x);
    __half2 b = *reinterpret_cast<__half2*>(&v.y);
    float2 fa = __half22float2(a), fb = __half22float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}
__device__ __forceinline__ uint2 float4_to_half4(float4 v) {
    __half2 a = __floats2half2_rn(v.x, v.y);
    __half2 b = __floats2half2_rn(v.z, v.w);
    uint2 r;
    r.x = *reinterpret_cast<uint32_t*>(&a);
    r.y = *reinterpret_cast<uint32_t*>(&b);
    return r;
}

// RGBA16F texel (clamped to the image).
__device__ __forceinline__ float4 fetch_rgba16f(const Img& im, int x, int y) {
    x = clampi(x, 0, im.w - 1);
    y = clampi(y, 0, im.h - 1);
    return half4_to_float4(__ldg(texel_ptr<uint2>(im, x, y)));
}
__device__ __forceinline__ float fetch_r32f(const Img& im, int x, int y) {
    x = clampi(x, 0, im.w - 1);
    y = clampi(y, 0, im.h - 1);
    return __ldg(texel_ptr<float>(im, x, y));
}
__device__ __forceinline__ uint32_t fetch_r32u(const Img& im, int x, int y) {
    if (!im.p) return 0u;
    x = clampi(x, 0, im.w - 1);
    y = clampi(y, 0, im.h - 1);
    return __ldg(texel_ptr<uint32_t>(im, x, y));
}
__device__ __forceinline__ float4 fetch_rgba32f(const Img& im, int x, int y) {
    if (!im.p) return make_float4(0.f, 0.f, 0.f, 0.f);
    x = clampi(x, 0, im.w - 1);
    y = clampi(y, 0, im.h - 1);
    return __ldg(texel_ptr<float4>(im, x, y));
}
// Velocity with 2 or 4 channels (missing channels read 0).
template <int MC> __device__ __forceinline__ float4 fetch_velocity(const Img& im, int x, int y) {
    x = clampi(x, 0, im.w - 1);
    y = clampi(y, 0, im.h - 1);
    if (MC == 4) return half4_to_float4(__ldg(texel_ptr<uint2>(im, x, y)));
    uint32_t v = __ldg(texel_ptr<uint32_t>(im, x, y));
    float2 f = __half22float2(*reinterpret_cast<__half2*>(&v));
    return make_float4(f.x, f.y, 0.f, 0.f);
}
// History texel in either format (null history reads zeros).
template <int HF> __device__ __forceinline__ float4 fetch_history(const Img& im, int x, int y) {
    if (!im.p) return make_float4(0.f, 0.f, 0.f, 0.f);
    x = clampi(x, 0, im.w - 1);
    y = clampi(y, 0, im.h - 1);
    if (HF == 0) return __ldg(texel_ptr<float4>(im, x, y));
    return half4_to_float4(__ldg(texel_ptr<uint2>(im, x, y)));
}

template <class T> __device__ __forceinline__ T* texel_ptr_w(const ImgW& im, int x, int y) {
    return reinterpret_cast<T*>(im.p + (size_t)y * im.pitch) + x;
}
__device__ __forceinline__ void store_rgba16f(const ImgW& im, int x, int y, float4 v) {
    *texel_ptr_w<uint2>(im, x, y) = float4_to_half4(v);
}
template <int HF> __device__ __forceinline__ void store_history(const ImgW& im, int x, int y, float4 v) {
    if (HF == 0) *texel_ptr_w<float4>(im, x, y) = v;
    else *texel_ptr_w<uint2>(im, x, y) = float4_to_half4(v);
}

__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }

// Exact-weight bilinear sample at (u, v) of a w x h image read through
// tex(x, y), clamp to edge (texel centres at k + 0.5) - the sampler model of
// the oracle; a NaN fraction weights the first tap by 1.
template <class F>
__device__ __forceinline__ float4 bilinear_uv(int w, int h, float u, float v, F&& tex) {
    float px = u * (float)w - 0.5f;
    float py = v * (float)h - 0.5f;
    float fx0 = floorf(px), fy0 = floorf(py);
    float fx = px - fx0, fy = py - fy0;
    int x0 = trunc_index(fx0), y0 = trunc_index(fy0);
    if (!(fx == fx)) fx = 0.f;
    if (!(fy == fy)) fy = 0.f;
    int xa = clampi(x0, 0, w - 1), xb = clampi(x0 + 1 < x0 ? x0 : x0 + 1, 0, w - 1);
    int ya = clampi(y0, 0, h - 1), yb = clampi(y0 + 1 < y0 ? y0 : y0 + 1, 0, h - 1);
    float4 a = tex(xa, ya), b = tex(xb, ya), c = tex(xa, yb), d = tex(xb, yb);
    float gx = 1.0f - fx, gy = 1.0f - fy;
    float4 top = make_float4(a.x * gx + b.x * fx, a.y * gx + b.y * fx, a.z * gx + b.z * fx, a.w * gx + b.w * fx);
    float4 bot = make_float4(c.x * gx + d.x * fx, c.y * gx + d.y * fx, c.z * gx + d.z * fx, c.w * gx + d.w * fx);
    return make_float4(top.x * gy + bot.x * fy, top.y * gy + bot.y * fy, top.z * gy + bot.z * fy,
                       top.w * gy + bot.w * fy);
}

// taa.comp:222-257: which jittered source sample lands in a target texel of
// a loW x loH -> hiW x hiH upsampling.  The shader tries the four corner
// offsets (0, 0), (1, 0), (0, 1), (1, 1) (1 = 0.999999) and keeps the last
// sample that lands in the texel; each coordinate depends on one axis only,
// so the candidates are formed per axis (upsample_axis, the shader's
// arithmetic on that axis) and paired (upsampled_pick).
struct UpAxis {
    float s[2];    // the candidate sample coordinate for offsets 0 and 0.999999
    bool hit[2];   // whether it lands in the texel on this axis
};
__device__ __forceinline__ UpAxis upsample_axis(int t, int hi, int lo, float tj, float scale) {
    UpAxis r;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float o = j ? 0.999999f : 0.f;
        r.s[j] = floorf((float)lo * ((float)t + o) / (float)hi) + 0.5f + tj;
        r.hit[j] = trunc_index(r.s[j] * scale) == t;
    }
    return r;
}
// The jitter of an axis in source texels (taa.comp:225-227) and the axis scale.
__host__ __device__ __forceinline__ float upsample_jitter(float jitter_ndc, float unjitter_factor, int lo) {
    return jitter_ndc * 0.5f * unjitter_factor * (float)lo * -1.0f;
}
// True (beta = 1) with the source texel (fx, fy) when a sample lands.
__device__ __forceinline__ bool upsampled_pick(const UpAxis& X, const UpAxis& Y, int& fx, int& fy) {
    float fdx = -1.f, fdy = -1.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int jx = k & 1, jy = k >> 1;
        if (X.hit[jx] && Y.hit[jy]) {
            fdx = X.s[jx];
            fdy = Y.s[jy];
        }
    }
    fx = trunc_index(floorf(fdx));
    fy = trunc_index(floorf(fdy));
    return fdx >= 0.0f;
}
__device__ __forceinline__ bool upsampled_source(const taa_uniforms_t& U, const taa_parameters_t& P, int tx, int ty,
                                                 int hiW, int hiH, int loW, int loH, int& fx, int& fy) {
    const UpAxis X = upsample_axis(tx, hiW, loW, upsample_jitter(U.mJitterNdc[0], P.mUnjitterFactor, loW),
                                   (float)hiW / (float)loW);
    const UpAxis Y = upsample_axis(ty, hiH, loH, upsample_jitter(U.mJitterNdc[1], P.mUnjitterFactor, loH),
                                   (float)hiH / (float)loH);
    return upsampled_pick(X, Y, fx, fy);
}

// taa.comp:551-556: the noise added to the result when mAddNoise is set,
// seeded by the pixel's uv and mSinTime.x.
__device__ __forceinline__ float4 taa_noise(const taa_uniforms_t& U, const taa_parameters_t& P, float u, float v) {
    const float sx = u + U.mSinTime[0] + 0.6959174f, sy = v + U.mSinTime[0] + 0.6959174f;
    const float s = sinf(sx * 12.9898f + sy * 78.233f);
    const float f = P.mNoiseFactor;
    return make_float4((fractf(s * 43758.5453f) * 2.0f - 1.0f) * f, (fractf(s * 28001.8384f) * 2.0f - 1.0f) * f,
                       (fractf(s * 50849.4141f) * 2.0f - 1.0f) * f, (fractf(s * 12996.89f) * 2.0f - 1.0f) * f);
}

// taa.comp:912-942: a pixel's debug output - mode mDebugMode of the box
// extents (0, 1), the rejection and the rectification's move (2), the blend
// weight (3), the velocity (4), the pixel speed (5), the screen and history
// values (6, 7) or the ray-trace-assist class (8) - scaled by mDebugScale and
// the mask and optionally centred.  Shared by the plain and tiled forms.
struct DebugIn {
    float3 mn, mx, rdiff;  // box bounds, clipped minus unclipped history (working space)
    bool rejected;
    float alpha, speed;     // the blend weight (after a reset), |uv - history uv|
    float4 vel, to_screen, to_hist;
    uint32_t seg;
};
__device__ __forceinline__ float4 debug_value(const taa_parameters_t& P, const DebugIn& d) {
    float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
    switch (P.mDebugMode) {
        case 0: g = make_float4(d.mx.x - d.mn.x, d.mx.y - d.mn.y, d.mx.z - d.mn.z, 0.f); break;
        case 1: {
            const float tx = d.mx.x - d.mn.x, ty = d.mx.y - d.mn.y, tz = d.mx.z - d.mn.z;
            const float v = tx * ty * tz;
            g = make_float4(v, v, v, 0.f);
            break;
        }
        case 2: {
            const float l = sqrtf(d.rdiff.x * d.rdiff.x + d.rdiff.y * d.rdiff.y + d.rdiff.z * d.rdiff.z);
            g = make_float4(d.rejected ? 1.f : 0.f, l, 0.f, 0.f);
            break;
        }
        case 3: g = make_float4(d.alpha, d.alpha, d.alpha, 0.f); break;
        case 4: g = d.vel; break;
        case 5: g = make_float4(d.speed, 0.f, 0.f, 0.f); break;
        case 6: g = d.to_screen; break;
        case 7: g = d.to_hist; break;
        case 8:
            switch (d.seg & 3u) {
                case 0: g = make_float4(0.f, 0.f, 1.f, 0.f); break;
                case 1: g = make_float4(1.f, 0.f, 0.f, 0.f); break;
                case 2: g = make_float4(1.f, 1.f, 0.f, 0.f); break;
                default: break;
            }
            break;
        default: break;
    }
    const float s = P.mDebugScale;
    g = make_float4(g.x * (s * P.mDebugMask[0]), g.y * (s * P.mDebugMask[1]), g.z * (s * P.mDebugMask[2]),
                    g.w * (s * P.mDebugMask[3]));
    if (P.mDebugCenter) g = make_float4(g.x * 0.5f + 0.5f, g.y * 0.5f + 0.5f, g.z * 0.5f + 0.5f, g.w * 0.5f + 0.5f);
    return g;
}

// Correctly rounded x / d for a constant divisor d with precomputed
// rd = RN(1/d): one product and one FMA-based residual correction
// (P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990).  The identity is
// checked exhaustively against IEEE division on the CPU for the divisors the
// kernels use.
__device__ __forceinline__ float div_const_rn(float x, float d, float rd) {
    float q = __fmul_rn(x, rd);
    float r = __fmaf_rn(-d, q, x);
    return __fmaf_rn(r, rd, q);
}

}  // namespace taa_dev
