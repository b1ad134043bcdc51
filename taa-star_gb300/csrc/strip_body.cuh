// strip_body.cuh - the tile body of the fast resolve forms (TAA_FORM_FAST and
// the learned rectifier's inference): 32x16 tiles of 128 threads, each a
// vertical strip of four pixels, with the arithmetic of the colour staging,
// the 3x3 box and the clip decision supplied by a policy class
// (resolve_fast32.cu: FP32; resolve_learned_strips.cu: the learned rectifier).
// The FP32 policy (TAA_FORM_FAST) is the resolve of the benchmark mode of the
// parameter block (YCoCg variance clip toward the box centre, velocity for
// every pixel, simple velocity sampling; Catmull-Rom or bilinear history;
// optional depth culling and out-of-screen rejection; RGBA32F history) in
// FP32 with the arithmetic reassociated for speed instead of rounded like
// the shader:
//
//   * the 3x3 moments (taa.comp:266-277) come from row sums that a thread's
//     vertically adjacent pixels share, with Cg and Cg^2 staged side by side
//     so one packed add accumulates both, and mean = m1 * (1/9);
//   * the separable Catmull-Rom filter (taa.comp:469-495) filters a row once
//     for every pixel of a strip that shares its horizontal position;
//   * the standard deviation is the hardware square-root approximation, the
//     clip's per-channel ratios (taa.comp:323-345) use the hardware
//     reciprocal approximation; the box centre is the mean and its half
//     extent gamma * sigma + 1e-7 (the shader's (max + min) / 2 and
//     (max - min) / 2 + 1e-7 of mean -/+ gamma * sigma);
//   * multiplies and adds contract into FMAs (uv stays the correctly rounded
//     (x + 0.5) / size: an ulp of uv moves a 4K Catmull-Rom tap by 1e-4 texel).
//
// Structure: a 32x16 tile per 128-thread CTA (eight CTAs per SM), each thread
// a vertical strip of four pixels; the colour tile with its 1-pixel halo
// staged in shared memory as YCoCg; a history window per tile (the
// Catmull-Rom taps of the tile's centre pixel widened by the tile and 3
// pixels of motion difference) copied by one TMA tensor copy on a bounded
// mbarrier wait, or by cp.async with edge clamps where it crosses the image
// border; pixels whose taps leave the window read global memory.  The window
// is placed by the thread that owns the tile's centre pixel, from the
// velocity it has loaded for its own pixel, so no extra load delays the copy.
// The kernel is bound by the shared-memory pipe (window and box reads), so
// the strip shares what it can: a strip with one horizontal position (equal
// velocity x) filters each of its seven window rows horizontally once and
// gives each pixel the vertical combination (7 x 4 taps for four pixels
// instead of 4 x 16), and its boxes share the staged rows (six rows of three
// texels for four pixels).
//
// Precision: frame relative L2 within 1e-4 of the FP64 oracle and of the
// exact FP32 forms on the benchmark sequences (measured 2e-5 to 6e-5, the
// distance at which the exact FP32 form itself sits from FP64), within 1e-5
// on the reference's golden fixtures (tests/test_gpu_fast.py).
#pragma once
#include <cuda.h>

#include <cstring>
#include <type_traits>

#include "kernels.h"
#include "sharpen.cuh"
#include "tiled_skeleton.cuh"

namespace taa_dev {
namespace fast32 {

using tiled::cp_async;
using tiled::cp_async_commit;
using tiled::cp_async_wait_all;
using tiled::first_wait_polls;
using tiled::mbar_expect_tx;
using tiled::mbar_init;
using tiled::mbar_wait_bounded;
using tiled::tma_load_3d;

// Resident CTAs per SM the register budget is sized for (a tuning constant).
#ifndef TAA_FAST_MIN_BLOCKS
#define TAA_FAST_MIN_BLOCKS 8
#endif
// Whether the history window's TMA copy treats a row as one run of floats
// (2-D tensor map) rather than one 16-byte texel per request (3-D map).
#ifndef TAA_FAST_TMA2D
#define TAA_FAST_TMA2D 1
#endif
// Whether a thread's two pixels read their Catmull-Rom rows once when their
// footprints are one row apart (a tuning switch).
#ifndef TAA_FAST_SHARED_TAPS
#define TAA_FAST_SHARED_TAPS 1
#endif

constexpr int NPX = 4;                            // pixels per thread: a vertical strip
constexpr int TX = 32, TY = 16, NT = TX * TY / NPX;  // tile, threads (one warp per 32 x 4 rows)
constexpr int SX = TX + 2, SY = TY + 2, NS = SX * SY;  // staged colour with its 1-pixel halo
constexpr int NSPT = (NS + NT - 1) / NT;               // staged texels per thread
constexpr int MARGIN = tiled::WIN_MARGIN;
constexpr int WW = TX + 3 + 2 * MARGIN, WH = TY + 3 + 2 * MARGIN;  // history window (texels)
constexpr int REF_TID = (TY / 2 / NPX) * 32 + TX / 2;  // the thread whose first pixel is the centre (16, 8)
static_assert(NPX * NT == TX * TY && NT % 32 == 0, "whole warps of strips");

// Everything a launch reads, flattened: pointers, row pitches in bytes, the
// few parameters the benchmark mode uses.
struct Args {
    const char* color;  // RGBA16F
    const char* depth;  // D32F
    const char* vel;    // RG16F or RGBA16F
    const char* hist;   // RGBA32F, or null (reads zeros)
    const char* hdepth; // D32F previous depth, or null
    char* hout;         // RGBA32F
    char* result;       // RGBA16F, or null
    unsigned int* status;
    uint32_t color_pitch, depth_pitch, vel_pitch, hist_pitch, hdepth_pitch, hout_pitch, result_pitch;
    int W, H;
    float inv_w, inv_h;  // correctly rounded 1 / W, 1 / H
    float alpha, rejection_alpha, gamma;
    int reject_outside, depth_cull, reset;
    int hout_half;       // history_out is RGBA16F (the history window then holds RGBA16F texels too)
};

// What a policy that may reproject reads besides Args (a kernel parameter of
// its own, so that the other kernels' arguments stay small).
struct Reproj {
    int vel_mode;                   // mUseVelocityVectors: 0 reproject, 1 velocity for movers, 2 for every pixel
    float inv_vp[16], hist_vp[16];  // mInverseViewProjMatrix, mHistoryViewProjMatrix (column-major)
    // the blend-weight modifiers and the chroma-axis shrink (taa.comp:283-311, 855-895),
    // read by the policies that run them
    int shrink, vel_alpha, lottes, near_clamp;
    float vel_alpha_max, vel_alpha_factor, min_alpha, max_alpha;
};
inline Reproj make_reproj(const taa_uniforms_t& U) {
    const taa_parameters_t& P = U.param[0];
    Reproj r;
    r.vel_mode = P.mUseVelocityVectors;
    for (int i = 0; i < 16; ++i) {
        r.inv_vp[i] = U.mInverseViewProjMatrix[i];
        r.hist_vp[i] = U.mHistoryViewProjMatrix[i];
    }
    r.shrink = P.mUseYCoCg && P.mShrinkChromaAxis;
    r.vel_alpha = P.mVelBasedAlpha != 0;
    r.lottes = P.mLumaWeightingLottes != 0;
    r.near_clamp = P.mReduceBlendNearClamp != 0;
    r.vel_alpha_max = P.mVelBasedAlphaMax;
    r.vel_alpha_factor = P.mVelBasedAlphaFactor;
    r.min_alpha = P.mMinAlpha;
    r.max_alpha = P.mMaxAlpha;
    return r;
}

// The arguments of a launch from a view's uniform block and bindings.
__host__ __device__ inline Args make_args(const taa_uniforms_t& U, const FrameArgs& f) {
    const taa_parameters_t& P = U.param[0];
    Args a;
    a.color = f.color.p;
    a.depth = f.depth.p;
    a.vel = f.velocity.p;
    a.hist = f.history.p;
    a.hdepth = f.history_depth.p;
    a.hout = f.history_out.p;
    a.result = f.result.p;
    a.status = f.status;
    a.color_pitch = (uint32_t)f.color.pitch;
    a.depth_pitch = (uint32_t)f.depth.pitch;
    a.vel_pitch = (uint32_t)f.velocity.pitch;
    a.hist_pitch = (uint32_t)f.history.pitch;
    a.hdepth_pitch = (uint32_t)f.history_depth.pitch;
    a.hout_pitch = (uint32_t)f.history_out.pitch;
    a.result_pitch = (uint32_t)f.result.pitch;
    a.W = f.out_w;
    a.H = f.out_h;
    a.inv_w = f.inv_out_w;
    a.inv_h = f.inv_out_h;
    a.alpha = P.mAlpha;
    a.rejection_alpha = P.mRejectionAlpha;
    a.gamma = P.mVarClipGamma;
    a.reject_outside = P.mRejectOutside != 0;
    a.depth_cull = P.mDepthCulling != 0;
    a.reset = U.mResetHistory != 0;
    a.hout_half = 0;
    return a;
}

// The history window's texel type and row length: RGBA32F texels, or (HF 1)
// RGBA16F texels in a row one texel longer, its origin on an even texel (a
// TMA coordinate is a multiple of 16 bytes).
template <int HF> struct WinOf {
    using T = float4;
    static constexpr int W = WW;
};
template <> struct WinOf<1> {
    using T = uint2;
    static constexpr int W = WW + 1;
};

template <class Staged, int HF = 0> struct SmemT {
    Staged col[NS];                                       // the staged colour tile in the policy's format
    alignas(128) typename WinOf<HF>::T win[WinOf<HF>::W * WH];  // the history window
    uint64_t bar;                                         // completion of the window's TMA copy
    int org[3];                                           // window origin x, y; 1 TMA, 2 cp.async, 0 none
    int abort;                                            // a persistent CTA stops after this tile (a window wait gave up)
};

template <class T> __device__ __forceinline__ const T* at(const char* base, uint32_t pitch, int x, int y) {
    return reinterpret_cast<const T*>(base + (size_t)(uint32_t)y * pitch) + x;
}
template <class T> __device__ __forceinline__ T* at_w(char* base, uint32_t pitch, int x, int y) {
    return reinterpret_cast<T*>(base + (size_t)(uint32_t)y * pitch) + x;
}

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ f2 mulp(f2 a, f2 b) {
    f2 d;
    asm("mul.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 addp(f2 a, f2 b) {
    f2 d;
    asm("add.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 fmap(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return d;
}

// One 16-byte shared-memory load.  A float4 whose fourth lane is unused would
// otherwise be read as an 8-byte and a 4-byte load; at the 16-byte stride of
// consecutive texels each of those occupies the shared-memory pipe as long as
// the whole 16 bytes do.
__device__ __forceinline__ uint2 lds64(const uint2* p) {
    uint2 v;
    asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(tiled::smem_addr(p)));
    return v;
}
__device__ __forceinline__ float4 lds128(const float4* p) {
    float4 v;
    // volatile: kept in program order with the barrier waits that publish the data
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "r"(tiled::smem_addr(p)));
    return v;
}
// A history texel of the window as FP32 (RGBA16F texels widened).
__device__ __forceinline__ float4 win_texel(const float4* p) { return lds128(p); }
__device__ __forceinline__ float4 win_texel(const uint2* p) { return half4_to_float4(lds64(p)); }

// RGBA16F texel -> YCoCg in FP32 (taa.comp:158-164)
__device__ __forceinline__ float3 ycocg(uint2 raw) {
    const float4 c = half4_to_float4(raw);
    const float rb = c.x + c.z;
    return make_float3(0.25f * rb + 0.5f * c.y, 0.5f * (c.x - c.z), 0.5f * c.y - 0.25f * rb);
}

// The clip toward the box centre m with the ratio ma (taa.comp:335-340: the
// history moves to m + (h - m) / ma when ma > 1), the blend with the current
// colour (taa.comp:848-900: mix(history, current, alpha)), the conversion
// back to RGB and the stores of the history (alpha 0) and the screen.
// The clipped, blended colour in RGB: (r, g, b, 0).
__device__ __forceinline__ float4 clip_blend(const float hc[3], const float m[3], float ma, const float cur[3],
                                             float alpha) {
    const float sc = ma > 1.0f ? rcp_approx(ma) : 1.0f;
    float o[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float hcl = fmaf(hc[c] - m[c], sc, m[c]);
        o[c] = fmaf(alpha, cur[c] - hcl, hcl);
    }
    const float tmp = o[0] - o[2];
    return make_float4(tmp + o[1], o[0] + o[2], tmp - o[1], 0.f);
}
__device__ __forceinline__ void store_out(const Args& a, int x, int y, float4 o) {
    if (a.hout_half) *at_w<uint2>(a.hout, a.hout_pitch, x, y) = float4_to_half4(o);
    else *at_w<float4>(a.hout, a.hout_pitch, x, y) = o;
    if (a.result) *at_w<uint2>(a.result, a.result_pitch, x, y) = float4_to_half4(make_float4(o.x, o.y, o.z, 1.0f));
}
__device__ __forceinline__ void clip_blend_store(const Args& a, int x, int y, const float hc[3], const float m[3],
                                                 float ma, const float cur[3], float alpha) {
    store_out(a, x, y, clip_blend(hc, m, ma, cur, alpha));
}
// The history sample in YCoCg (taa.comp:158-164).
__device__ __forceinline__ void hist_ycocg(float3 h, float hc[3]) {
    hc[0] = 0.25f * (h.x + h.z) + 0.5f * h.y;
    hc[1] = 0.5f * (h.x - h.z);
    hc[2] = 0.5f * h.y - 0.25f * (h.x + h.z);
}

// The 3x3 moments of one staged row segment (three texels): the (Y, Co) sum,
// the (Cg, Cg^2) sum and the (Y^2, Co^2) sum.
struct Row {
    f2 a, c, q;
};
__device__ __forceinline__ Row row_sums(const float4* p) {
    f2 a0, c0, a1, c1, a2, c2;
    load_pairs(p, a0, c0);
    load_pairs(p + 1, a1, c1);
    load_pairs(p + 2, a2, c2);
    Row r;
    r.a = addp(addp(a0, a1), a2);
    r.c = addp(addp(c0, c1), c2);
    r.q = fmap(a2, a2, fmap(a1, a1, mulp(a0, a0)));
    return r;
}
__device__ __forceinline__ Row add(const Row& u, const Row& v) { return {addp(u.a, v.a), addp(u.c, v.c), addp(u.q, v.q)}; }

// The variance box of one pixel: centre (the mean) and half extent gamma * sigma + 1e-7.
struct Box {
    float m[3], e[3];
};
__device__ __forceinline__ Box box_of(const Row& s, float gamma) {
    const f2 n = dup(1.0f / 9.0f);
    const f2 mean = mulp(s.a, n);  // (Y, Co)
    const f2 cg = mulp(s.c, n);    // (mean Cg, m2 Cg / 9)
    const f2 var = fmap(neg2(mean), mean, mulp(s.q, n));
    const float var_cg = fmaf(-f2lo(cg), f2lo(cg), f2hi(cg));
    Box b;
    b.m[0] = f2lo(mean);
    b.m[1] = f2hi(mean);
    b.m[2] = f2lo(cg);
    b.e[0] = fmaf(gamma, sqrt_approx(fmaxf(f2lo(var), 0.f)), 1e-7f);
    b.e[1] = fmaf(gamma, sqrt_approx(fmaxf(f2hi(var), 0.f)), 1e-7f);
    b.e[2] = fmaf(gamma, sqrt_approx(fmaxf(var_cg, 0.f)), 1e-7f);
    return b;
}

// Catmull-Rom weights of both axes as (x, y) pairs (taa.comp:464-467, the
// same polynomials in Horner form), and the first tap.
struct Taps {
    f2 w[4];
    int ux, uy;
};
template <int INTERP>
__device__ __forceinline__ Taps taps_of(float hu, float hv, const Args& a) {
    Taps t;
    const f2 it = mulp(pk(hu, hv), pk((float)a.W, (float)a.H));
    const float bx = floorf(f2lo(it) - 0.5f), by = floorf(f2hi(it) - 0.5f);
    const f2 f = addp(it, pk(-0.5f - bx, -0.5f - by));
    if constexpr (INTERP == 2) {
        const f2 one = dup(1.0f), half = dup(0.5f);
        const f2 f2_ = mulp(f, f);
        t.w[0] = mulp(f, fmap(f, fmap(dup(-0.5f), f, one), dup(-0.5f)));
        t.w[1] = fmap(f2_, fmap(dup(1.5f), f, dup(-2.5f)), one);
        t.w[2] = mulp(f, fmap(f, fmap(dup(-1.5f), f, dup(2.0f)), half));
        t.w[3] = mulp(mulp(half, f2_), addp(f, dup(-1.0f)));
        t.ux = trunc_index(bx) - 1;
        t.uy = trunc_index(by) - 1;
    } else {
        // bilinear (taa.comp:546): weights (1 - f, f); a NaN fraction weights the first tap by 1
        float fx = f2lo(f), fy = f2hi(f);
        if (!(fx == fx)) fx = 0.f;
        if (!(fy == fy)) fy = 0.f;
        t.w[0] = pk(1.0f - fx, 1.0f - fy);
        t.w[1] = pk(fx, fy);
        t.ux = trunc_index(bx);
        t.uy = trunc_index(by);
    }
    return t;
}

// The filter over N x N texels read through tex(i, j): rows of N taps
// weighted by x, then the rows weighted by y; (R, G) as a pair, B alone.
template <int N, class F> __device__ __forceinline__ float3 filter(const Taps& t, F&& tex) {
    f2 acc = dup(0.f);
    float accb = 0.f;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        f2 r = dup(0.f);
        float rb = 0.f;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const float4 s = tex(i, j);
            const float wx = f2lo(t.w[i]);
            r = fmap(dup(wx), pk(s.x, s.y), r);
            rb = fmaf(wx, s.z, rb);
        }
        const float wy = f2hi(t.w[j]);
        acc = fmap(dup(wy), r, acc);
        accb = fmaf(wy, rb, accb);
    }
    return make_float3(f2lo(acc), f2hi(acc), accb);
}

// Catmull-Rom (or bilinear) weights of one axis at fraction f (taa.comp:464-467).
template <int INTERP> __device__ __forceinline__ void axis_weights(float f, float w[4]) {
    if constexpr (INTERP == 2) {
        const float f2 = f * f;
        w[0] = f * fmaf(f, fmaf(-0.5f, f, 1.0f), -0.5f);
        w[1] = fmaf(f2, fmaf(1.5f, f, -2.5f), 1.0f);
        w[2] = f * fmaf(f, fmaf(-1.5f, f, 2.0f), 0.5f);
        w[3] = 0.5f * f2 * (f - 1.0f);
    } else {
        if (!(f == f)) f = 0.f;  // a NaN fraction weights the first tap by 1 (taa.comp:546)
        w[0] = 1.0f - f;
        w[1] = f;
        w[2] = w[3] = 0.f;
    }
}
// The first tap of an axis and its fraction: it = position * size.
// `it` is the texel-space position, a separately rounded product (__fmul_rn:
// a product the compiler contracted into the subtraction below would round
// the fraction differently from taps_of's, and a pixel's history sample would
// depend on whether its strip takes the shared-row path).
template <int INTERP> __device__ __forceinline__ int axis_first(float it, float& f) {
    const float b = floorf(it - 0.5f);
    f = it + (-0.5f - b);
    return trunc_index(b) - (INTERP == 2 ? 1 : 0);
}

// One 32x16 tile (tile_x, tile_y) of a view; every thread of the CTA calls it.
// `phase` is the parity the window barrier completes next (PERSIST: the CTA
// takes several tiles with one barrier initialised by the caller; otherwise
// the thread that starts the copy initialises it).  A wait that gives up sets
// the status bit and leaves the tile unwritten; with PERSIST it also sets
// sm.abort, which the caller reads after the barrier that separates tiles.
// Whether a policy's parameter mode may reproject a pixel through the
// matrices instead of its velocity (mUseVelocityVectors 0 or 1): its
// `static constexpr bool kReproject`, false when it has none; such a policy's
// Ctx holds `const Reproj* rp`.
template <class P, class = void> struct reprojects : std::false_type {};
template <class P> struct reprojects<P, std::void_t<decltype(P::kReproject)>> : std::bool_constant<P::kReproject> {};

// taa.comp:426-430: the pixel's history position and expected depth from the
// depth and the two matrices (FP32; the fast forms' reassociated arithmetic).
__device__ __forceinline__ void reproject(const Reproj& a, float u, float v, float depth, float& hu, float& hv,
                                          float& ehd) {
    const float c0 = fmaf(u, 2.0f, -1.0f), c1 = fmaf(v, 2.0f, -1.0f);
    float ws[4], hs[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        ws[i] = fmaf(a.inv_vp[i], c0, fmaf(a.inv_vp[4 + i], c1, fmaf(a.inv_vp[8 + i], depth, a.inv_vp[12 + i])));
#pragma unroll
    for (int i = 0; i < 4; ++i)
        hs[i] = fmaf(a.hist_vp[i], ws[0], fmaf(a.hist_vp[4 + i], ws[1], fmaf(a.hist_vp[8 + i], ws[2], a.hist_vp[12 + i] * ws[3])));
    const float rw = 1.0f / hs[3];
    hu = fmaf(hs[0] * rw, 0.5f, 0.5f);
    hv = fmaf(hs[1] * rw, 0.5f, 0.5f);
    ehd = hs[2] * rw;
}

// What a policy's finisher may read of the strip's pixels besides their
// boxes and history samples: uv, the history positions, the expected and the
// previous depth (a finisher that reads none of it costs nothing for it).
struct PixelInfo {
    float u, v[NPX], hu[NPX], hv[NPX], ehd[NPX], pd[NPX];
};

// ORIGIN: (tile_x, tile_y) is the pixel origin of the 32x16 region, which
// may start at -1 (a fused sharpener resolves a ring around its output);
// loads are then edge-clamped on every side and the policy chooses what it
// stores.
template <class Pol, int INTERP, int MC, bool PERSIST, bool ORIGIN = false, int HF = 0>
__device__ __forceinline__ void strip_tile(const Args& a, const CUtensorMap* hmap, int tma_ok, int tile_x,
                                           int tile_y, SmemT<typename Pol::Staged, HF>& sm, uint32_t& phase,
                                           typename Pol::Ctx& ctx) {
    using HistT = typename WinOf<HF>::T;
    constexpr int WWS = WinOf<HF>::W;  // the window's row length in texels
    using RawVel = typename std::conditional<MC == 4, uint2, uint32_t>::type;
    constexpr int SPAN = INTERP == 2 ? 4 : 2;
    const int tid = threadIdx.x, lx = tid & 31, sy = tid >> 5;
    const int W = a.W, H = a.H;
    const int x0 = ORIGIN ? tile_x : tile_x * TX, y0 = ORIGIN ? tile_y : tile_y * TY;
    // a pixel's loads at edge-clamped coordinates
    auto crow = [&](int y) { return ORIGIN ? clampi(y, 0, H - 1) : min(y, H - 1); };
    const int x = x0 + lx, cx = ORIGIN ? clampi(x, 0, W - 1) : min(x, W - 1);
    const int ya = y0 + NPX * sy;  // the strip's first row
    const bool have_hist = a.hist != nullptr;

    // 1. loads: the strip's depths and velocities, this thread's staged colour texels
    float dep[NPX];
    RawVel vraw[NPX];
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        const int cy = crow(ya + k);
        dep[k] = __ldg(at<float>(a.depth, a.depth_pitch, cx, cy));
        vraw[k] = __ldg(at<RawVel>(a.vel, a.vel_pitch, cx, cy));
    }
    uint2 st[NSPT];
#pragma unroll
    for (int j = 0; j < NSPT; ++j) {
        const int i = tid + j * NT;
        st[j] = make_uint2(0u, 0u);
        if (j < NSPT - 1 || i < NS) {
            const int ry = i / SX, rx = i - ry * SX;
            st[j] = __ldg(at<uint2>(a.color, a.color_pitch, clampi(x0 - 1 + rx, 0, W - 1), clampi(y0 - 1 + ry, 0, H - 1)));
        }
    }
    // the first window wait's poll limit, loaded with the inputs
    const uint32_t polls = first_wait_polls(a.status);
    // 2. history positions (uv - velocity; uv = (texel + 0.5) / size correctly
    //    rounded: a sampling position one ulp off moves a 4K Catmull-Rom tap by
    //    1e-4 texel), the previous depth under them
    PixelInfo px;
    px.u = div_const_rn((float)cx + 0.5f, (float)W, a.inv_w);
    float (&hu)[NPX] = px.hu, (&hv)[NPX] = px.hv, (&ehd)[NPX] = px.ehd, (&pd)[NPX] = px.pd;
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        const float4 vel = tiled::velocity_of<MC>(vraw[k]);
        px.v[k] = div_const_rn((float)crow(ya + k) + 0.5f, (float)H, a.inv_h);
        bool use_velocity = true;
        if constexpr (reprojects<Pol>::value) {
            const int vm = ctx.rp->vel_mode;
            use_velocity = vm == 2 || (vm == 1 && vel.w >= 0.5f);
            if (!use_velocity) reproject(*ctx.rp, px.u, px.v[k], dep[k], hu[k], hv[k], ehd[k]);
        }
        if (use_velocity) {
            hu[k] = px.u - vel.x;
            hv[k] = px.v[k] - vel.y;
            ehd[k] = dep[k] - vel.z;
        }
        pd[k] = 0.f;
        if (a.depth_cull && a.hdepth)
            pd[k] = __ldg(at<float>(a.hdepth, a.hdepth_pitch, clampi(trunc_index(hu[k] * (float)W), 0, W - 1),
                                    clampi(trunc_index(hv[k] * (float)H), 0, H - 1)));
    }
    // 3. the thread owning the tile's centre pixel places the history window
    //    (its own pixel's taps widened by the tile and MARGIN) and starts the copy
    if (tid == REF_TID && have_hist) {
        float f;
        const int rux = axis_first<INTERP>(__fmul_rn(hu[0], (float)W), f);
        const int ruy = axis_first<INTERP>(__fmul_rn(hv[0], (float)H), f);
        int wx0 = rux - (cx - x0) - MARGIN;
        if (HF == 1) wx0 -= wx0 & 1;  // an even texel: its TMA coordinate is a multiple of 16 bytes
        const int wy0 = ruy - (crow(ya) - y0) - MARGIN;
        const bool interior = wx0 >= 0 && wy0 >= 0 && wx0 <= W - WWS && wy0 <= H - WH;
        const int mode = tma_ok && interior ? 1 : 2;
        sm.org[0] = wx0;
        sm.org[1] = wy0;
        sm.org[2] = mode;
        if (mode == 1) {
            if (!PERSIST) mbar_init(&sm.bar, 1);
            mbar_expect_tx(&sm.bar, (uint32_t)(sizeof(HistT) * WWS * WH));
            if (TAA_FAST_TMA2D) tiled::tma_load_2d(sm.win, hmap, 4 * wx0, wy0, &sm.bar);
            else tma_load_3d(sm.win, hmap, 0, wx0, wy0, &sm.bar);
        }
    }
    // 4. staged colour
#pragma unroll
    for (int j = 0; j < NSPT; ++j) {
        const int i = tid + j * NT;
        if (j < NSPT - 1 || i < NS) sm.col[i] = Pol::stage(st[j]);
    }
    __syncthreads();
    int wx0 = 0, wy0 = 0, mode = 0;
    if (have_hist) {
        wx0 = sm.org[0];
        wy0 = sm.org[1];
        mode = sm.org[2];
    }
    if (mode == 2) {
        // a window across the image border: every texel edge-clamped
        const int lane = tid & 31, warp = tid >> 5;
        for (int r = warp; r < WH; r += NT / 32) {
            const int gy = clampi(wy0 + r, 0, H - 1);
            for (int c = lane; c < WWS; c += 32)
                cp_async<sizeof(HistT)>(&sm.win[r * WWS + c],
                                        at<HistT>(a.hist, a.hist_pitch, clampi(wx0 + c, 0, W - 1), gy));
        }
        cp_async_commit();
    }
    // rejection (taa.comp:787-823): out of the screen, or the previous depth
    // under the history position too far from the expected one
    unsigned rej = 0;
#pragma unroll
    for (int k = 0; k < NPX; ++k)
        if ((a.reject_outside && (hu[k] < 0.f || hv[k] < 0.f || hu[k] >= 1.f || hv[k] >= 1.f)) ||
            (a.depth_cull && fabsf(pd[k] - ehd[k]) > 0.1f * (1.0f - pd[k])))
            rej |= 1u << k;

    bool landed = true;
    if (mode == 1) {
        landed = mbar_wait_bounded(&sm.bar, phase & 1u, polls);
        if (!landed) {
            atomicOr(a.status, kStatusWindowTimeout);
            mbar_wait_bounded(&sm.bar, phase & 1u);  // the copy may still land in this CTA's memory
            if (PERSIST) sm.abort = 1;
        }
        phase ^= 1u;
    } else if (mode == 2) {
        cp_async_wait_all();
        __syncthreads();
    }
    // 5. the history samples.  A strip whose pixels share a horizontal
    //    position (equal velocity x) and whose footprints are one row apart
    //    filters each of its SPAN + NPX - 1 window rows horizontally once and
    //    gives every pixel its vertical combination of them.
    float3 h[NPX];
#pragma unroll
    for (int k = 0; k < NPX; ++k) h[k] = make_float3(0.f, 0.f, 0.f);
    if (have_hist && landed) {
        float fx, fy[NPX];
        const int ux = axis_first<INTERP>(__fmul_rn(hu[0], (float)W), fx);
        int uy[NPX];
        bool coherent = true;
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            uy[k] = axis_first<INTERP>(__fmul_rn(hv[k], (float)H), fy[k]);
            coherent = coherent && __float_as_uint(hu[k]) == __float_as_uint(hu[0]) && uy[k] == uy[0] + k;
        }
        const int bx = ux - wx0, by = uy[0] - wy0;
        coherent = coherent && (unsigned)bx <= (unsigned)(WWS - SPAN) && (unsigned)by <= (unsigned)(WH - SPAN - NPX + 1);
        if (TAA_FAST_SHARED_TAPS && coherent) {
            float wx[4], wy[NPX][4];
            axis_weights<INTERP>(fx, wx);
#pragma unroll
            for (int k = 0; k < NPX; ++k) axis_weights<INTERP>(fy[k], wy[k]);
            const HistT* wp = &sm.win[by * WWS + bx];
            f2 acc[NPX];
            float accb[NPX];
#pragma unroll
            for (int k = 0; k < NPX; ++k) {
                acc[k] = dup(0.f);
                accb[k] = 0.f;
            }
#pragma unroll
            for (int j = 0; j < SPAN + NPX - 1; ++j) {
                f2 r = dup(0.f);
                float rb = 0.f;
#pragma unroll
                for (int i = 0; i < SPAN; ++i) {
                    const float4 t = win_texel(&wp[j * WWS + i]);
                    r = fmap(dup(wx[i]), pk(t.x, t.y), r);
                    rb = fmaf(wx[i], t.z, rb);
                }
#pragma unroll
                for (int k = 0; k < NPX; ++k) {
                    if (j - k >= 0 && j - k < SPAN) {
                        acc[k] = fmap(dup(wy[k][j - k]), r, acc[k]);
                        accb[k] = fmaf(wy[k][j - k], rb, accb[k]);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < NPX; ++k) h[k] = make_float3(f2lo(acc[k]), f2hi(acc[k]), accb[k]);
        } else {
#pragma unroll
            for (int k = 0; k < NPX; ++k) {
                const Taps t = taps_of<INTERP>(hu[k], hv[k], a);
                const int tbx = t.ux - wx0, tby = t.uy - wy0;
                if ((unsigned)tbx <= (unsigned)(WWS - SPAN) && (unsigned)tby <= (unsigned)(WH - SPAN)) {
                    const HistT* wp = &sm.win[tby * WWS + tbx];
                    h[k] = filter<SPAN>(t, [&](int i, int j) { return win_texel(&wp[j * WWS + i]); });
                } else {
                    h[k] = filter<SPAN>(t, [&](int i, int j) {
                        const HistT* g = at<HistT>(a.hist, a.hist_pitch, clampi(t.ux + i, 0, W - 1),
                                                   clampi(t.uy + j, 0, H - 1));
                        if constexpr (HF == 1) return half4_to_float4(__ldg(g));
                        else return __ldg(g);
                    });
                }
            }
        }
    }
    // 6. per pixel: the box, clip, blend, stores (the policy's arithmetic)
    Pol::finish(a, &sm.col[(NPX * sy) * SX + lx], x, ya, h, rej, landed, px, ctx);
}

// The FP32 policy of TAA_FORM_FAST: the colour staged as (Y, Co, Cg, Cg^2)
// in FP32; the boxes from row sums the strip's pixels share.
struct F32Pol {
    using Staged = float4;
    struct Ctx {};
    static __device__ __forceinline__ float4 stage(uint2 raw) {
        const float3 c = ycocg(raw);
        return make_float4(c.x, c.y, c.z, c.z * c.z);
    }
    // the strip's pixels (x, ya + k): box from rows k .. k+2 of the six staged
    // rows at sp (the staged texel (x - 1, ya - 1)), clip, blend, stores
    static __device__ __forceinline__ void finish(const Args& a, const float4* sp, int x, int ya, const float3 h[NPX],
                                                  unsigned rej, bool landed, const PixelInfo&, Ctx&) {
        Row r0 = row_sums(sp), r1 = row_sums(sp + SX);
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            const Row r2 = row_sums(sp + (k + 2) * SX);
            const Row s = add(add(r0, r1), r2);
            r0 = r1;
            r1 = r2;
            const int y = ya + k;
            if (!(x < a.W && y < a.H && landed)) continue;
            store_out(a, x, y, pixel(a, s, h[k], (rej >> k) & 1u, &sp[(k + 1) * SX + 1]));
        }
    }
    // one pixel: the box from its 3x3 moments s, the clip of its history
    // sample h, the blend with its staged colour at c
    static __device__ __forceinline__ float4 pixel(const Args& a, const Row& s, float3 h, bool rejected,
                                                   const float4* c) {
        const Box b = box_of(s, a.gamma);
        float hc[3];
        hist_ycocg(h, hc);
        float ma = 0.f;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) ma = fmaxf(ma, fabsf(hc[ch] - b.m[ch]) * rcp_approx(b.e[ch]));
        const float alpha = a.reset ? 1.0f : (rejected ? a.rejection_alpha : a.alpha);
        const float4 c0 = lds128(c);
        const float cur[3] = {c0.x, c0.y, c0.z};
        return clip_blend(hc, b.m, ma, cur, alpha);
    }
};

// The 3x3 minimum and maximum of one staged row segment (three texels).
struct RowMinMax {
    float mn[3], mx[3];
};
__device__ __forceinline__ RowMinMax row_minmax(const float4* p) {
    const float4 t0 = lds128(p), t1 = lds128(p + 1), t2 = lds128(p + 2);
    return {{fminf(t0.x, fminf(t1.x, t2.x)), fminf(t0.y, fminf(t1.y, t2.y)), fminf(t0.z, fminf(t1.z, t2.z))},
            {fmaxf(t0.x, fmaxf(t1.x, t2.x)), fmaxf(t0.y, fmaxf(t1.y, t2.y)), fmaxf(t0.z, fmaxf(t1.z, t2.z))}};
}

// The policy of TAA_FORM_FAST for the reference's default parameter block
// (taa.hpp:31-76): RGB, the 3x3 minimum/maximum box (taa.comp:288-291) from
// row extrema the strip's pixels share, the history clamped to it
// (taa.comp:831), velocity for movers only or for every pixel, or
// reprojection through the matrices (taa.comp:393-431).
struct ClampRgbPol {
    using Staged = float4;
    struct Ctx {
        const Reproj* rp;
    };
    static constexpr bool kReproject = true;
    static __device__ __forceinline__ float4 stage(uint2 raw) {
        const float4 c = half4_to_float4(raw);
        return make_float4(c.x, c.y, c.z, 0.f);
    }
    static __device__ __forceinline__ void finish(const Args& a, const float4* sp, int x, int ya, const float3 h[NPX],
                                                  unsigned rej, bool landed, const PixelInfo&, Ctx&) {
        RowMinMax q0 = row_minmax(sp), q1 = row_minmax(sp + SX);
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            const RowMinMax q2 = row_minmax(sp + (k + 2) * SX);
            float mn[3], mx[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                mn[c] = fminf(q0.mn[c], fminf(q1.mn[c], q2.mn[c]));
                mx[c] = fmaxf(q0.mx[c], fmaxf(q1.mx[c], q2.mx[c]));
            }
            q0 = q1;
            q1 = q2;
            const int y = ya + k;
            if (!(x < a.W && y < a.H && landed)) continue;
            const float hs[3] = {h[k].x, h[k].y, h[k].z};
            const float4 c0 = lds128(&sp[(k + 1) * SX + 1]);
            const float cur[3] = {c0.x, c0.y, c0.z};
            const float alpha = a.reset ? 1.0f : ((rej >> k) & 1u ? a.rejection_alpha : a.alpha);
            float o[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float hc = fminf(fmaxf(hs[c], mn[c]), mx[c]);
                o[c] = fmaf(alpha, cur[c] - hc, hc);
            }
            store_out(a, x, y, make_float4(o[0], o[1], o[2], 0.f));
        }
    }
};

// TAA_FORM_FAST with a fused sharpener (TAA_FLAG_FUSED_SHARPEN): the strip
// body in RING mode resolves a 32x16 region around a 30x14 output tile, keeps
// the FP16-rounded screen colour of the whole region (what the two-pass form's
// sharpen pass reads back from the result image) over the dead history
// window, and sharpens the tile from there.  Each interior pixel is the value
// the two-pass form computes for it (the same arithmetic on the same inputs;
// the sharpeners round every operation), so the outputs are its bits.
// The ring costs 512 / 420 = 1.22x the resolves.  A CTA that sweeps a column
// of regions (each row resolved once, two rows carried in shared memory) cut
// that to 1.07x but ran 13% slower: its steps serialise each region's loads
// behind the previous region's arithmetic.
template <int SHARPEN>  // TAA_SHARPEN_SIMPLE or TAA_SHARPEN_CAS
struct FusedF32Pol {
    using Staged = float4;
    struct Ctx {
        uint2* screen;   // [TY][TX] RGBA16F region colour, over the window
        char* sharp;     // RGBA16F output
        uint32_t sharp_pitch;
        float k;         // CAS peak, or the simple sharpener's factor
    };
    static __device__ __forceinline__ float4 stage(uint2 raw) { return F32Pol::stage(raw); }
    static __device__ __forceinline__ void finish(const Args& a, const float4* sp, int x, int ya, const float3 h[NPX],
                                                  unsigned rej, bool landed, const PixelInfo&, Ctx& ctx) {
        const int lx = threadIdx.x & 31, row0 = NPX * (threadIdx.x >> 5);
        // x0 = x - lx >= -1: lx >= 1 puts x inside the image's left edge
        const bool col_in = lx >= 1 && lx <= TX - 2 && x < a.W;
        uint2 scr[NPX];
        Row r0 = row_sums(sp), r1 = row_sums(sp + SX);
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            const Row r2 = row_sums(sp + (k + 2) * SX);
            const Row s = add(add(r0, r1), r2);
            r0 = r1;
            r1 = r2;
            // every pixel of the region (ring and outside pixels from edge-clamped loads)
            const float4 o = F32Pol::pixel(a, s, h[k], (rej >> k) & 1u, &sp[(k + 1) * SX + 1]);
            scr[k] = float4_to_half4(make_float4(o.x, o.y, o.z, 1.0f));
            const int row = row0 + k, y = ya + k;
            if (col_in && row >= 1 && row <= TY - 2 && y < a.H && landed) store_out(a, x, y, o);
        }
        __syncthreads();  // every thread is done with the window the screen overlays
#pragma unroll
        for (int k = 0; k < NPX; ++k) ctx.screen[(row0 + k) * TX + lx] = scr[k];
        __syncthreads();
        if (!ctx.sharp || !col_in || !landed) return;
        const int x0 = x - lx, y0 = ya - row0;
        auto at = [&](int gx, int gy) {
            const uint2 v = ctx.screen[(clampi(gy, 0, a.H - 1) - y0) * TX + (clampi(gx, 0, a.W - 1) - x0)];
            const float4 c = half4_to_float4(v);
            return make_float3(c.x, c.y, c.z);
        };
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            const int row = row0 + k, y = ya + k;
            if (row < 1 || row > TY - 2 || y >= a.H) continue;
            float3 r;
            if (SHARPEN == 2)
                r = cas_pixel(at(x, y - 1), at(x - 1, y), at(x, y), at(x + 1, y), at(x, y + 1), ctx.k);
            else
                r = simple_sharpen_pixel(at(x - 1, y), at(x + 1, y), at(x, y - 1), at(x, y + 1), at(x, y), ctx.k);
            *at_w<uint2>(ctx.sharp, ctx.sharp_pitch, x, y) = float4_to_half4(make_float4(r.x, r.y, r.z, 1.0f));
        }
    }
};
static_assert(sizeof(float4) * WW * WH >= sizeof(uint2) * TX * TY, "the screen fits over the window");

// Resident CTAs per SM the fused kernel's register budget is sized for (a tuning constant).
#ifndef TAA_FUSED_MIN_BLOCKS
#define TAA_FUSED_MIN_BLOCKS 7
#endif
template <int SHARPEN, int INTERP, int MC>
__global__ void __launch_bounds__(NT, TAA_FUSED_MIN_BLOCKS)
    resolve_strips_sharpen(const Args a, const __grid_constant__ CUtensorMap hmap, const int tma_ok, char* sharp,
                           uint32_t sharp_pitch, float k) {
    __shared__ SmemT<float4> sm;
    uint32_t phase = 0;
    typename FusedF32Pol<SHARPEN>::Ctx ctx{reinterpret_cast<uint2*>(sm.win), sharp, sharp_pitch, k};
    strip_tile<FusedF32Pol<SHARPEN>, INTERP, MC, false, true>(a, &hmap, tma_ok, (int)blockIdx.x * (TX - 2) - 1,
                                                              (int)blockIdx.y * (TY - 2) - 1, sm, phase, ctx);
}


// One view, one CTA per tile; HF 1: RGBA16F history (a.hout_half set).
template <class Pol, int INTERP, int MC, int HF = 0>
__global__ void __launch_bounds__(NT, TAA_FAST_MIN_BLOCKS)
    resolve_strips(const Args a, const __grid_constant__ CUtensorMap hmap, const int tma_ok) {
    __shared__ SmemT<typename Pol::Staged, HF> sm;
    uint32_t phase = 0;
    typename Pol::Ctx ctx;
    strip_tile<Pol, INTERP, MC, false, false, HF>(a, &hmap, tma_ok, blockIdx.x, blockIdx.y, sm, phase, ctx);
}

// One view with a policy that may reproject (its Reproj a kernel parameter).
template <class Pol, int INTERP, int MC, int HF = 0>
__global__ void __launch_bounds__(NT, TAA_FAST_MIN_BLOCKS)
    resolve_strips_reproj(const Args a, const __grid_constant__ CUtensorMap hmap, const int tma_ok,
                          const __grid_constant__ Reproj rp) {
    __shared__ SmemT<typename Pol::Staged, HF> sm;
    uint32_t phase = 0;
    typename Pol::Ctx ctx{&rp};
    strip_tile<Pol, INTERP, MC, false, false, HF>(a, &hmap, tma_ok, blockIdx.x, blockIdx.y, sm, phase, ctx);
}

// Many views in one launch: each CTA takes jobs blockIdx.x, blockIdx.x +
// gridDim.x, ... of the job list (view, tile x, tile y; common.cuh); a view's
// arguments are rebuilt in shared memory when a CTA's job moves to another
// view.  maps[v] is view v's 2-D history map for the 41x25 window, usable
// when tma_ok[v].
// Resident CTAs per SM the batch kernel's register budget is sized for (a
// tuning constant: at 6 the kernel keeps its view arguments and job state in
// registers without spilling; the 48-view batch runs at 0.90 of the single
// 4K view's per-pixel rate, against 0.88 at 8 and 0.78 at 5).
#ifndef TAA_FAST_BATCH_MIN_BLOCKS
#define TAA_FAST_BATCH_MIN_BLOCKS 6
#endif
template <class Pol, int INTERP, int MC>
__global__ void __launch_bounds__(NT, TAA_FAST_BATCH_MIN_BLOCKS)
    resolve_strips_batch(const BatchView* __restrict__ views, const CUtensorMap* __restrict__ maps,
                         const int* __restrict__ tma_ok, const uint32_t* __restrict__ jobs, const int njobs) {
    __shared__ SmemT<typename Pol::Staged> sm;
    __shared__ Args s_args;
    if (threadIdx.x == 0) {
        mbar_init(&sm.bar, 1);
        sm.abort = 0;
    }
    uint32_t phase = 0;
    int cur_view = -1;
    for (int j = blockIdx.x; j < njobs; j += gridDim.x) {
        const uint32_t job = __ldg(jobs + j);
        const int vi = job_view(job);
        if (vi != cur_view) {
            __syncthreads();  // every thread has read the previous view's arguments
            if (threadIdx.x == 0) {
                s_args = make_args(views[vi].U, views[vi].a);
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(maps + vi) : "memory");
            }
            cur_view = vi;
            __syncthreads();
        }
        typename Pol::Ctx ctx;
        strip_tile<Pol, INTERP, MC, true>(s_args, maps + vi, __ldg(tma_ok + vi), job_tile_x(job), job_tile_y(job),
                                          sm, phase, ctx);
        __syncthreads();  // the next tile reuses the shared memory
        if (sm.abort) return;
    }
}

}  // namespace fast32
}  // namespace taa_dev
