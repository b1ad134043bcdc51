// tiled_skeleton.cuh - the CTA structure shared by the tiled FP32 and FP16 resolve forms.
//
// One 256-thread CTA resolves a 32x8 tile, one pixel per thread:
//   1. each thread requests its pixel's velocity and depth and one or two
//      texels of the tile's source colour plus 1-pixel halo; warp 0 alone
//      reads the velocity of the tile's reference pixel and places the
//      history window: the reference pixel's Catmull-Rom taps widened by the
//      tile and a margin of WIN_MARGIN pixels of motion difference;
//   2. a window that lies inside the history image is copied into shared
//      memory by one TMA tensor copy (cp.async.bulk.tensor) that thread 0
//      issues on an mbarrier; a window that crosses the image border is
//      copied by all threads with cp.async, edge-clamping each texel.  Either
//      way the window is indexed by unclamped texel coordinates, so a
//      pixel's 16 taps are 4x4 consecutive entries read from one base;
//   3. while the window is in flight the staged colour gives the 3x3 box
//      (the arithmetic policy decides how: exact FP32 or packed FP16);
//   4. a pixel whose taps fall inside the window reads them from shared
//      memory, any other pixel (motion differing from the reference pixel's
//      by more than the margin) reads them from global memory with clamped
//      coordinates; then rejection, rectification and blend finish the pixel.
//
// The wait for the TMA copy polls its mbarrier a bounded number of times; a
// copy that has not landed by then sets kStatusWindowTimeout in the device
// status word, and the CTA waits a second bounded while for the copy before
// it leaves.
//
// The arithmetic lives in a policy class `Pol` so that the exact FP32 form
// (compiled with -fmad=false, bit-identical to the oracle) and the FP16 form
// share the memory pipeline.
#pragma once
#include <cuda.h>

#include <cstring>
#include <type_traits>

#include "../../include/taa_gb300.h"
#include "common.cuh"
#include "f32x2.cuh"
#include "kernels.h"
#include "segmentation.cuh"

namespace taa_dev {
namespace tiled {

// resident threads per SM the register budget of a tile kernel is sized for
// (a tuning constant: 6 CTAs of 256 threads)
#ifndef TAA_TILE_MIN_BLOCKS
#define TAA_TILE_MIN_BLOCKS 6
#endif
constexpr int WIN_MARGIN = 3;  // motion difference (px) the history window absorbs

// A tile shape: TX x TY pixels, one per thread, staged with a 1-pixel halo;
// its history window spans the reference pixel's Catmull-Rom taps widened by
// the tile and WIN_MARGIN on each side.
template <int TX_, int TY_> struct Shape {
    static constexpr int TX = TX_, TY = TY_, NT = TX * TY, NPX = 1;
    static constexpr bool kMulti = false;  // one pixel per thread (tile_body)
    static constexpr int SX = TX + 2, SY = TY + 2, NS = SX * SY;
    static constexpr int WW = TX + 3 + 2 * WIN_MARGIN;
    static constexpr int WH = TY + 3 + 2 * WIN_MARGIN;
    static constexpr int MIN_BLOCKS =
        TAA_TILE_MIN_BLOCKS * 256 / NT < 1 ? 1 : (TAA_TILE_MIN_BLOCKS * 256 / NT > 32 ? 32 : TAA_TILE_MIN_BLOCKS * 256 / NT);
    static_assert(NT % 32 == 0 && NT <= 1024, "whole warps");
    static_assert(NS <= 2 * NT, "each thread stages at most two colour texels");
};
using DefaultShape = Shape<32, 8>;

// Stored window width: RGBA16F windows start on an even texel (a TMA copy of
// half texels starts on a 16-byte boundary), so their width is even.
template <class S, int HF> struct Win {
    static constexpr int W = HF == 0 ? S::WW : S::WW + (S::WW & 1);
    static constexpr int ALIGN = HF == 0 ? 1 : 2;
};
// Polls of the window's mbarrier before the wait gives up, each suspending the
// thread in hardware until the phase completes or kWaitPollNs pass (so a
// waiting warp issues a few instructions, not a spin loop): about 80 ms in
// all, far above any real copy time.  The first wait of a tile reads its
// limit from the word after the device status word (kWaitPolls unless a test
// lowers it); the second, which drains a copy that the first gave up on,
// always polls kWaitPolls times.
constexpr uint32_t kWaitPolls = TAA_WINDOW_WAIT_POLLS;
constexpr uint32_t kWaitPollNs = 20000;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst_smem, const void* src) {
    if (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst_smem)), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(smem_addr(dst_smem)), "l"(src), "n"(BYTES)
                     : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// mbarrier and TMA tensor copies (PTX ISA: mbarrier, cp.async.bulk.tensor).
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // the barrier's initialisation becomes visible to the TMA unit (async proxy)
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity), "r"(kWaitPollNs)
        : "memory");
    return done != 0;
}
// Bounded wait for phase `parity` of the barrier: false after `polls` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t polls = kWaitPolls) {
    for (uint32_t i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// The first window wait's poll limit (the word after the status word).
__device__ __forceinline__ uint32_t first_wait_polls(const unsigned int* status) { return __ldcg(status + 1); }
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];\n" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_addr(bar))
        : "memory");
}

// Compile-time view of the parameter block: Hot = the benchmark mode (variance
// clip in YCoCg, clip towards the box centre, velocity for every pixel, simple
// velocity sampling, no tonemap / luma weighting / near-clamp reduction).
template <bool Hot> struct Mode {
    const taa_parameters_t& P;
    __device__ bool ycocg() const { return Hot || P.mUseYCoCg; }
    __device__ bool tonemap() const { return !Hot && P.mToneMapLumaKaris; }
    __device__ bool variance() const { return Hot || P.mVarianceClipping; }
    __device__ bool shaped() const { return !Hot && P.mShapedNeighbourhood; }
    __device__ bool shrink() const { return !Hot && P.mUseYCoCg && P.mShrinkChromaAxis; }
    __device__ int clip() const { return Hot ? 2 : P.mColorClampingOrClipping; }
    __device__ int use_velocity() const { return Hot ? 2 : P.mUseVelocityVectors; }
    __device__ int velocity_sample() const { return Hot ? 0 : P.mVelocitySampleMode; }
    __device__ bool vel_alpha() const { return !Hot && P.mVelBasedAlpha; }
    __device__ bool lottes() const { return !Hot && P.mLumaWeightingLottes; }
    __device__ bool near_clamp() const { return !Hot && P.mReduceBlendNearClamp; }
    __device__ bool noise() const { return !Hot && P.mAddNoise; }
    __device__ bool anti_ghost() const { return !Hot && P.mDynamicAntiGhosting; }
};

inline bool is_hot(const taa_parameters_t& P) {
    return P.mUseYCoCg && !P.mToneMapLumaKaris && P.mVarianceClipping && !P.mShrinkChromaAxis && !P.mRayTraceAugment &&
           P.mColorClampingOrClipping == 2 && P.mUseVelocityVectors == 2 && P.mVelocitySampleMode == 0 &&
           !P.mVelBasedAlpha && !P.mLumaWeightingLottes && !P.mReduceBlendNearClamp && !P.mAddNoise &&
           !P.mDynamicAntiGhosting;
}

struct C3 { float x, y, z; };

// What a policy's finish records for the debug outputs: the rectification's
// move (clipped minus unclipped history) and the blend weight.
struct FinishOut {
    float3 rdiff;
    float alpha;
};

// History filter taps: up to 16 texels (clamped coordinates) with weights.
// INTERP 2: 4x4 separable Catmull-Rom; 0: one bilinear 2x2; 1: four bilinear
// 2x2 sets combined with the "b-spline" weights.
struct Taps {
    float wx[4], wy[4];
    int ux, uy;  // unclamped coordinate of the first tap
    // clamped coordinate of tap i (global reads only; the window holds clamped texels)
    __device__ __forceinline__ int xs(int i, int w) const { return clampi(ux + i, 0, w - 1); }
    __device__ __forceinline__ int ys(int j, int h) const { return clampi(uy + j, 0, h - 1); }
};

template <class Pol, int INTERP> struct HistoryTaps {
    Taps t[INTERP == 1 ? 4 : 1];
    float s0[2], s1[2];  // b-spline combination weights

    __device__ __forceinline__ void setup(float u, float v, int w, int h, f2 z) {
        if (INTERP == 2) {
            Pol::catmullrom_taps(u, v, w, h, t[0], z);
        } else if (INTERP == 0) {
            Pol::bilinear_taps(u, v, w, h, t[0]);
        } else {
            float t0[2], t1[2];
            Pol::bspline_positions(u, v, w, h, s0, s1, t0, t1);
            Pol::bilinear_taps(t0[0], t0[1], w, h, t[0]);
            Pol::bilinear_taps(t1[0], t0[1], w, h, t[1]);
            Pol::bilinear_taps(t0[0], t1[1], w, h, t[2]);
            Pol::bilinear_taps(t1[0], t1[1], w, h, t[3]);
        }
    }
};

template <int HF> struct HistTexel;
template <> struct HistTexel<0> { using T = float4; static constexpr int B = 16; };
template <> struct HistTexel<1> { using T = uint2; static constexpr int B = 8; };

template <int HF> __device__ __forceinline__ float4 to_f4(float4 v) { return v; }
template <int HF> __device__ __forceinline__ float4 to_f4(uint2 v) { return half4_to_float4(v); }

// History position of pixel (cx, cy) (taa.comp:391-438).
template <class Pol, int MC, bool HOT>
__device__ __forceinline__ void history_position(const taa_uniforms_t& U, const FrameArgs& a, const Mode<HOT>& M,
                                                 int cx, int cy, float4 vs, float depth, float u, float v, float& hu,
                                                 float& hv, float& ehd) {
    const bool can = !(M.use_velocity() == 0 || (M.use_velocity() == 1 && vs.w < 0.5f));
    if (can) {
        if (M.velocity_sample() == 1) {
            // 3x3 "longest": the reference keeps the last of its eight taps,
            // (+1, +1), whatever their lengths (taa.comp:398-412)
            const float4 s = fetch_velocity<MC>(a.velocity, cx + 1, cy + 1);
            vs.x = s.x;
            vs.y = s.y;
        } else if (M.velocity_sample() == 2) {
            int bdx = -1, bdy = -1;
            float dc = fetch_r32f(a.depth, cx - 1, cy - 1);
#pragma unroll
            for (int k = 1; k < 9; ++k) {
                int dx = k % 3 - 1, dy = k / 3 - 1;
                float d = fetch_r32f(a.depth, cx + dx, cy + dy);
                if (d < dc) { bdx = dx; bdy = dy; dc = d; }
            }
            vs = fetch_velocity<MC>(a.velocity, cx + bdx, cy + bdy);
        }
        hu = u - vs.x;
        hv = v - vs.y;
        ehd = depth - vs.z;
    } else {
        Pol::reproject(U, u, v, depth, hu, hv, ehd);
    }
}

// taa.comp:796-811, dynamic anti-ghosting: a pixel with no moving object in
// its cross whose history was written under one (history alpha > 0) is
// rejected; its own "moving" bit becomes the history alpha it writes.
template <int MC>
__device__ __forceinline__ void anti_ghosting(const FrameArgs& a, int cx, int cy, float hist_alpha, bool& rejected,
                                              float& dyn) {
    const float eps = 1e-5f;
    auto mov = [&](int dx, int dy) {
        const float4 v = fetch_velocity<MC>(a.velocity, cx + dx, cy + dy);
        return (fabsf(v.x) > eps || fabsf(v.y) > eps) && (fabsf(v.w) >= 0.5f);
    };
    const bool mL = mov(-1, 0), mR = mov(1, 0), mT = mov(0, -1), mB = mov(0, 1), mC = mov(0, 0);
    if (!(mL || mR || mT || mB || mC) && hist_alpha > 0.0f) rejected = true;
    dyn = mC ? 1.0f : 0.0f;
}

// Shared memory of one tile.
template <class Pol, class S, int HF> struct TileSmem {
    typename Pol::Staged col[S::NS];
    alignas(128) typename HistTexel<HF>::T win[Win<S, HF>::W * S::WH];
    uint64_t bar;  // completion of the window's TMA copy
    int org[3];    // window origin x, y and how it is copied (1 TMA, 2 cp.async)
    int abort;     // a persistent CTA stops after this tile (a window wait gave up)
};

// One thread's inputs of a tile, as loaded (converted where they are used, so
// that a load issued ahead of time does not stall the thread until then):
// its pixel's depth and velocity and one or two staged colour texels.
template <int MC> struct TileIn {
    float depth;
    typename std::conditional<MC == 4, uint2, uint32_t>::type vel;
    uint2 st0, st1;
};
template <int MC> __device__ __forceinline__ float4 velocity_of(uint32_t v) {
    const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&v));
    return make_float4(f.x, f.y, 0.f, 0.f);
}
template <int MC> __device__ __forceinline__ float4 velocity_of(uint2 v) { return half4_to_float4(v); }

template <class S, int MC>
__device__ __forceinline__ TileIn<MC> load_tile_inputs(const FrameArgs& a, int tile_x, int tile_y) {
    constexpr int TX = S::TX, NT = S::NT, SX = S::SX, NS = S::NS;
    const int tid = threadIdx.x;
    const int W = a.out_w, H = a.out_h;
    const int x0 = tile_x * TX, y0 = tile_y * S::TY;
    const int cx = min(x0 + tid % TX, W - 1), cy = min(y0 + tid / TX, H - 1);
    TileIn<MC> in;
    in.depth = __ldg(texel_ptr<float>(a.depth, cx, cy));
    in.vel = __ldg(texel_ptr<decltype(in.vel)>(a.velocity, cx, cy));
    const int sy = tid / SX, sx = tid - sy * SX;
    in.st0 = __ldg(texel_ptr<uint2>(a.color, clampi(x0 - 1 + sx, 0, W - 1), clampi(y0 - 1 + sy, 0, H - 1)));
    in.st1 = make_uint2(0u, 0u);
    if (tid + NT < NS) {
        const int i = tid + NT, sy1 = i / SX, sx1 = i - sy1 * SX;
        in.st1 = __ldg(texel_ptr<uint2>(a.color, clampi(x0 - 1 + sx1, 0, W - 1), clampi(y0 - 1 + sy1, 0, H - 1)));
    }
    return in;
}

// The tile's reference pixel: its centre, clamped into the image.
template <class S> __device__ __forceinline__ void reference_pixel(const FrameArgs& a, int tile_x, int tile_y, int& rx,
                                                                   int& ry) {
    rx = min(tile_x * S::TX + S::TX / 2, a.out_w - 1);
    ry = min(tile_y * S::TY + S::TY / 2, a.out_h - 1);
}

// The history window of a tile, placed at its reference pixel (depth rdepth,
// velocity rvs): the pixel's Catmull-Rom taps widened by the tile and
// WIN_MARGIN.  The calling thread writes the origin and copy mode to org[0..2]
// and, for a window inside the image with TMA usable, starts its copy into
// `win` on `bar`.  Run by one thread, or by a warp whose lane 0 writes.
template <class Pol, class S, int HF, int MC, int INTERP, bool HOT>
__device__ __forceinline__ void place_window(const taa_uniforms_t& U, const FrameArgs& a, const Mode<HOT>& M,
                                             const CUtensorMap* hmap, bool tma_ok, int tile_x, int tile_y,
                                             float rdepth, float4 rvs, typename HistTexel<HF>::T* win, uint64_t* bar,
                                             int* org, bool writer) {
    constexpr int WWS = Win<S, HF>::W, WH = S::WH;
    const Img& hi = a.history;
    int rx, ry;
    reference_pixel<S>(a, tile_x, tile_y, rx, ry);
    const int x0 = tile_x * S::TX, y0 = tile_y * S::TY;
    float ru = div_const_rn((float)rx + 0.5f, (float)a.out_w, a.inv_out_w);
    float rv = div_const_rn((float)ry + 0.5f, (float)a.out_h, a.inv_out_h);
    float rhu, rhv, rehd;
    history_position<Pol, MC, HOT>(U, a, M, rx, ry, rvs, rdepth, ru, rv, rhu, rhv, rehd);
    const int k0 = INTERP == 2 ? 1 : 0;  // Catmull-Rom starts one texel before floor(p - 0.5)
    const int rux = trunc_index(floorf(rhu * (float)hi.w - 0.5f)) - k0;
    const int ruy = trunc_index(floorf(rhv * (float)hi.h - 0.5f)) - k0;
    // the reference pixel sits at (rx - x0, ry - y0) in the tile; floor to the stored alignment
    const int wx0 = (rux - (rx - x0) - WIN_MARGIN) & ~(Win<S, HF>::ALIGN - 1);
    const int wy0 = ruy - (ry - y0) - WIN_MARGIN;
    const bool interior = wx0 >= 0 && wy0 >= 0 && wx0 <= hi.w - WWS && wy0 <= hi.h - WH;
    const int mode = tma_ok && interior ? 1 : 2;
    if (writer) {
        org[0] = wx0;
        org[1] = wy0;
        org[2] = mode;
        if (mode == 1) {
            mbar_expect_tx(bar, (uint32_t)(sizeof(typename HistTexel<HF>::T) * WWS * WH));
            if (HF == 0) tma_load_3d(win, hmap, 0, wx0, wy0, bar);
            else tma_load_2d(win, hmap, 4 * wx0, wy0, bar);
        }
    }
}

// The tile after its inputs are loaded and its window placed: history
// position, staging of the colour, the 3x3 box while the window is in flight,
// the history sample (from the window when all taps fall inside it, from
// global memory otherwise), then the finisher.  Every thread of the CTA
// calls it.  `col`, `win`, `bar`, `org` are the tile's shared buffers; `phase`
// is the barrier phase the window copy completes; prev_depth_in, when not
// null, is this thread's previous-frame depth at its history position,
// fetched ahead (depth culling); `abort` (persistent CTAs) is set when a
// window wait gave up.
// The anti-ghosting mask reaches the finishers that store a history alpha.
template <class Fin> __device__ __forceinline__ void set_dynamic_mask(Fin&, float) {}
struct StoreFinish;
__device__ __forceinline__ void set_dynamic_mask(StoreFinish& fin, float dyn);

// The barrier among the threads that compute a tile (the whole CTA).
struct CtaSync {
    static __device__ __forceinline__ void sync() { __syncthreads(); }
};

template <class Pol, class S, int HF, int MC, int INTERP, bool HOT, class Sync = CtaSync, class Fin>
__device__ __forceinline__ void tile_compute(const taa_uniforms_t& U, const FrameArgs& a, int tile_x, int tile_y,
                                             const TileIn<MC>& in, const float* prev_depth_in,
                                             typename Pol::Staged* col, typename HistTexel<HF>::T* win,
                                             uint64_t* bar, const int* org, uint32_t phase, int* abort, Fin& fin) {
    using HT = typename HistTexel<HF>::T;
    constexpr int TX = S::TX, NT = S::NT, SX = S::SX, NS = S::NS, WH = S::WH;
    constexpr int WWS = Win<S, HF>::W;

    const taa_parameters_t& P = U.param[0];
    const Mode<HOT> M{P};
    const int tid = threadIdx.x;
    const int lx = tid % TX, ly = tid / TX;
    const int W = a.out_w, H = a.out_h;
    const int x = tile_x * TX + lx, y = tile_y * S::TY + ly;
    const bool inside = x < W && y < H;
    const int cx = min(x, W - 1), cy = min(y, H - 1);
    const Img& hi = a.history;
    const bool have_hist = hi.p != nullptr;
    const bool windowed = have_hist && INTERP != 1;

    // own history position; (u, v) = (texel + 0.5) / size, correctly rounded, as a pair
    const f2 z{a.neg_zero2};
    const f2 uv = div_const_rn2(add2(pk((float)cx, (float)cy), dup(0.5f)), pk(-(float)W, -(float)H),
                                pk(a.inv_out_w, a.inv_out_h), z);
    float u = f2lo(uv), v = f2hi(uv);
    float hu, hv, ehd;
    history_position<Pol, MC, HOT>(U, a, M, cx, cy, velocity_of<MC>(in.vel), in.depth, u, v, hu, hv, ehd);
    float prev_depth = 0.f;
    const bool depth_cull = P.mDepthCulling != 0;
    if (depth_cull && a.history_depth.p) {
        if (prev_depth_in) {
            prev_depth = *prev_depth_in;
        } else {
            int tx_ = clampi(trunc_index(hu * (float)a.color.w), 0, a.color.w - 1);
            int ty_ = clampi(trunc_index(hv * (float)a.color.h), 0, a.color.h - 1);
            prev_depth = __ldg(texel_ptr<float>(a.history_depth, tx_, ty_));
        }
    }

    // staged colour in the policy's working format
    const bool tm = M.tonemap(), yc = M.ycocg();
    col[tid] = Pol::stage(in.st0, tm, yc);
    if (tid + NT < NS) col[tid + NT] = Pol::stage(in.st1, tm, yc);
    Sync::sync();
    int wx0 = 0, wy0 = 0, mode = 0;
    if (windowed) {
        wx0 = org[0];
        wy0 = org[1];
        mode = org[2];
    }
    if (mode == 2) {
        // a window across the image border: every texel edge-clamped
        const int lane = tid & 31, warp = tid >> 5;
        for (int r = warp; r < WH; r += NT / 32) {
            const int gy = clampi(wy0 + r, 0, hi.h - 1);
            const char* row = hi.p + (size_t)gy * hi.pitch;
            for (int c = lane; c < WWS; c += 32)
                cp_async<HistTexel<HF>::B>(&win[r * WWS + c],
                                           row + (size_t)clampi(wx0 + c, 0, hi.w - 1) * HistTexel<HF>::B);
        }
        cp_async_commit();
    }
    // the 3x3 box while the window is in flight
    typename Pol::Box box;
    Pol::template box<HOT>(&col[(ly + 1) * SX + lx + 1], SX, M, P.mVarClipGamma, box, z);
    if (Pol::kExactCentre) Pol::centre_colour(box, a.color, cx, cy, tm, yc);

    bool landed = true;
    if (mode == 1) {
        landed = mbar_wait_bounded(bar, phase & 1u, first_wait_polls(a.status));
        if (!landed) {
            atomicOr(a.status, kStatusWindowTimeout);
            mbar_wait_bounded(bar, phase & 1u);  // the copy may still land in this CTA's memory
            if (abort) *abort = 1;
        }
    } else if (mode == 2) {
        cp_async_wait_all();
        Sync::sync();
    }
    const bool valid = inside && landed;
    // rejection (taa.comp:787-823) first, so its inputs die before the filter
    bool rejected = false;
    if (P.mRejectOutside && (hu < 0.f || hv < 0.f || hu >= 1.f || hv >= 1.f)) rejected = true;
    if (depth_cull) {
        float hd = prev_depth;
        if (fabsf(hd - ehd) > 0.1f * (1.0f - hd)) rejected = true;
    }
    // the history sample: from the window when all taps fall inside it
    float4 hraw = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
        if (have_hist) {
            HistoryTaps<Pol, INTERP> taps;
            taps.setup(hu, hv, hi.w, hi.h, z);
            const int span = INTERP == 2 ? 4 : 2;
            const int bx = taps.t[0].ux - wx0, by = taps.t[0].uy - wy0;
            const bool in_win = windowed && bx >= 0 && by >= 0 && bx + span <= WWS && by + span <= WH;
            if (in_win) {
                const HT* base = &win[by * WWS + bx];
                hraw = Pol::template filter_window<INTERP, HF, !HOT>(taps, base, WWS);
            } else {
                hraw = Pol::template filter<INTERP, !HOT>(
                    taps, hi.w, hi.h, [&](int tx_, int ty_) { return fetch_history<HF>(hi, tx_, ty_); });
            }
        }
    }
    if (M.anti_ghost()) {
        float dyn = 0.f;
        anti_ghosting<MC>(a, cx, cy, hraw.w, rejected, dyn);
        set_dynamic_mask(fin, dyn);
    }
    // rectification, blend and stores: every thread of the CTA calls the
    // finisher (valid says whether its pixel is in the image and resolved)
    const C3 c0 = Pol::centre(box, &col[(ly + 1) * SX + lx + 1]);
    Fin::template run<Pol, HF, HOT>(U, a, P, M, box, c0, hraw, u, v, hu, hv, ehd, prev_depth, rejected, valid, x, y,
                                    tm, fin);
}

// One tile of the resolve: pixels (tile_x * TX + i, tile_y * TY + j).  Pol
// provides the working colour format and the box, tap, filter and finishing
// arithmetic (policy_f32.cuh, resolve_half.cu).  `hmap` is the history image's
// tensor map (box Win::W x WH texels) when `tma_ok`; otherwise every window is
// copied with cp.async.  `sm.bar` is initialised by the caller; `phase` is the
// barrier phase the next TMA copy completes.  A wait that gives up sets the
// status bit and leaves the tile's pixels unwritten; in a persistent loop
// (PERSIST) it also sets sm.abort, which the caller reads after the barrier
// that separates tiles, so the whole CTA stops together.
template <class Pol, class S, int HF, int MC, int INTERP, bool HOT, bool PERSIST, class Fin>
__device__ __forceinline__ void tile_body(const taa_uniforms_t& U, const FrameArgs& a, const CUtensorMap* hmap,
                                          bool tma_ok, int tile_x, int tile_y, TileSmem<Pol, S, HF>& sm,
                                          uint32_t& phase, Fin& fin) {
    const TileIn<MC> in = load_tile_inputs<S, MC>(a, tile_x, tile_y);
    const bool windowed = a.history.p != nullptr && INTERP != 1;
    if (windowed && threadIdx.x < 32) {
        // warp 0 places the window at the tile's reference pixel; thread 0 starts the copy
        int rx, ry;
        reference_pixel<S>(a, tile_x, tile_y, rx, ry);
        const float rdepth = __ldg(texel_ptr<float>(a.depth, rx, ry));
        const float4 rvs = fetch_velocity<MC>(a.velocity, rx, ry);
        place_window<Pol, S, HF, MC, INTERP, HOT>(U, a, Mode<HOT>{U.param[0]}, hmap, tma_ok, tile_x, tile_y, rdepth,
                                                  rvs, sm.win, &sm.bar, sm.org, threadIdx.x == 0);
    }
    tile_compute<Pol, S, HF, MC, INTERP, HOT>(U, a, tile_x, tile_y, in, nullptr, sm.col, sm.win, &sm.bar, sm.org,
                                              phase, PERSIST ? &sm.abort : nullptr, fin);
    if (windowed && sm.org[2] == 1) phase ^= 1u;
}

// The finisher of the plain tiled forms: the policy's rectification and
// blend (taa.comp:825-900), then the history and screen stores; `dyn` is the
// history alpha it writes (the anti-ghosting mask, else 0).
struct StoreFinish {
    float dyn = 0.f;
    uint32_t seg = 0;                            // the ray-trace-assist class (debug mode 8)
    float4 dvel = make_float4(0.f, 0.f, 0.f, 0.f);  // the pixel's velocity (debug mode 4)
    template <class Pol, int HF, bool HOT>
    static __device__ __forceinline__ void run(const taa_uniforms_t& U, const FrameArgs& a, const taa_parameters_t& P,
                                               const Mode<HOT>& M, const typename Pol::Box& box, const C3& c0,
                                               float4 hraw, float u, float v, float hu, float hv, float, float,
                                               bool rejected, bool valid, int x, int y, bool tm, StoreFinish& fin) {
        if (!valid) return;
        float4 o;
        constexpr bool kDebug = Pol::kDebug && !HOT;
        FinishOut fo;
        if constexpr (Pol::kExactFallback) {
            // a policy whose clip can be ill-conditioned for its precision finishes
            // such a pixel from the source texels in FP32
            const typename Pol::At at{&a, x, y, tm};
            o = Pol::template finish_at<HOT>(U, P, M, box, c0, hraw, u, v, hu, hv, rejected, &at);
        } else if constexpr (kDebug) {
            o = Pol::template finish<HOT>(U, P, M, box, c0, hraw, u, v, hu, hv, rejected, 1.0f,
                                          a.debug.p ? &fo : nullptr);
        } else {
            o = Pol::template finish<HOT>(U, P, M, box, c0, hraw, u, v, hu, hv, rejected);
        }
        const float4 to_hist = make_float4(o.x, o.y, o.z, fin.dyn);
        store_history<HF>(a.history_out, x, y, to_hist);
        if (tm) o = Pol::un_tonemap(o);
        const float4 to_screen = make_float4(o.x, o.y, o.z, 1.0f);
        if (a.result.p) store_rgba16f(a.result, x, y, to_screen);
        if constexpr (kDebug) {
            if (a.debug.p) {
                DebugIn d;
                Pol::box_bounds(box, d.mn, d.mx);
                d.rdiff = fo.rdiff;
                d.rejected = rejected;
                d.alpha = fo.alpha;
                const float du = u - hu, dv = v - hv;
                d.speed = sqrtf(du * du + dv * dv);
                d.vel = fin.dvel;
                d.to_screen = to_screen;
                d.to_hist = to_hist;
                d.seg = fin.seg;
                store_rgba16f(a.debug, x, y, debug_value(P, d));
            }
        }
    }
};

__device__ __forceinline__ void set_dynamic_mask(StoreFinish& fin, float dyn) { fin.dyn = dyn; }

// A tile of TX x (TYT * NPX) pixels resolved by TX x TYT threads, each taking
// NPX vertically adjacent pixels (rows NPX * ly ... NPX * ly + NPX - 1); staged
// with a 1-pixel halo, its history window spans the reference pixel's
// Catmull-Rom taps widened by the tile and WIN_MARGIN on each side.
#ifndef TAA_MULTI_MIN_BLOCKS
#define TAA_MULTI_MIN_BLOCKS 4  // resident 256-thread CTAs per SM (64 registers)
#endif
template <int TX_, int TYT_, int NPX_> struct MultiShape {
    static constexpr int TX = TX_, TYT = TYT_, NPX = NPX_, TY = TYT * NPX, NT = TX * TYT;
    static constexpr bool kMulti = true;  // NPX pixels per thread (multi_body)
    static constexpr int SX = TX + 2, SY = TY + 2, NS = SX * SY;
    static constexpr int NSPT = (NS + NT - 1) / NT;  // staged texels per thread
    static constexpr int WW = TX + 3 + 2 * WIN_MARGIN;
    static constexpr int WH = TY + 3 + 2 * WIN_MARGIN;
    static_assert(NT % 32 == 0 && NT <= 1024, "whole warps");
};

// The neighbourhood the ray-trace-assist classification reads, staged for a
// tile and its 1-pixel halo: material ids, view-space depth, normals and luma
// (each computed once per texel instead of once per tap).
template <class S, bool RT> struct SegStage {
    uint32_t mat[S::NS];
    float ldep[S::NS];
    seg::N3 nrm[S::NS];
    float lum[S::NS];
};
template <class S> struct SegStage<S, false> {};

// segmentation.cuh's accessor over a staged tile whose first staged texel is
// the image texel (x0 - 1, y0 - 1); coordinates come edge-clamped.
template <class S> struct StagedSeg {
    const SegStage<S, true>& st;
    const FrameArgs& a;
    int x0, y0;
    __device__ int at(int x, int y) const { return (y - y0 + 1) * S::SX + (x - x0 + 1); }
    __device__ uint32_t material(int x, int y) const { return st.mat[at(x, y)]; }
    __device__ seg::N3 normal(int x, int y) const { return st.nrm[at(x, y)]; }
    __device__ float lin_depth(int x, int y) const { return st.ldep[at(x, y)]; }
    __device__ float luma(int x, int y) const { return st.lum[at(x, y)]; }
    __device__ uint32_t prev_material(int x, int y) const { return fetch_r32u(a.prev_material, x, y); }
    __device__ uint32_t prev_segmask(int x, int y) const { return fetch_r32u(a.prev_segmask, x, y); }
};

// One multi-pixel tile: the steps of tile_compute with each thread's NPX
// pixels interleaved.  Shared per thread: its index arithmetic, the parameter
// reads, the staging share, the window origin and the wait; per pixel: depth,
// velocity and history position, the previous-frame depth, the 3x3 box, the
// history sample and the finisher (the same arithmetic as the one-pixel
// kernels, so the same bits).  RT adds the ray-trace-assist classification
// (segmentation.cuh) on a staged neighbourhood: a pixel it marks is rejected,
// and the mask is stored when bound.  `sm.bar` is initialised by the caller;
// `phase` is the barrier phase the next TMA copy completes.  A wait that gives
// up sets the status bit and leaves the tile's pixels unwritten; in a
// persistent loop (PERSIST) it also sets sm.abort, which the caller reads
// after the barrier that separates tiles.
template <class Pol, class S, int HF, int MC, int INTERP, bool HOT, bool RT, bool PERSIST>
__device__ __forceinline__ void multi_body(const taa_uniforms_t& U, const FrameArgs& a, const CUtensorMap* hmap,
                                           bool tma_ok, int tile_x, int tile_y, TileSmem<Pol, S, HF>& sm,
                                           SegStage<S, RT>& ss, uint32_t& phase) {
    using RawVel = typename std::conditional<MC == 4, uint2, uint32_t>::type;
    constexpr int TX = S::TX, NT = S::NT, NPX = S::NPX, SX = S::SX, NS = S::NS, WH = S::WH;
    constexpr int WWS = Win<S, HF>::W;
    const int tid = threadIdx.x;
    const taa_parameters_t& P = U.param[0];
    const Mode<HOT> M{P};
    const int lx = tid % TX, ly = tid / TX;
    const int W = a.out_w, H = a.out_h;
    const int x0 = tile_x * TX, y0 = tile_y * S::TY;
    const int x = x0 + lx, cx = min(x, W - 1);
    // 1. loads: the pixels' depth and velocity, this thread's staged colour texels
    float depth[NPX];
    RawVel vel[NPX];
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        const int cy = min(y0 + NPX * ly + k, H - 1);
        depth[k] = __ldg(texel_ptr<float>(a.depth, cx, cy));
        vel[k] = __ldg(texel_ptr<RawVel>(a.velocity, cx, cy));
    }
    uint2 st[S::NSPT];
#pragma unroll
    for (int j = 0; j < S::NSPT; ++j) {
        const int i = tid + j * NT;
        st[j] = make_uint2(0u, 0u);
        if (i < NS) {
            const int sy = i / SX, sx = i - sy * SX;
            st[j] = __ldg(texel_ptr<uint2>(a.color, clampi(x0 - 1 + sx, 0, W - 1), clampi(y0 - 1 + sy, 0, H - 1)));
        }
    }
    // 2. warp 0 places the history window; thread 0 starts the copy
    const Img& hi = a.history;
    const bool have_hist = hi.p != nullptr;
    const bool windowed = have_hist && INTERP != 1;
    if (windowed && tid < 32) {
        int rx, ry;
        reference_pixel<S>(a, tile_x, tile_y, rx, ry);
        const float rdepth = __ldg(texel_ptr<float>(a.depth, rx, ry));
        const float4 rvs = fetch_velocity<MC>(a.velocity, rx, ry);
        place_window<Pol, S, HF, MC, INTERP, HOT>(U, a, M, hmap, tma_ok, tile_x, tile_y, rdepth, rvs, sm.win,
                                                  &sm.bar, sm.org, tid == 0);
    }
    // 3. the pixels' history positions and previous-frame depths
    const f2 z{a.neg_zero2};
    const bool depth_cull = P.mDepthCulling != 0;
    float u[NPX], v[NPX], hu[NPX], hv[NPX], ehd[NPX], prev_depth[NPX];
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        const int cy = min(y0 + NPX * ly + k, H - 1);
        const f2 uv = div_const_rn2(add2(pk((float)cx, (float)cy), dup(0.5f)), pk(-(float)W, -(float)H),
                                    pk(a.inv_out_w, a.inv_out_h), z);
        u[k] = f2lo(uv);
        v[k] = f2hi(uv);
        history_position<Pol, MC, HOT>(U, a, M, cx, cy, velocity_of<MC>(vel[k]), depth[k], u[k], v[k], hu[k], hv[k],
                                       ehd[k]);
        prev_depth[k] = 0.f;
        if (depth_cull && a.history_depth.p) {
            int tx_ = clampi(trunc_index(hu[k] * (float)a.color.w), 0, a.color.w - 1);
            int ty_ = clampi(trunc_index(hv[k] * (float)a.color.h), 0, a.color.h - 1);
            prev_depth[k] = __ldg(texel_ptr<float>(a.history_depth, tx_, ty_));
        }
    }
    // 4. staged colour in the policy's working format (and the classification's neighbourhood)
    const bool tm = M.tonemap(), yc = M.ycocg();
#pragma unroll
    for (int j = 0; j < S::NSPT; ++j)
        if (tid + j * NT < NS) sm.col[tid + j * NT] = Pol::stage(st[j], tm, yc);
    if constexpr (RT) {
        const uint32_t fl = P.mRayTraceAugmentFlags;
#pragma unroll
        for (int j = 0; j < S::NSPT; ++j) {
            const int i = tid + j * NT;
            if (i >= NS) continue;
            const int sy = i / SX, sx = i - sy * SX;
            const int gx = clampi(x0 - 1 + sx, 0, W - 1), gy = clampi(y0 - 1 + sy, 0, H - 1);
            if (fl & (TAA_RTFLAG_MID | TAA_RTFLAG_DIS)) ss.mat[i] = fetch_r32u(a.material, gx, gy);
            if (fl & TAA_RTFLAG_DPT)
                ss.ldep[i] = seg::lin_depth(fetch_r32f(a.depth, gx, gy), U.mCamNearPlane, U.mCamFarPlane);
            if (fl & TAA_RTFLAG_NRM) {
                const float4 un = fetch_rgba32f(a.uvnrm, gx, gy);
                ss.nrm[i] = seg::normal_from(un.z, un.w);
            }
            if (fl & TAA_RTFLAG_LUM) {
                const float4 c = half4_to_float4(st[j]);
                ss.lum[i] = seg::luma(c.x, c.y, c.z);
            }
        }
    }
    __syncthreads();
    int wx0 = 0, wy0 = 0, mode = 0;
    if (windowed) {
        wx0 = sm.org[0];
        wy0 = sm.org[1];
        mode = sm.org[2];
    }
    if (mode == 2) {
        const int lane = tid & 31, warp = tid >> 5;
        for (int r = warp; r < WH; r += NT / 32) {
            const int gy = clampi(wy0 + r, 0, hi.h - 1);
            const char* row = hi.p + (size_t)gy * hi.pitch;
            for (int c = lane; c < WWS; c += 32)
                cp_async<HistTexel<HF>::B>(&sm.win[r * WWS + c],
                                           row + (size_t)clampi(wx0 + c, 0, hi.w - 1) * HistTexel<HF>::B);
        }
        cp_async_commit();
    }
    // 5. the boxes while the window is in flight
    typename Pol::Box box[NPX];
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        Pol::template box<HOT>(&sm.col[(NPX * ly + k + 1) * SX + lx + 1], SX, M, P.mVarClipGamma, box[k], z);
        if (Pol::kExactCentre)
            Pol::centre_colour(box[k], a.color, cx, min(y0 + NPX * ly + k, H - 1), tm, yc);
    }
    bool landed = true;
    if (mode == 1) {
        landed = mbar_wait_bounded(&sm.bar, phase & 1u, first_wait_polls(a.status));
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
    // 6. per pixel: rejection, history sample, rectification, blend, stores
    StoreFinish fin;
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        const int y = y0 + NPX * ly + k;
        const bool valid = x < W && y < H && landed;
        bool rejected = false;
        if (P.mRejectOutside && (hu[k] < 0.f || hv[k] < 0.f || hu[k] >= 1.f || hv[k] >= 1.f)) rejected = true;
        if (depth_cull) {
            const float hd = prev_depth[k];
            if (fabsf(hd - ehd[k]) > 0.1f * (1.0f - hd)) rejected = true;
        }
        if constexpr (RT) {
            if (x < W && y < H) {
                const uint32_t sg = seg::classify(P, x, y, hu[k], hv[k], W, H, StagedSeg<S>{ss, a, x0, y0});
                if ((sg & 3u) != 0) rejected = true;
                if (valid && a.segmask.p) *texel_ptr_w<uint32_t>(a.segmask, x, y) = sg;
                fin.seg = sg;
            }
        }
        float4 hraw = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid && have_hist) {
            HistoryTaps<Pol, INTERP> taps;
            taps.setup(hu[k], hv[k], hi.w, hi.h, z);
            const int span = INTERP == 2 ? 4 : 2;
            const int bx = taps.t[0].ux - wx0, by = taps.t[0].uy - wy0;
            const bool in_win = windowed && bx >= 0 && by >= 0 && bx + span <= WWS && by + span <= WH;
            if (in_win) {
                hraw = Pol::template filter_window<INTERP, HF, !HOT>(taps, &sm.win[by * WWS + bx], WWS);
            } else {
                hraw = Pol::template filter<INTERP, !HOT>(
                    taps, hi.w, hi.h, [&](int tx_, int ty_) { return fetch_history<HF>(hi, tx_, ty_); });
            }
        }
        if (M.anti_ghost()) anti_ghosting<MC>(a, cx, min(y, H - 1), hraw.w, rejected, fin.dyn);
        if (!HOT && a.debug.p && P.mDebugMode == 4) fin.dvel = fetch_velocity<MC>(a.velocity, x, y);
        const C3 c0 = Pol::centre(box[k], &sm.col[(NPX * ly + k + 1) * SX + lx + 1]);
        StoreFinish::run<Pol, HF, HOT>(U, a, P, M, box[k], c0, hraw, u[k], v[k], hu[k], hv[k], ehd[k], prev_depth[k],
                                       rejected, valid, x, y, tm, fin);
    }
}


// One view, one CTA per multi-pixel tile.
template <class Pol, class S, int HF, int MC, int INTERP, bool HOT, bool RT>
__global__ void __launch_bounds__(S::NT, TAA_MULTI_MIN_BLOCKS * 256 / S::NT)
    resolve_tile_multi(const taa_uniforms_t U, const FrameArgs a, const __grid_constant__ CUtensorMap hmap,
                       const int tma_ok) {
    __shared__ TileSmem<Pol, S, HF> sm;
    __shared__ SegStage<S, RT> ss;
    if (threadIdx.x == 0) mbar_init(&sm.bar, 1);
    uint32_t phase = 0;
    multi_body<Pol, S, HF, MC, INTERP, HOT, RT, false>(U, a, &hmap, tma_ok != 0, blockIdx.x, blockIdx.y, sm, ss,
                                                        phase);
}

// One view, one CTA per tile.
template <class Pol, class S, int HF, int MC, int INTERP, bool HOT>
__global__ void __launch_bounds__(S::NT, S::MIN_BLOCKS)
    resolve_tile(const taa_uniforms_t U, const FrameArgs a, const __grid_constant__ CUtensorMap hmap, const int tma_ok) {
    __shared__ TileSmem<Pol, S, HF> sm;
    if (threadIdx.x == 0) mbar_init(&sm.bar, 1);
    uint32_t phase = 0;
    StoreFinish fin;
    tile_body<Pol, S, HF, MC, INTERP, HOT, false>(U, a, &hmap, tma_ok != 0, blockIdx.x, blockIdx.y, sm, phase, fin);
}

// Resident 256-thread CTAs per SM the batch kernels' register budget is sized
// for (a tuning constant: 4, 64 registers, measured fastest on the 48-view batch).
#ifndef TAA_BATCH_MIN_BLOCKS
#define TAA_BATCH_MIN_BLOCKS 4
#endif
// The same for the multi-pixel shapes, which hold more live state per thread
// (3: up to 85 registers, measured fastest on the 48-view batch).
#ifndef TAA_BATCH_MULTI_MIN_BLOCKS
#define TAA_BATCH_MULTI_MIN_BLOCKS 3
#endif
template <class S> constexpr int batch_min_blocks() {
    constexpr int b = (S::kMulti ? TAA_BATCH_MULTI_MIN_BLOCKS : TAA_BATCH_MIN_BLOCKS) * 256 / S::NT;
    return b < 1 ? 1 : (b > 32 ? 32 : b);
}

// Many views in one launch: each CTA takes jobs blockIdx.x, blockIdx.x +
// gridDim.x, ... from the schedule's job list (BatchView and the job encoding
// are in common.cuh) - a persistent loop when the grid is smaller than the
// list.  A view's arguments are copied into shared memory when a CTA's job
// moves to another view.  maps[v] is view v's history tensor map for this tile
// shape, usable when tma_ok[v].
template <class Pol, class S, int HF, int MC, int INTERP, bool HOT>
__global__ void __launch_bounds__(S::NT, batch_min_blocks<S>())
    resolve_batch(const BatchView* __restrict__ views, const CUtensorMap* __restrict__ maps,
                  const int* __restrict__ tma_ok, const uint32_t* __restrict__ jobs, const int njobs) {
    __shared__ TileSmem<Pol, S, HF> sm;
    __shared__ __align__(16) BatchView s_view;
    static_assert(sizeof(BatchView) % 16 == 0, "copied as 16-byte words");
    constexpr int kWords = (int)(sizeof(BatchView) / 16);
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
            const uint4* src = reinterpret_cast<const uint4*>(views + vi);
            for (int w = threadIdx.x; w < kWords; w += S::NT) reinterpret_cast<uint4*>(&s_view)[w] = __ldg(src + w);
            if (threadIdx.x == 0)
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(maps + vi) : "memory");
            cur_view = vi;
            __syncthreads();
        }
        if constexpr (S::kMulti) {
            SegStage<S, false> none;
            multi_body<Pol, S, HF, MC, INTERP, HOT, false, true>(s_view.U, s_view.a, maps + vi,
                                                                  __ldg(tma_ok + vi) != 0, job_tile_x(job),
                                                                  job_tile_y(job), sm, none, phase);
        } else {
            StoreFinish fin;
            tile_body<Pol, S, HF, MC, INTERP, HOT, true>(s_view.U, s_view.a, maps + vi, __ldg(tma_ok + vi) != 0,
                                                         job_tile_x(job), job_tile_y(job), sm, phase, fin);
        }
        __syncthreads();  // the next tile reuses the shared memory
        if (sm.abort) return;
    }
}

#ifndef TAA_TILE_NPX
#define TAA_TILE_NPX 2  // pixels per thread of the single-view tiled forms
#endif

template <class Pol, int HF, int MC, int INTERP, bool HOT, bool RT = false>
cudaError_t launch_tile(const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    using S = typename std::conditional<TAA_TILE_NPX == 1, DefaultShape, MultiShape<32, 8, TAA_TILE_NPX>>::type;
    dim3 grid((a.out_w + S::TX - 1) / S::TX, (a.out_h + S::TY - 1) / S::TY);
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int tma_ok = INTERP != 1 && a.history.p && a.history.w >= Win<S, HF>::W && a.history.h >= S::WH &&
                       encode_history_map(a.history, HF, Win<S, HF>::W, S::WH, &map);
    if (TAA_TILE_NPX == 1 && !RT)
        resolve_tile<Pol, DefaultShape, HF, MC, INTERP, HOT><<<grid, S::NT, 0, s>>>(U, a, map, tma_ok);
    else
        resolve_tile_multi<Pol, MultiShape<32, 8, TAA_TILE_NPX>, HF, MC, INTERP, HOT, RT><<<grid, S::NT, 0, s>>>(
            U, a, map, tma_ok);
    return cudaGetLastError();
}

template <class Pol, int HF, int MC>
cudaError_t launch_interp(int interp, const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    const bool hot = is_hot(U.param[0]) && !a.debug.p, rt = U.param[0].mRayTraceAugment != 0;
    switch (interp) {
        case 0:
            return hot  ? launch_tile<Pol, HF, MC, 0, true>(U, a, s)
                   : rt ? launch_tile<Pol, HF, MC, 0, false, true>(U, a, s)
                        : launch_tile<Pol, HF, MC, 0, false>(U, a, s);
        case 1:
            return hot  ? launch_tile<Pol, HF, MC, 1, true>(U, a, s)
                   : rt ? launch_tile<Pol, HF, MC, 1, false, true>(U, a, s)
                        : launch_tile<Pol, HF, MC, 1, false>(U, a, s);
        default:
            return hot  ? launch_tile<Pol, HF, MC, 2, true>(U, a, s)
                   : rt ? launch_tile<Pol, HF, MC, 2, false, true>(U, a, s)
                        : launch_tile<Pol, HF, MC, 2, false>(U, a, s);
    }
}

template <class Pol>
cudaError_t launch_form(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U, const FrameArgs& a,
                        cudaStream_t s) {
    if (history_fmt == 0)
        return motion_ch == 4 ? launch_interp<Pol, 0, 4>(interp, U, a, s) : launch_interp<Pol, 0, 2>(interp, U, a, s);
    return motion_ch == 4 ? launch_interp<Pol, 1, 4>(interp, U, a, s) : launch_interp<Pol, 1, 2>(interp, U, a, s);
}

}  // namespace tiled
}  // namespace taa_dev
