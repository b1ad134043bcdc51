// resolve_learned_strips.cu - inference of the learned history rectifier
// (TAA_FORM_LEARNED, learned.cuh) on the strip body of the fast forms
// (strip_body.cuh): the colour tile staged in FP32 YCoCg, each thread a
// vertical strip of four pixels whose 3x3 boxes (mean, standard deviation,
// minimum, maximum) come from staged rows the strip shares; the history
// sample from the tile's TMA window; then for each of the strip's four
// pixels in turn, every warp runs its 32 lanes' features through the network
// with warp-wide MMAs (mma.sync m16n8k16, FP16 in, FP32 out, activations in
// registers) and clips and blends with the predicted weight and box scale
// (the plain variance clip where the scale leaves [0.5, 2]).
//
// Cost at 1920x1080 (CUDA graph of 8 frames): 77 us a frame, against 44 us
// for the tiled FP32 form and 31 us for TAA_FORM_FAST; without the network
// the same kernel takes 44 us.  The network's 36 mma.sync per 32 pixels
// (2 m-tiles x (8 + 8 + 2)) keep the tensor pipe 20 % busy (its peak is one
// m16n8k16 per 2 cycles per SM: 15 us for 2.07M pixels); the kernel is bound
// by latency at 20 warps per SM (5 CTAs of 96 registers and 42 KB), with the
// layers' dependent MMA chains, the feature and activation round trips
// through shared memory and instruction fetch (the unrolled network) in the
// stall reasons.  The tcgen05 variant (TAA_FLAG_LEARNED_TCGEN05, below) waits
// on six CTA-wide MMA round trips a tile and measures 89 us.
//
// The training records come from the tiled collection kernel of learned.cu;
// the features here are the same functions of the same quantities (the box
// from row sums and a product by 1/9 instead of the FP32 form's order - the
// network does not see the difference).
#include <cstring>

#include "learned.cuh"
#include "strip_body.cuh"

namespace taa_dev {
namespace fast32 {

constexpr int kLearnedWarps = NT / 32;
using Net = learned::WarpNetN<kLearnedWarps>;

struct LearnedStripPol {
    using Staged = float4;
    struct Ctx {
        Net* net;
    };
    static __device__ __forceinline__ float4 stage(uint2 raw) { return F32Pol::stage(raw); }

    static __device__ __forceinline__ void finish(const Args& a, const float4* sp, int x, int ya, const float3 h[NPX],
                                                  unsigned rej, bool landed, const PixelInfo& px, Ctx& ctx) {
        Row r0 = row_sums(sp), r1 = row_sums(sp + SX);
        RowMinMax q0 = row_minmax(sp), q1 = row_minmax(sp + SX);
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            const Row r2 = row_sums(sp + (k + 2) * SX);
            const RowMinMax q2 = row_minmax(sp + (k + 2) * SX);
            const Row s = add(add(r0, r1), r2);
            learned::FeatureIn fi;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                fi.mn[c] = fminf(q0.mn[c], fminf(q1.mn[c], q2.mn[c]));
                fi.mx[c] = fmaxf(q0.mx[c], fmaxf(q1.mx[c], q2.mx[c]));
            }
            r0 = r1;
            r1 = r2;
            q0 = q1;
            q1 = q2;
            const int y = ya + k;
            const bool valid = x < a.W && y < a.H && landed;
            // mean and standard deviation of the box (taa.comp:266-277)
            const f2 n = dup(1.0f / 9.0f);
            const f2 mean = mulp(s.a, n), cg = mulp(s.c, n);
            const f2 var = fmap(neg2(mean), mean, mulp(s.q, n));
            fi.mean[0] = f2lo(mean);
            fi.mean[1] = f2hi(mean);
            fi.mean[2] = f2lo(cg);
            fi.sigma[0] = learned::sqrt_approx(fmaxf(f2lo(var), 0.f));
            fi.sigma[1] = learned::sqrt_approx(fmaxf(f2hi(var), 0.f));
            fi.sigma[2] = learned::sqrt_approx(fmaxf(fmaf(-f2lo(cg), f2lo(cg), f2hi(cg)), 0.f));
            hist_ycocg(h[k], fi.hist);
            const float4 c0 = lds128(&sp[(k + 1) * SX + 1]);
            fi.cur[0] = c0.x;
            fi.cur[1] = c0.y;
            fi.cur[2] = c0.z;
            const float du = (px.u - px.hu[k]) * (float)a.W, dv = (px.v[k] - px.hv[k]) * (float)a.H;
            fi.vel_px = learned::sqrt_approx(du * du + dv * dv);
            fi.depth_rel = a.depth_cull ? __fdividef(px.pd[k] - px.ehd[k], 0.1f * (1.0f - px.pd[k]) + 1e-6f) : 0.f;
            const bool rejected = (rej >> k) & 1u;
            fi.rejected = rejected;
            float f[learned::kIn];
            if (valid) {
                learned::features(fi, f);
            } else {
#pragma unroll
                for (int i = 0; i < learned::kIn; ++i) f[i] = 0.f;
            }
            // every lane of the warp takes part in the network
            float o0, o1;
            learned::forward_warp(*ctx.net, f, o0, o1);
            if (!valid) continue;
            float alpha = learned::out_alpha(o0), scale = learned::out_scale(o1);
            if (!(scale >= 0.5f && scale <= 2.0f)) {  // outside the trusted range: the plain variance clip
                scale = 1.f;
                alpha = a.alpha;
            }
            if (a.reset) alpha = 1.0f;
            else if (rejected) alpha = a.rejection_alpha;
            float e[3], o[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) e[c] = scale * a.gamma * fi.sigma[c] + 1e-7f;
            learned::rectify_blend(fi.mean, e, fi.hist, fi.cur, alpha, o);
            const float tmp = o[0] - o[2];
            const float rr = tmp + o[1], g = o[0] + o[2], bl = tmp - o[1];
            *at_w<float4>(a.hout, a.hout_pitch, x, y) = make_float4(rr, g, bl, 0.f);
            if (a.result)
                *at_w<uint2>(a.result, a.result_pitch, x, y) = float4_to_half4(make_float4(rr, g, bl, 1.0f));
        }
    }
};

// The same inference with the network on the 5th-generation tensor cores:
// the CTA's 512 pixels go through it in two rounds of 256 (pixels 0-1, then
// 2-3 of every strip), each round two 128-row blocks (row = thread) whose
// FP16 activations sit in canonical K-major tiles over the history window
// (dead once the history is sampled); per layer one thread issues the four
// tcgen05.mma (M 128, N 32, K 16) into tensor memory, everyone waits on the
// commit, reads its two rows back (tcgen05.ld), applies the ReLU and writes
// the next layer's operand in place.
struct LearnedTcPol {
    using Staged = float4;
    static constexpr int kTile = learned::kRows * learned::kIn * 2;  // one 128-row activation tile
    static constexpr int NB = 2;  // 128-row blocks per round
    struct Ctx {
        char* tiles;       // the two activation tiles (over the history window)
        const char* w;     // the blob's inference matrices in shared memory
        uint64_t* bar;     // MMA completion
        uint32_t tmem;     // one 32-column accumulator per block
        uint32_t phase;
        bool ok;
    };
    static __device__ __forceinline__ float4 stage(uint2 raw) { return F32Pol::stage(raw); }

    static __device__ __forceinline__ void finish(const Args& a, const float4* sp, int x, int ya, const float3 h[NPX],
                                                  unsigned rej, bool landed, const PixelInfo& px, Ctx& ctx) {
        using namespace learned;
        const int t = threadIdx.x;
        const uint32_t lane_cols = ctx.tmem + ((uint32_t)((t >> 5) & 3) * 32u << 16);
        char* const tiles[NB] = {ctx.tiles, ctx.tiles + kTile};
        __syncthreads();  // every thread is done with the history window the tiles overlay
        Row r0 = row_sums(sp), r1 = row_sums(sp + SX);
        RowMinMax q0 = row_minmax(sp), q1 = row_minmax(sp + SX);
#pragma unroll
        for (int half = 0; half < NPX / NB; ++half) {
            float mean[NB][3], sigma[NB][3];
#pragma unroll
            for (int kk = 0; kk < NB; ++kk) {
                const int k = NB * half + kk;
                const Row r2 = row_sums(sp + (k + 2) * SX);
                const RowMinMax q2 = row_minmax(sp + (k + 2) * SX);
                const Row s = add(add(r0, r1), r2);
                FeatureIn fi;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    fi.mn[c] = fminf(q0.mn[c], fminf(q1.mn[c], q2.mn[c]));
                    fi.mx[c] = fmaxf(q0.mx[c], fmaxf(q1.mx[c], q2.mx[c]));
                }
                r0 = r1;
                r1 = r2;
                q0 = q1;
                q1 = q2;
                const bool valid = x < a.W && ya + k < a.H && landed;
                const f2 n = dup(1.0f / 9.0f);
                const f2 m = mulp(s.a, n), cg = mulp(s.c, n);
                const f2 var = fmap(neg2(m), m, mulp(s.q, n));
                fi.mean[0] = f2lo(m);
                fi.mean[1] = f2hi(m);
                fi.mean[2] = f2lo(cg);
                fi.sigma[0] = sqrt_approx(fmaxf(f2lo(var), 0.f));
                fi.sigma[1] = sqrt_approx(fmaxf(f2hi(var), 0.f));
                fi.sigma[2] = sqrt_approx(fmaxf(fmaf(-f2lo(cg), f2lo(cg), f2hi(cg)), 0.f));
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    mean[kk][c] = fi.mean[c];
                    sigma[kk][c] = fi.sigma[c];
                }
                hist_ycocg(h[k], fi.hist);
                const float4 c0 = lds128(&sp[(k + 1) * SX + 1]);
                fi.cur[0] = c0.x;
                fi.cur[1] = c0.y;
                fi.cur[2] = c0.z;
                const float du = (px.u - px.hu[k]) * (float)a.W, dv = (px.v[k] - px.hv[k]) * (float)a.H;
                fi.vel_px = sqrt_approx(du * du + dv * dv);
                fi.depth_rel =
                    a.depth_cull ? __fdividef(px.pd[k] - px.ehd[k], 0.1f * (1.0f - px.pd[k]) + 1e-6f) : 0.f;
                fi.rejected = (rej >> k) & 1u;
                float f[kIn];
                if (valid) {
                    features(fi, f);
                } else {
#pragma unroll
                    for (int i = 0; i < kIn; ++i) f[i] = 0.f;
                }
                store_row(tiles[kk], t, f);
            }
            // the network on the round's 256 pixels
            float acc[32];
            sync_for_mma();
            ctx.ok &= layer(tiles, ctx.w + Blob::W1, kHid, ctx.tmem, NB, ctx.bar, ctx.phase);
#pragma unroll
            for (int kk = 0; kk < NB; ++kk) {
                tc::ld32(lane_cols + (uint32_t)(kk * 32), acc);
                store_row_relu(tiles[kk], t, acc);
            }
            sync_for_mma();
            ctx.ok &= layer(tiles, ctx.w + Blob::W2, kHid, ctx.tmem, NB, ctx.bar, ctx.phase);
#pragma unroll
            for (int kk = 0; kk < NB; ++kk) {
                tc::ld32(lane_cols + (uint32_t)(kk * 32), acc);
                store_row_relu(tiles[kk], t, acc);
            }
            sync_for_mma();
            ctx.ok &= layer(tiles, ctx.w + Blob::W3, kOutPad, ctx.tmem, NB, ctx.bar, ctx.phase);
            float o[NB][2];
#pragma unroll
            for (int kk = 0; kk < NB; ++kk) {
                float v[16];
                tc::ld16(lane_cols + (uint32_t)(kk * 32), v);
                o[kk][0] = v[0];
                o[kk][1] = v[1];
            }
            tc::fence_before_sync();  // the next round's MMAs overwrite these columns after a barrier
#pragma unroll
            for (int kk = 0; kk < NB; ++kk) {
                const int k = NB * half + kk, y = ya + k;
                if (!(x < a.W && y < a.H && landed)) continue;
                const bool rejected = (rej >> k) & 1u;
                float alpha = out_alpha(o[kk][0]), scale = out_scale(o[kk][1]);
                if (!(scale >= 0.5f && scale <= 2.0f)) {  // outside the trusted range: the plain variance clip
                    scale = 1.f;
                    alpha = a.alpha;
                }
                if (a.reset) alpha = 1.0f;
                else if (rejected) alpha = a.rejection_alpha;
                float hy[3], cur[3], e[3], out[3];
                hist_ycocg(h[k], hy);
                const float4 c0 = lds128(&sp[(k + 1) * SX + 1]);
                cur[0] = c0.x;
                cur[1] = c0.y;
                cur[2] = c0.z;
#pragma unroll
                for (int c = 0; c < 3; ++c) e[c] = scale * a.gamma * sigma[kk][c] + 1e-7f;
                rectify_blend(mean[kk], e, hy, cur, alpha, out);
                const float tmp = out[0] - out[2];
                const float rr = tmp + out[1], g = out[0] + out[2], bl = tmp - out[1];
                *at_w<float4>(a.hout, a.hout_pitch, x, y) = make_float4(rr, g, bl, 0.f);
                if (a.result)
                    *at_w<uint2>(a.result, a.result_pitch, x, y) = float4_to_half4(make_float4(rr, g, bl, 1.0f));
            }
        }
    }
};

// Resident CTAs per SM (42 KB of shared memory each: the strip tile and the
// network's weights and feature rows).
#ifndef TAA_LEARNED_STRIP_MIN_BLOCKS
#define TAA_LEARNED_STRIP_MIN_BLOCKS 5
#endif

template <int MC>
__global__ void __launch_bounds__(NT, TAA_LEARNED_STRIP_MIN_BLOCKS)
    resolve_strips_learned(const Args a, const __grid_constant__ CUtensorMap hmap, const int tma_ok,
                           const char* __restrict__ blob) {
    __shared__ SmemT<float4> sm;
    __shared__ Net net;
    learned::load_warp_weights(net, blob);
    __syncthreads();
    uint32_t phase = 0;
    LearnedStripPol::Ctx ctx{&net};
    strip_tile<LearnedStripPol, 2, MC, false>(a, &hmap, tma_ok, blockIdx.x, blockIdx.y, sm, phase, ctx);
}

#ifndef TAA_LEARNED_TC_STRIP_MIN_BLOCKS
#define TAA_LEARNED_TC_STRIP_MIN_BLOCKS 5
#endif

// Shared memory of the tensor-core variant beside the strip tile: the blob's
// inference matrices, the MMA barrier and the tensor-memory base.
struct TcNetSmem {
    alignas(128) char w[learned::Blob::INFER_BYTES];
    uint64_t bar;
    uint32_t tmem;
};
static_assert(sizeof(float4) * WW * WH >= 2 * LearnedTcPol::kTile, "the activation tiles fit over the window");

template <int MC>
__global__ void __launch_bounds__(NT, TAA_LEARNED_TC_STRIP_MIN_BLOCKS)
    resolve_strips_learned_tc(const Args a, const __grid_constant__ CUtensorMap hmap, const int tma_ok,
                              const char* __restrict__ blob) {
    __shared__ SmemT<float4> sm;
    __shared__ TcNetSmem net;
    if (threadIdx.x == 0) mbar_init(&net.bar, 1);
    learned::copy_blob(net.w, blob, learned::Blob::INFER_BYTES);
    constexpr uint32_t kCols = 32 * LearnedTcPol::NB;
    if (threadIdx.x < 32) tc::tmem_alloc(&net.tmem, kCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    uint32_t phase = 0;
    LearnedTcPol::Ctx ctx{reinterpret_cast<char*>(sm.win), net.w, &net.bar, net.tmem, 0u, true};
    strip_tile<LearnedTcPol, 2, MC, false>(a, &hmap, tma_ok, blockIdx.x, blockIdx.y, sm, phase, ctx);
    if (!ctx.ok && threadIdx.x == 0) atomicOr(a.status, kStatusWindowTimeout);
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_free(net.tmem, kCols);
}

}  // namespace fast32

cudaError_t launch_resolve_learned_strips_tc(int motion_ch, const taa_uniforms_t& U, const FrameArgs& f,
                                             const char* blob, cudaStream_t s) {
    using namespace fast32;
    const Args a = make_args(U, f);
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int tma_ok = a.hist && f.history.w >= WW && f.history.h >= WH &&
                       encode_history_map(f.history, TAA_FAST_TMA2D ? 2 : 0, WW, WH, &map);
    const dim3 grid((a.W + TX - 1) / TX, (a.H + TY - 1) / TY);
    if (motion_ch == 4) resolve_strips_learned_tc<4><<<grid, NT, 0, s>>>(a, map, tma_ok, blob);
    else resolve_strips_learned_tc<2><<<grid, NT, 0, s>>>(a, map, tma_ok, blob);
    return cudaGetLastError();
}

cudaError_t launch_resolve_learned_strips(int motion_ch, const taa_uniforms_t& U, const FrameArgs& f,
                                          const char* blob, cudaStream_t s) {
    using namespace fast32;
    const Args a = make_args(U, f);
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int tma_ok = a.hist && f.history.w >= WW && f.history.h >= WH &&
                       encode_history_map(f.history, TAA_FAST_TMA2D ? 2 : 0, WW, WH, &map);
    const dim3 grid((a.W + TX - 1) / TX, (a.H + TY - 1) / TY);
    if (motion_ch == 4) resolve_strips_learned<4><<<grid, NT, 0, s>>>(a, map, tma_ok, blob);
    else resolve_strips_learned<2><<<grid, NT, 0, s>>>(a, map, tma_ok, blob);
    return cudaGetLastError();
}

}  // namespace taa_dev
