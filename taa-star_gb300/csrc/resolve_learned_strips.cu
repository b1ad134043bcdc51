// resolve_learned_strips.cu - inference of the learned history rectifier
// (TAA_FORM_LEARNED, learned.cuh) on the strip body of the fast forms
// (strip_body.cuh): the colour tile staged in FP32 YCoCg, each thread a
// vertical strip of four pixels whose 3x3 boxes (mean, standard deviation,
// minimum, maximum) come from staged rows the strip shares, each row read
// once for its sums and extrema; the history sample from the tile's TMA
// window.  Then the strip's pixels go through the network two at a time:
// every warp writes its 64 pixels' FP16 feature rows over the history window
// (dead once every warp has its samples), loads the three layers' weight
// fragments into registers and runs its four 16-row m-tiles through the
// layers with warp-wide MMAs (mma.sync m16n8k16, FP16 in, FP32 out, the
// activations rounded and clamped by one cvt.rn.relu per pair and kept in
// registers); each pixel then clips and blends with its predicted weight and
// box scale (the plain variance clip where the scale leaves [0.5, 2]).
//
// Cost at 1920x1080 (20 launches on one frame): 68 us, against 48 us for
// the exact tiled FP32 form and 34 us for TAA_FORM_FAST.  Measured by parts
// (variants with a part removed): the network 16 us, the features 6 us; the
// rest is the strip body at 128 registers (4 CTAs per SM: fewer registers
// spill and measure slower, 5 CTAs 73 us).  The weights reach shared memory
// by cp.async from the blob's row-major image while the strip's inputs load
// (a per-element copy from the canonical layout at the start of every CTA
// cost 11 us).  The tcgen05 variant (TAA_FLAG_LEARNED_TCGEN05, below) runs
// the same network with the same bits, its features and activations in
// tensor memory: 79 us (93 us with the activations in shared-memory operand
// tiles and six CTA-wide MMA round trips a tile, a variant since removed).
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

// Pixels of a strip that go through the network together: the warp's rows
// are KB x 32 (KB m-tile pairs), so a layer's weight fragments, held in
// registers for the whole strip, meet 2 x KB independent m-tiles.
#ifndef TAA_LEARNED_BATCH
#define TAA_LEARNED_BATCH 2
#endif
// Whether a batch reads its first two staged rows again instead of holding
// the previous batch's across the network (spill-free at 126 registers: 68.4
// against 69.2 us per 1080p frame).
#ifndef TAA_LEARNED_RECOMPUTE_ROWS
#define TAA_LEARNED_RECOMPUTE_ROWS 1
#endif
constexpr int KB = TAA_LEARNED_BATCH;
static_assert(NPX % KB == 0, "the strip splits into whole batches");
constexpr int kFeatRow = learned::kIn * 2;  // bytes of one FP16 feature row
static_assert(NT / 32 * KB * 32 * kFeatRow <= (int)sizeof(float4) * WW * WH,
              "every warp's feature rows fit over the history window");

// The network's weights (padded rows: conflict-free ldmatrix) and one output
// pair per feature row of a batch (the feature rows overlay the history
// window, free once every warp has its samples).
struct NetSmem {
    alignas(16) __half w1[learned::kHid][learned::kPad];
    alignas(16) __half w2[learned::kHid][learned::kPad];
    alignas(16) __half w3[8][learned::kPad];
    float2 out[kLearnedWarps][KB * 32];
};
static_assert(offsetof(NetSmem, w2) == 2560 && offsetof(NetSmem, w3) == 5120,
              "w1, w2, w3 back to back as in the blob's image");

// Byte offset of 16-byte chunk c (features 8c .. 8c+7) of feature row r: the
// chunks of rows 2i and 2i+1 are rotated by i, so the eight rows an ldmatrix
// phase reads (and the eight a store phase writes) fall in distinct banks.
__device__ __forceinline__ uint32_t feat_off(int r, int c) { return (uint32_t)(r * kFeatRow + ((c ^ ((r >> 1) & 3)) << 4)); }

// Two FP32 activations rounded to FP16 and clamped at zero, packed (a low,
// b high) in one conversion: learned::pack_relu's values.
__device__ __forceinline__ uint32_t cvt_relu(float a, float b) {
    uint32_t d;
    asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
    return d;
}

// One hidden layer of a 16-row m-tile with the B fragments in registers: the
// arithmetic of learned::warp_layer.
__device__ __forceinline__ void layer_rb(const uint32_t (&a)[2][4], const uint32_t (&b)[4][4], uint32_t (&h)[2][4]) {
    float acc[4][4];
#pragma unroll
    for (int nj = 0; nj < 4; ++nj) {
        acc[nj][0] = acc[nj][1] = acc[nj][2] = acc[nj][3] = 0.f;
        learned::mma16816(acc[nj], a[0], b[nj][0], b[nj][1]);
        learned::mma16816(acc[nj], a[1], b[nj][2], b[nj][3]);
    }
#pragma unroll
    for (int kj = 0; kj < 2; ++kj) {
        h[kj][0] = cvt_relu(acc[2 * kj][0], acc[2 * kj][1]);
        h[kj][1] = cvt_relu(acc[2 * kj][2], acc[2 * kj][3]);
        h[kj][2] = cvt_relu(acc[2 * kj + 1][0], acc[2 * kj + 1][1]);
        h[kj][3] = cvt_relu(acc[2 * kj + 1][2], acc[2 * kj + 1][3]);
    }
}

// The 3x3 sums and extrema of one staged row segment from one read of its texels.
__device__ __forceinline__ void row_stats(const float4* p, Row& r, RowMinMax& q) {
    const float4 t0 = lds128(p), t1 = lds128(p + 1), t2 = lds128(p + 2);
    const f2 a0 = pk(t0.x, t0.y), a1 = pk(t1.x, t1.y), a2 = pk(t2.x, t2.y);
    r.a = addp(addp(a0, a1), a2);
    r.c = addp(addp(pk(t0.z, t0.w), pk(t1.z, t1.w)), pk(t2.z, t2.w));
    r.q = fmap(a2, a2, fmap(a1, a1, mulp(a0, a0)));
    q = {{fminf(t0.x, fminf(t1.x, t2.x)), fminf(t0.y, fminf(t1.y, t2.y)), fminf(t0.z, fminf(t1.z, t2.z))},
         {fmaxf(t0.x, fmaxf(t1.x, t2.x)), fmaxf(t0.y, fmaxf(t1.y, t2.y)), fmaxf(t0.z, fmaxf(t1.z, t2.z))}};
}

struct LearnedStripPol {
    using Staged = float4;
    struct Ctx {
        NetSmem* net;
        char* feat;  // the feature rows, over the history window (dead once the samples are taken)
    };
    static __device__ __forceinline__ float4 stage(uint2 raw) { return F32Pol::stage(raw); }

    static __device__ __forceinline__ void finish(const Args& a, const float4* sp, int x, int ya, const float3 h[NPX],
                                                  unsigned rej, bool landed, const PixelInfo& px, Ctx& ctx) {
        using namespace learned;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        NetSmem& net = *ctx.net;
        char* const ft = ctx.feat + warp * (KB * 32 * kFeatRow);
        // the motion features of the strip's pixels (the rest of PixelInfo dies here)
        float vel_px[NPX], depth_rel[NPX];
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            const float du = (px.u - px.hu[k]) * (float)a.W, dv = (px.v[k] - px.hv[k]) * (float)a.H;
            vel_px[k] = learned::sqrt_approx(du * du + dv * dv);
            depth_rel[k] = a.depth_cull ? __fdividef(px.pd[k] - px.ehd[k], 0.1f * (1.0f - px.pd[k]) + 1e-6f) : 0.f;
        }
        // every warp has its history samples (the window is free) and its share of the weights
        cp_async_wait_all();
        __syncthreads();
        Row r0, r1;
        RowMinMax q0, q1;
#pragma unroll
        for (int hb = 0; hb < NPX / KB; ++hb) {
            // the batch's first two staged rows (read again rather than held
            // across the network: fewer live registers)
            if (TAA_LEARNED_RECOMPUTE_ROWS || hb == 0) {
                row_stats(sp + (hb * KB) * SX, r0, q0);
                row_stats(sp + (hb * KB + 1) * SX, r1, q1);
            }
            float mean[KB][3], sigma[KB][3];
            // features of the batch's pixels: FP16 row kk * 32 + lane
#pragma unroll
            for (int kk = 0; kk < KB; ++kk) {
                const int k = hb * KB + kk;
                Row r2;
                RowMinMax q2;
                row_stats(sp + (k + 2) * SX, r2, q2);
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
                // mean and standard deviation of the box (taa.comp:266-277)
                const f2 n = dup(1.0f / 9.0f);
                const f2 m = mulp(s.a, n), cg = mulp(s.c, n);
                const f2 var = fmap(neg2(m), m, mulp(s.q, n));
                fi.mean[0] = f2lo(m);
                fi.mean[1] = f2hi(m);
                fi.mean[2] = f2lo(cg);
                fi.sigma[0] = learned::sqrt_approx(fmaxf(f2lo(var), 0.f));
                fi.sigma[1] = learned::sqrt_approx(fmaxf(f2hi(var), 0.f));
                fi.sigma[2] = learned::sqrt_approx(fmaxf(fmaf(-f2lo(cg), f2lo(cg), f2hi(cg)), 0.f));
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
                fi.vel_px = vel_px[k];
                fi.depth_rel = depth_rel[k];
                fi.rejected = (rej >> k) & 1u;
                float f[kIn];
                if (valid) {
                    features(fi, f);
                } else {
#pragma unroll
                    for (int i = 0; i < kIn; ++i) f[i] = 0.f;
                }
                const int row = kk * 32 + lane;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    __half2 q[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) q[e] = __floats2half2_rn(f[8 * j + 2 * e], f[8 * j + 2 * e + 1]);
                    uint4 wv;
                    wv.x = *reinterpret_cast<uint32_t*>(&q[0]);
                    wv.y = *reinterpret_cast<uint32_t*>(&q[1]);
                    wv.z = *reinterpret_cast<uint32_t*>(&q[2]);
                    wv.w = *reinterpret_cast<uint32_t*>(&q[3]);
                    *reinterpret_cast<uint4*>(ft + feat_off(row, j)) = wv;
                }
            }
            __syncwarp();
            // the three layers' B fragments, held for the batch's 2 x KB m-tiles
            uint32_t b1[4][4], b2[4][4], b3[4];
#pragma unroll
            for (int nj = 0; nj < 4; ++nj) {
                ldsm_x4(b1[nj], &net.w1[nj * 8 + (lane & 7)][(lane >> 3) * 8]);
                ldsm_x4(b2[nj], &net.w2[nj * 8 + (lane & 7)][(lane >> 3) * 8]);
            }
            ldsm_x4(b3, &net.w3[lane & 7][(lane >> 3) * 8]);
            // the network on the batch's m-tiles (m-tile mt: rows 16 mt .. 16 mt + 15)
#pragma unroll
            for (int mt = 0; mt < 2 * KB; ++mt) {
                uint32_t a0[2][4], a1[2][4], a2[2][4];
#pragma unroll
                for (int kj = 0; kj < 2; ++kj) ldsm_x4(a0[kj], ft + feat_off(mt * 16 + (lane & 15), 2 * kj + (lane >> 4)));
                layer_rb(a0, b1, a1);
                layer_rb(a1, b2, a2);
                float o[4] = {0.f, 0.f, 0.f, 0.f};
                mma16816(o, a2[0], b3[0], b3[1]);
                mma16816(o, a2[1], b3[2], b3[3]);
                // outputs 0 and 1 of rows g and g + 8 sit in lane 4 g
                if ((lane & 3) == 0) {
                    net.out[warp][mt * 16 + (lane >> 2)] = make_float2(o[0], o[1]);
                    net.out[warp][mt * 16 + (lane >> 2) + 8] = make_float2(o[2], o[3]);
                }
            }
            __syncwarp();
            // clip and blend with the predicted weight and box scale
#pragma unroll
            for (int kk = 0; kk < KB; ++kk) {
                const int k = hb * KB + kk, y = ya + k;
                const float2 oo = net.out[warp][kk * 32 + lane];
                if (!(x < a.W && y < a.H && landed)) continue;
                float alpha = out_alpha(oo.x), scale = out_scale(oo.y);
                if (!(scale >= 0.5f && scale <= 2.0f)) {  // outside the trusted range: the plain variance clip
                    scale = 1.f;
                    alpha = a.alpha;
                }
                float hy[3], cur[3], e[3], o[3];
                hist_ycocg(h[k], hy);
                const float4 c0 = lds128(&sp[(k + 1) * SX + 1]);
                cur[0] = c0.x;
                cur[1] = c0.y;
                cur[2] = c0.z;
                if (current_outlier(mean[kk], sigma[kk], cur, a.gamma)) alpha = fminf(alpha, a.alpha);
                if (a.reset) alpha = 1.0f;
                else if ((rej >> k) & 1u) alpha = a.rejection_alpha;
#pragma unroll
                for (int c = 0; c < 3; ++c) e[c] = scale * a.gamma * sigma[kk][c] + 1e-7f;
                rectify_blend(mean[kk], e, hy, cur, alpha, o);
                const float tmp = o[0] - o[2];
                const float rr = tmp + o[1], g = o[0] + o[2], bl = tmp - o[1];
                *at_w<float4>(a.hout, a.hout_pitch, x, y) = make_float4(rr, g, bl, 0.f);
                if (a.result)
                    *at_w<uint2>(a.result, a.result_pitch, x, y) = float4_to_half4(make_float4(rr, g, bl, 1.0f));
            }
            __syncwarp();  // the batch's feature rows and outputs are free
        }
    }
};

// Resident CTAs per SM the register budget is sized for (34 KB of shared
// memory each: the strip tile, the network's weights and outputs).
#ifndef TAA_LEARNED_STRIP_MIN_BLOCKS
#define TAA_LEARNED_STRIP_MIN_BLOCKS 4
#endif

template <int MC>
__global__ void __launch_bounds__(NT, TAA_LEARNED_STRIP_MIN_BLOCKS)
    resolve_strips_learned(const Args a, const __grid_constant__ CUtensorMap hmap, const int tma_ok,
                           const char* __restrict__ blob) {
    __shared__ SmemT<float4> sm;
    __shared__ NetSmem net;
    // the weights' image copied asynchronously: the strip body's loads go out
    // first; the copies complete (cp.async.wait_group 0) before the barrier in
    // front of the network
    for (int w = threadIdx.x; w < learned::Blob::WARP_BYTES / 16; w += NT)
        cp_async<16>(reinterpret_cast<char*>(&net.w1[0][0]) + 16 * w, blob + learned::Blob::WARP + 16 * w);
    cp_async_commit();
    uint32_t phase = 0;
    LearnedStripPol::Ctx ctx{&net, reinterpret_cast<char*>(sm.win)};
    strip_tile<LearnedStripPol, 2, MC, false>(a, &hmap, tma_ok, blockIdx.x, blockIdx.y, sm, phase, ctx);
}

// The network on the 5th-generation tensor cores with every activation in
// tensor memory: each thread (one TMEM lane, row = thread) stores its pixel's
// 32 FP16 features as 16 packed columns (tcgen05.st); per layer one thread
// issues, for each of the round's NBT 128-row blocks, two MMAs that read A
// from those columns and B (the weights) from shared memory and accumulate
// 32 FP32 columns; every thread reads its row back (tcgen05.ld), rounds and
// clamps it to FP16 pairs (cvt.rn.relu) and stores it as the next layer's A.
// No activation passes through shared memory.  Columns: D of block b at
// 32 b, A of block b at 32 NBT + 16 b.
#ifndef TAA_LEARNED_TM_NB
#define TAA_LEARNED_TM_NB 2
#endif
#ifndef TAA_LEARNED_TM_STRIP_MIN_BLOCKS
#define TAA_LEARNED_TM_STRIP_MIN_BLOCKS 4
#endif
template <int NBT> struct LearnedTmemPol {
    using Staged = float4;
    static constexpr int NB = NBT;
    static constexpr uint32_t kCols = NB == 1 ? 64u : NB == 2 ? 128u : 256u;
    static_assert(NPX % NB == 0 && 48 * NB <= (int)kCols, "whole rounds in the allocation");
    struct Ctx {
        const char* w;   // the blob's inference matrices in shared memory
        uint64_t* bar;   // MMA completion
        uint32_t tmem;
        uint32_t phase;
        bool ok;
    };
    static __device__ __forceinline__ float4 stage(uint2 raw) { return F32Pol::stage(raw); }

    // One layer for the round's blocks: A from TMEM, B = w (K 32), N = n.
    static __device__ __forceinline__ bool layer(Ctx& ctx, const char* w, int n) {
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (threadIdx.x == 0) {
            const uint32_t idesc = tc::idesc_f16(128, n);
#pragma unroll
            for (int b = 0; b < NB; ++b)
#pragma unroll
                for (int ks = 0; ks < 2; ++ks)
                    tc::mma_f16_ta(ctx.tmem + (uint32_t)(32 * b), ctx.tmem + (uint32_t)(32 * NB + 16 * b + 8 * ks),
                                   tc::smem_desc(w + ks * 256, 128, 512), idesc, ks > 0);
            tc::commit(ctx.bar);
        }
        const bool ok = learned::wait_bar(ctx.bar, ctx.phase);
        ctx.phase ^= 1u;
        tc::fence_after_sync();
        return ok;
    }

    static __device__ __forceinline__ void finish(const Args& a, const float4* sp, int x, int ya, const float3 h[NPX],
                                                  unsigned rej, bool landed, const PixelInfo& px, Ctx& ctx) {
        using namespace learned;
        const int t = threadIdx.x;
        const uint32_t lane_base = ((uint32_t)((t >> 5) & 3) * 32u) << 16;
        const uint32_t d0 = ctx.tmem + lane_base, a0 = ctx.tmem + lane_base + (uint32_t)(32 * NB);
        float vel_px[NPX], depth_rel[NPX];
#pragma unroll
        for (int k = 0; k < NPX; ++k) {
            const float du = (px.u - px.hu[k]) * (float)a.W, dv = (px.v[k] - px.hv[k]) * (float)a.H;
            vel_px[k] = sqrt_approx(du * du + dv * dv);
            depth_rel[k] = a.depth_cull ? __fdividef(px.pd[k] - px.ehd[k], 0.1f * (1.0f - px.pd[k]) + 1e-6f) : 0.f;
        }
        Row r0, r1;
        RowMinMax q0, q1;
        row_stats(sp, r0, q0);
        row_stats(sp + SX, r1, q1);
#pragma unroll
        for (int rd = 0; rd < NPX / NB; ++rd) {
            float mean[NB][3], sigma[NB][3];
#pragma unroll
            for (int kk = 0; kk < NB; ++kk) {
                const int k = NB * rd + kk;
                Row r2;
                RowMinMax q2;
                row_stats(sp + (k + 2) * SX, r2, q2);
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
                fi.vel_px = vel_px[k];
                fi.depth_rel = depth_rel[k];
                fi.rejected = (rej >> k) & 1u;
                float f[kIn];
                if (valid) {
                    features(fi, f);
                } else {
#pragma unroll
                    for (int i = 0; i < kIn; ++i) f[i] = 0.f;
                }
                uint32_t q[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    __half2 hh = __floats2half2_rn(f[2 * i], f[2 * i + 1]);
                    q[i] = *reinterpret_cast<uint32_t*>(&hh);
                }
                tc::st16(a0 + (uint32_t)(16 * kk), q);
            }
            tc::wait_st();
            // hidden layers: D -> ReLU'd FP16 -> the next A, in tensor memory
#pragma unroll
            for (int l = 0; l < 2; ++l) {
                ctx.ok &= layer(ctx, ctx.w + (l == 0 ? Blob::W1 : Blob::W2), kHid);
#pragma unroll
                for (int kk = 0; kk < NB; ++kk) {
                    float acc[32];
                    tc::ld32(d0 + (uint32_t)(32 * kk), acc);
                    uint32_t q[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) q[i] = cvt_relu(acc[2 * i], acc[2 * i + 1]);
                    tc::st16(a0 + (uint32_t)(16 * kk), q);
                }
                tc::wait_st();
            }
            ctx.ok &= layer(ctx, ctx.w + Blob::W3, kOutPad);
            float o[NB][2];
#pragma unroll
            for (int kk = 0; kk < NB; ++kk) {
                float v[16];
                tc::ld16(d0 + (uint32_t)(32 * kk), v);
                o[kk][0] = v[0];
                o[kk][1] = v[1];
            }
#pragma unroll
            for (int kk = 0; kk < NB; ++kk) {
                const int k = NB * rd + kk, y = ya + k;
                if (!(x < a.W && y < a.H && landed)) continue;
                float alpha = out_alpha(o[kk][0]), scale = out_scale(o[kk][1]);
                if (!(scale >= 0.5f && scale <= 2.0f)) {  // outside the trusted range: the plain variance clip
                    scale = 1.f;
                    alpha = a.alpha;
                }
                float hy[3], cur[3], e[3], out[3];
                hist_ycocg(h[k], hy);
                const float4 c0 = lds128(&sp[(k + 1) * SX + 1]);
                cur[0] = c0.x;
                cur[1] = c0.y;
                cur[2] = c0.z;
                if (current_outlier(mean[kk], sigma[kk], cur, a.gamma)) alpha = fminf(alpha, a.alpha);
                if (a.reset) alpha = 1.0f;
                else if ((rej >> k) & 1u) alpha = a.rejection_alpha;
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
using TmPol = LearnedTmemPol<TAA_LEARNED_TM_NB>;

struct TmNetSmem {
    alignas(128) char w[learned::Blob::INFER_BYTES];
    uint64_t bar;
    uint32_t tmem;
};

template <int MC>
__global__ void __launch_bounds__(NT, TAA_LEARNED_TM_STRIP_MIN_BLOCKS)
    resolve_strips_learned_tm(const Args a, const __grid_constant__ CUtensorMap hmap, const int tma_ok,
                              const char* __restrict__ blob) {
    __shared__ SmemT<float4> sm;
    __shared__ TmNetSmem net;
    if (threadIdx.x == 0) mbar_init(&net.bar, 1);
    learned::copy_blob(net.w, blob, learned::Blob::INFER_BYTES);
    if (threadIdx.x < 32) tc::tmem_alloc(&net.tmem, TmPol::kCols);
    tc::fence_smem_to_async();  // the weights, written here, are read by the tensor core
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    uint32_t phase = 0;
    TmPol::Ctx ctx{net.w, &net.bar, net.tmem, 0u, true};
    strip_tile<TmPol, 2, MC, false>(a, &hmap, tma_ok, blockIdx.x, blockIdx.y, sm, phase, ctx);
    if (!ctx.ok && threadIdx.x == 0) atomicOr(a.status, kStatusWindowTimeout);
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_free(net.tmem, TmPol::kCols);
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
    if (motion_ch == 4) resolve_strips_learned_tm<4><<<grid, NT, 0, s>>>(a, map, tma_ok, blob);
    else resolve_strips_learned_tm<2><<<grid, NT, 0, s>>>(a, map, tma_ok, blob);
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
