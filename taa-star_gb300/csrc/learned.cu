// learned.cu - kernels of the learned history rectifier (learned.cuh):
//   * resolve_learned: the tiled resolve whose rectification and blend come
//     from the MLP, run on the tensor cores for each 128-pixel half of a tile;
//     in collection mode it resolves with the plain variance clip instead and
//     writes training records (features, the quantities the blend needs, the
//     supersampled ground truth) for a hashed sample of pixels;
//   * mlp_forward: the network alone on given features (for tests);
//   * mlp_train: forward, loss and backward over records, weight gradients
//     accumulated in tensor memory across a CTA's tiles;
//   * mlp_adam: the Adam update of the FP32 master weights and the rebuild of
//     the FP16 blob the other kernels read.
// Compiled with -fmad=false like the other units that share policy_f32.cuh.
#include "kernels.h"
#include "learned.cuh"
#include "policy_f32.cuh"

namespace taa_dev {
namespace learned {

using tiled::C3;
using tiled::Mode;

// A training record: one pixel of a collected frame.
struct __align__(16) Record {
    __half f[kIn];                        // the features as the network reads them
    float mean[3], sigma[3], hist[3], cur[3];  // YCoCg
    float gt[3];                          // RGB, 64-spp ground truth
    float gamma, alpha_fixed;             // mVarClipGamma; blend weight when the network does not choose it
    uint32_t flags;                       // 1: alpha is fixed (rejected or reset)
    uint32_t key[2];                      // collection call, pixel index: the canonical order of the records
};
static_assert(sizeof(Record) == 144, "record layout");

// ---------------------------------------------------------------- the policy

// The box the features need: mean and standard deviation (the shader's
// variance box, taa.comp:266-277, as the exact FP32 form computes it) and the
// 3x3 minimum and maximum.
struct LearnedPol : tiled::ExactF32 {
    struct Box {
        C3 mean, sigma, mn, mx;
    };
    static __device__ __forceinline__ C3 centre(const Box&, const float4* staged_centre) {
        const float4 t = *staged_centre;
        return C3{t.x, t.y, t.z};
    }
    static constexpr bool kExactCentre = false;
    static __device__ __forceinline__ void centre_colour(Box&, const Img&, int, int, bool, bool) {}

    template <bool HOT>
    static __device__ __forceinline__ void box(const float4* nb, int ns, const Mode<HOT>&, float, Box& b, f2 z) {
        const int off[9] = {0, -ns - 1, -ns, -ns + 1, -1, 1, ns - 1, ns, ns + 1};
        f2 pa, pb, m1a, m1b, m2a, m2b;
        load_pairs(&nb[0], m1a, m1b);
        m2a = mul2(m1a, m1a, z);
        m2b = mul2(m1b, m1b, z);
        C3 mn{f2lo(m1a), f2hi(m1a), f2lo(m1b)}, mx = mn;
#pragma unroll
        for (int k = 1; k < 9; ++k) {
            load_pairs(&nb[off[k]], pa, pb);
            m1a = add2(m1a, pa);
            m1b = add2(m1b, pb);
            m2a = fma2(pa, pa, m2a);
            m2b = fma2(pb, pb, m2b);
            mn = {fminf(mn.x, f2lo(pa)), fminf(mn.y, f2hi(pa)), fminf(mn.z, f2lo(pb))};
            mx = {fmaxf(mx.x, f2lo(pa)), fmaxf(mx.y, f2hi(pa)), fmaxf(mx.z, f2lo(pb))};
        }
        // the learned form needs no rounding parity: products by 1/9 and a hardware square root
        const f2 rN = dup(1.0f / 9.0f);
        const f2 mean_a = mul2(m1a, rN, z), mean_b = mul2(m1b, rN, z);
        const f2 var_a = fma2(neg2(mean_a), mean_a, mul2(m2a, rN, z));
        const f2 var_b = fma2(neg2(mean_b), mean_b, mul2(m2b, rN, z));
        b.mean = {f2lo(mean_a), f2hi(mean_a), f2lo(mean_b)};
        b.sigma = {sqrt_approx(fmaxf(0.f, f2lo(var_a))), sqrt_approx(fmaxf(0.f, f2hi(var_a))),
                   sqrt_approx(fmaxf(0.f, f2lo(var_b)))};
        b.mn = mn;
        b.mx = mx;
    }
};

// ---------------------------------------------------------------- shared memory

// A CTA's network state: NB activation tiles for each of its two 128-row
// blocks (2: features and layer 2 share one, layer 1 the other; 3: the
// training pass keeps both layers), the weights (the first BLOB bytes of the
// blob), the barrier of the MMAs and the TMEM base.
template <int NB, int BLOB> struct NetSmem {
    alignas(128) char a[NB][2][kRows * kIn * 2];
    alignas(128) char blob[BLOB];
    uint64_t bar;      // MMA completion, whole-CTA forward and training
    uint64_t bar_wg[2];  // MMA completion of each warpgroup's block (inference)
    uint32_t tmem;
};
using InferSmem = NetSmem<2, Blob::INFER_BYTES>;


// The network on the features in a[0][*]; thread t (block t / 128, row t % 128)
// ends with its outputs.  All threads of the CTA call it.  False if a wait
// gave up (the outputs are then meaningless).
// Inference: each warpgroup runs the network on its own 128-row block, with
// its own barrier and MMA-issuing thread, so the two halves of a tile do not
// wait for each other.
template <int NB, int BLOB>
__device__ __forceinline__ bool forward_group(NetSmem<NB, BLOB>& s, uint32_t& phase, float& o0, float& o1) {
    const int wg = threadIdx.x >> 7, row = threadIdx.x & 127;
    const bool issuer = row == 0;
    const uint32_t cols = s.tmem + (uint32_t)(wg * 32);
    const uint32_t lane_cols = cols + ((uint32_t)((threadIdx.x >> 5) & 3) * 32u << 16);
    constexpr int L2 = NB == 2 ? 0 : 2;
    uint64_t* bar = &s.bar_wg[wg];
    bool ok = true;
    float acc[32];
    sync_group_for_mma(wg);
    ok &= layer_block(s.a[0][wg], s.blob + Blob::W1, kHid, cols, issuer, bar, phase);
    tc::ld32(lane_cols, acc);
    store_row_relu(s.a[1][wg], row, acc);
    sync_group_for_mma(wg);
    ok &= layer_block(s.a[1][wg], s.blob + Blob::W2, kHid, cols, issuer, bar, phase);
    tc::ld32(lane_cols, acc);
    store_row_relu(s.a[L2][wg], row, acc);
    sync_group_for_mma(wg);
    ok &= layer_block(s.a[L2][wg], s.blob + Blob::W3, kOutPad, cols, issuer, bar, phase);
    float o[16];
    tc::ld16(lane_cols, o);
    o0 = o[0];
    o1 = o[1];
    tc::fence_before_sync();
    return ok;
}

// The biases ride in column 31 of each matrix (input 31 and hidden unit 31
// are the constant 1), so a layer is the MMA and the ReLU of its FP16 output.
template <int NB, int BLOB>
__device__ __forceinline__ bool forward(NetSmem<NB, BLOB>& s, int nblocks, uint32_t& phase, float& o0, float& o1) {
    const int blk = threadIdx.x >> 7, row = threadIdx.x & 127;
    const uint32_t lane_cols = s.tmem + ((uint32_t)((threadIdx.x >> 5) & 3) * 32u << 16) + (uint32_t)(blk * 32);
    constexpr int L2 = NB == 2 ? 0 : 2;  // where layer 2's activations go
    char* t0[2] = {s.a[0][0], s.a[0][1]};
    char* t1[2] = {s.a[1][0], s.a[1][1]};
    char* t2[2] = {s.a[L2][0], s.a[L2][1]};
    bool ok = true;
    float acc[32];
    sync_for_mma();
    ok &= layer(t0, s.blob + Blob::W1, kHid, s.tmem, nblocks, &s.bar, phase);
    tc::ld32(lane_cols, acc);
    store_row_relu(s.a[1][blk], row, acc);
    sync_for_mma();
    ok &= layer(t1, s.blob + Blob::W2, kHid, s.tmem, nblocks, &s.bar, phase);
    tc::ld32(lane_cols, acc);
    store_row_relu(s.a[L2][blk], row, acc);
    sync_for_mma();
    ok &= layer(t2, s.blob + Blob::W3, kOutPad, s.tmem, nblocks, &s.bar, phase);
    float o[16];
    tc::ld16(lane_cols, o);
    o0 = o[0];
    o1 = o[1];
    tc::fence_before_sync();
    return ok;
}

// ---------------------------------------------------------------- warp-level network

// ---------------------------------------------------------------- the finisher

// Records are written for pixels whose hash falls below `sample_below`.
__device__ __forceinline__ uint32_t pixel_hash(uint32_t seed, int x, int y) {
    uint32_t h = seed ^ (uint32_t)x * 0x9E3779B1u ^ (uint32_t)y * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}

struct CollectArgs {
    Record* records;
    uint32_t* count;
    uint32_t capacity;
    uint32_t seed;
    uint32_t call;           // the trainer's count of collections before this one
    uint32_t sample_below;   // hash threshold: fraction * 2^32
    Img truth;               // RGBA32F ground truth
};

// COLLECT: resolve with the plain variance clip and write records; else the
// network on the tensor cores, per warpgroup through TMEM (TC) or per warp
// with warp-wide MMAs.
template <bool COLLECT, bool TC> struct LearnedFinish {
    InferSmem* net;
    WarpNet* wnet;
    uint32_t phase;
    CollectArgs col;

    template <class Pol, int HF, bool HOT>
    __device__ __forceinline__ static void run(const taa_uniforms_t& U, const FrameArgs& a, const taa_parameters_t& P,
                                               const Mode<HOT>&, const typename Pol::Box& box, const C3& c0,
                                               float4 hraw, float u, float v, float hu, float hv, float ehd,
                                               float prev_depth, bool rejected, bool valid, int x, int y, bool,
                                               LearnedFinish& self) {
        const float hist[3] = {.25f * hraw.x + .5f * hraw.y + .25f * hraw.z, .5f * hraw.x - .5f * hraw.z,
                               -.25f * hraw.x + .5f * hraw.y - .25f * hraw.z};
        const float mean[3] = {box.mean.x, box.mean.y, box.mean.z};
        const float sigma[3] = {box.sigma.x, box.sigma.y, box.sigma.z};
        const float cur[3] = {c0.x, c0.y, c0.z};
        const float g = P.mVarClipGamma;
        const bool fixed_alpha = rejected || U.mResetHistory;
        const float alpha_fixed = U.mResetHistory ? 1.f : (rejected ? P.mRejectionAlpha : P.mAlpha);

        FeatureIn fi;
        for (int c = 0; c < 3; ++c) {
            fi.mean[c] = mean[c];
            fi.sigma[c] = sigma[c];
            fi.hist[c] = hist[c];
            fi.cur[c] = cur[c];
        }
        fi.mn[0] = box.mn.x; fi.mn[1] = box.mn.y; fi.mn[2] = box.mn.z;
        fi.mx[0] = box.mx.x; fi.mx[1] = box.mx.y; fi.mx[2] = box.mx.z;
        const float du = (u - hu) * (float)a.out_w, dv = (v - hv) * (float)a.out_h;
        fi.vel_px = sqrt_approx(du * du + dv * dv);
        fi.depth_rel = P.mDepthCulling ? __fdividef(prev_depth - ehd, 0.1f * (1.0f - prev_depth) + 1e-6f) : 0.f;
        fi.rejected = rejected;
        float f[kIn];
        if (valid) {
            features(fi, f);
        } else {
#pragma unroll
            for (int i = 0; i < kIn; ++i) f[i] = 0.f;
        }

        float alpha, scale;
        if (COLLECT) {
            // the plain variance clip resolves; the sampled pixels become records
            alpha = fixed_alpha ? alpha_fixed : P.mAlpha;
            scale = 1.f;
            if (valid && pixel_hash(self.col.seed, x, y) < self.col.sample_below) {
                const uint32_t i = atomicAdd(self.col.count, 1u);
                if (i < self.col.capacity) {
                    Record& r = self.col.records[i];
                    for (int k = 0; k < kIn; ++k) r.f[k] = __float2half_rn(f[k]);
                    for (int c = 0; c < 3; ++c) {
                        r.mean[c] = mean[c];
                        r.sigma[c] = sigma[c];
                        r.hist[c] = hist[c];
                        r.cur[c] = cur[c];
                    }
                    const float4 gt = __ldg(texel_ptr<float4>(self.col.truth, x, y));
                    r.gt[0] = gt.x;
                    r.gt[1] = gt.y;
                    r.gt[2] = gt.z;
                    r.gamma = g;
                    r.alpha_fixed = alpha_fixed;
                    r.flags = fixed_alpha ? 1u : 0u;
                    r.key[0] = self.col.call;
                    r.key[1] = (uint32_t)y * (uint32_t)a.out_w + (uint32_t)x;
                }
            }
        } else {
            float o0 = 0.f, o1 = 0.f;
            if (TC) {
                InferSmem& s = *self.net;
                store_row(s.a[0][threadIdx.x >> 7], threadIdx.x & 127, f);
                const bool ok = forward_group(s, self.phase, o0, o1);
                if (!ok && threadIdx.x == 0) atomicOr(a.status, kStatusWindowTimeout);
            } else {
                forward_warp(*self.wnet, f, o0, o1);
            }
            alpha = out_alpha(o0);
            scale = out_scale(o1);
            if (!(scale >= 0.5f && scale <= 2.0f)) {  // outside the trusted range: the plain variance clip
                scale = 1.f;
                alpha = P.mAlpha;
            }
            if (current_outlier(mean, sigma, cur, g)) alpha = fminf(alpha, P.mAlpha);
            if (fixed_alpha) alpha = alpha_fixed;
        }
        if (!valid) return;
        float e[3], o[3];
        for (int c = 0; c < 3; ++c) e[c] = scale * g * sigma[c] + 1e-7f;
        rectify_blend(mean, e, hist, cur, alpha, o);
        const float tmp = o[0] - o[2];
        const float4 rgb = make_float4(tmp + o[1], o[0] + o[2], tmp - o[1], 0.f);
        store_history<HF>(a.history_out, x, y, rgb);
        if (a.result.p) store_rgba16f(a.result, x, y, make_float4(rgb.x, rgb.y, rgb.z, 1.0f));
    }
};

// ---------------------------------------------------------------- resolve kernel

using S = tiled::DefaultShape;

// Resident CTAs per SM the learned kernels' register budget is sized for
// (the tensor-memory path needs 64 registers: 4).
#ifndef TAA_LEARNED_MIN_BLOCKS
#define TAA_LEARNED_MIN_BLOCKS 4
#endif
template <int HF, int MC, bool COLLECT, bool TC>
__global__ void __launch_bounds__(S::NT, TC ? 4 : TAA_LEARNED_MIN_BLOCKS)
    resolve_learned(const taa_uniforms_t U, const FrameArgs a, const __grid_constant__ CUtensorMap hmap,
                    const int tma_ok, const char* __restrict__ blob, const CollectArgs col) {
    __shared__ tiled::TileSmem<LearnedPol, S, HF> sm;
    extern __shared__ __align__(128) char dyn[];
    InferSmem& net = *reinterpret_cast<InferSmem*>(dyn);
    WarpNet& wnet = *reinterpret_cast<WarpNet*>(dyn);
    if (threadIdx.x == 0) {
        tiled::mbar_init(&sm.bar, 1);
        if (!COLLECT && TC) {
            tiled::mbar_init(&net.bar_wg[0], 1);
            tiled::mbar_init(&net.bar_wg[1], 1);
        }
    }
    if (!COLLECT && TC) {
        copy_blob(net.blob, blob, Blob::INFER_BYTES);
        if (threadIdx.x < 32) tc::tmem_alloc(&net.tmem, 64);
    }
    if (!COLLECT && !TC) load_warp_weights(wnet, blob);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    LearnedFinish<COLLECT, TC> fin{&net, &wnet, 0u, col};
    uint32_t phase = 0;
    tiled::tile_body<LearnedPol, S, HF, MC, 2, false, false>(U, a, &hmap, tma_ok != 0, blockIdx.x, blockIdx.y, sm,
                                                             phase, fin);
    if (!COLLECT && TC) {
        tc::fence_before_sync();
        __syncthreads();
        if (threadIdx.x < 32) tc::tmem_free(net.tmem, 64);
    }
}

// ---------------------------------------------------------------- the network alone

__global__ void __launch_bounds__(128) mlp_forward(const char* __restrict__ blob, const float* __restrict__ feat,
                                                   float* __restrict__ out, int n, unsigned int* status) {
    extern __shared__ __align__(128) char dyn[];
    InferSmem& net = *reinterpret_cast<InferSmem*>(dyn);
    if (threadIdx.x == 0) tiled::mbar_init(&net.bar, 1);
    copy_blob(net.blob, blob, Blob::INFER_BYTES);
    if (threadIdx.x < 32) tc::tmem_alloc(&net.tmem, 32);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    uint32_t phase = 0;
    for (int base = blockIdx.x * kRows; base < n; base += gridDim.x * kRows) {
        const int p = base + (int)threadIdx.x;
        float f[kIn];
        for (int i = 0; i < kIn; ++i) f[i] = p < n ? feat[(size_t)p * kIn + i] : 0.f;
        store_row(net.a[0][0], threadIdx.x, f);
        float o0, o1;
        if (!forward(net, 1, phase, o0, o1) && threadIdx.x == 0) atomicOr(status, kStatusWindowTimeout);
        if (p < n) {
            out[(size_t)p * 2] = o0;
            out[(size_t)p * 2 + 1] = o1;
        }
        __syncthreads();  // the next rows reuse the tiles
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_free(net.tmem, 32);
}

// ---------------------------------------------------------------- training

// Gradient buffer layout: the Weights struct, then the loss sum and the
// number of records that contributed.
constexpr int kParams = (int)(sizeof(Weights) / sizeof(float));
constexpr int kGradFloats = kParams + 2;

// The space the loss compares colours in: linear (TAA_MLP_LOSS 1, the space
// the PSNR against the ground truth is measured in) or compressed by
// x / (1 + |x|) (TAA_MLP_LOSS 0).
#ifndef TAA_MLP_LOSS
#define TAA_MLP_LOSS 1
#endif
__device__ __forceinline__ float tonemap_g(float x) { return TAA_MLP_LOSS ? x : x / (1.f + fabsf(x)); }
__device__ __forceinline__ float tonemap_dg(float x) {
    const float d = 1.f + fabsf(x);
    return TAA_MLP_LOSS ? 1.f : 1.f / (d * d);
}

// Loss of one record and its gradient with respect to the two outputs
// (see the C ABI's taa_mlp_gradients for the definition).
// As in inference, a box scale outside [0.5, 2] falls back to the plain
// variance clip (scale 1, the record's plain alpha) and passes no gradient;
// a penalty kPenalty * (|o1| - 1)^2 pulls such an output back into range.
constexpr float kPenalty = 1.0f;
__device__ __forceinline__ float record_loss(const Record& r, float o0, float o1, float& d0, float& d1) {
    const bool fixed_alpha = r.flags & 1u;
    const float s = out_scale(o1);
    const bool s_in = s >= 0.5f && s <= 2.0f;
    // an outlier current sample: the blend weight no more than the plain one (current_outlier)
    const bool capped = !fixed_alpha && s_in && current_outlier(r.mean, r.sigma, r.cur, r.gamma) &&
                        out_alpha(o0) > r.alpha_fixed;
    const float alpha = (fixed_alpha || !s_in || capped) ? r.alpha_fixed : out_alpha(o0);
    const float sc = s_in ? s : 1.0f;
    float e[3], dd[3], ma = 0.f;
    int k = 0;
    for (int c = 0; c < 3; ++c) {
        e[c] = sc * r.gamma * r.sigma[c] + 1e-7f;
        dd[c] = r.hist[c] - r.mean[c];
        const float q = fabsf(dd[c] / e[c]);
        if (q > ma) {
            ma = q;
            k = c;
        }
    }
    const bool clipped = ma > 1.f;
    const float kf = clipped ? 1.f / ma : 1.f;
    float hc[3], out[3];
    for (int c = 0; c < 3; ++c) {
        hc[c] = r.mean[c] + dd[c] * kf;
        out[c] = hc[c] * (1.f - alpha) + r.cur[c] * alpha;
    }
    const float tmp = out[0] - out[2];
    const float rgb[3] = {tmp + out[1], out[0] + out[2], tmp - out[1]};
    float loss = 0.f, dr[3];
    for (int c = 0; c < 3; ++c) {
        const float diff = tonemap_g(rgb[c]) - tonemap_g(r.gt[c]);
        loss += diff * diff;
        dr[c] = 2.f * diff * tonemap_dg(rgb[c]);
    }
    const float dout[3] = {dr[0] + dr[1] + dr[2], dr[0] - dr[2], -dr[0] + dr[1] - dr[2]};
    float dalpha = 0.f, dsc = 0.f;
    for (int c = 0; c < 3; ++c) {
        dalpha += dout[c] * (r.cur[c] - hc[c]);
        // hc = mean + d * e_k / |d_k| when clipped: d(hc)/d(sc) = d * gamma * sigma_k / |d_k|
        if (clipped) dsc += dout[c] * (1.f - alpha) * dd[c] * (r.gamma * r.sigma[k] / fabsf(dd[k]));
    }
    d0 = (fixed_alpha || !s_in || capped) ? 0.f : dalpha * alpha * (1.f - alpha);
    d1 = s_in ? dsc * s * 0.69314718055994531f : 0.f;
    if (!s_in) {
        const float over = fabsf(o1) - 1.f;
        loss += kPenalty * over * over;
        d1 = 2.f * kPenalty * over * (o1 > 0.f ? 1.f : -1.f);
    }
    return loss;
}

struct TrainSmem {
    NetSmem<3, Blob::BYTES> net;
    alignas(128) char g3[kRows * 16 * 2];      // dLoss/dOutputs, [128][16] (2 used)
    alignas(128) char g2[kRows * kHid * 2];    // dLoss/dH2 after the ReLU mask
    alignas(128) char at[128 * kRows * 2];     // a gradient, transposed: [128 (32 or 2 used)][128 pixels]
    alignas(128) char bt[kHid * kRows * 2];    // an activation, transposed: [32][128 pixels]
    float loss[4];   // per warp: summed in warp order, so every run adds them the same way
    float count[4];
};

// Transposed copy of one pixel's n values into a [rows][128 pixels] canonical tile.
__device__ __forceinline__ void store_col(char* tile, int p, const float* v, int n) {
    for (int o = 0; o < n; ++o) *reinterpret_cast<__half*>(tile + tc::canon(o, p, kRows)) = __float2half_rn(v[o]);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Weight gradient D += AT . BT^T over the tile's 128 pixels (8 MMAs, K = 16 each).
__device__ __forceinline__ bool weight_grad(TrainSmem& s, uint32_t cols, bool first, uint32_t& phase) {
    sync_for_mma();
    if (threadIdx.x == 0) {
        const uint32_t idesc = tc::idesc_f16(128, kHid);
        for (int ks = 0; ks < kRows / 16; ++ks)
            tc::mma_f16(s.net.tmem + cols, tc::smem_desc(s.at + ks * 256, 128, kRows * 16),
                        tc::smem_desc(s.bt + ks * 256, 128, kRows * 16), idesc, !(first && ks == 0));
        tc::commit(&s.net.bar);
    }
    const bool ok = wait_bar(&s.net.bar, phase);
    phase ^= 1u;
    tc::fence_after_sync();
    return ok;
}

__global__ void __launch_bounds__(128) mlp_train(const char* __restrict__ blob, const Record* __restrict__ recs,
                                                 const uint32_t* __restrict__ order, int first, int count,
                                                 float* __restrict__ partial, unsigned int* status) {
    extern __shared__ __align__(128) char dyn[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>(dyn);
    const int t = threadIdx.x, warp = t >> 5;
    // this CTA's slab of gradient sums: written whole, then added up over the
    // CTAs in a fixed order by mlp_sum_partials (no atomics: training repeats bit for bit)
    float* const slab = partial + (size_t)blockIdx.x * kGradFloats;
    for (int i = t; i < kGradFloats; i += 128) slab[i] = 0.f;
    if (t == 0) tiled::mbar_init(&s.net.bar, 1);
    if (t < 4) {
        s.loss[t] = 0.f;
        s.count[t] = 0.f;
    }
    copy_blob(s.net.blob, blob, Blob::BYTES);
    for (int w = t; w < (int)sizeof(s.at) / 16; w += 128) reinterpret_cast<uint4*>(s.at)[w] = make_uint4(0, 0, 0, 0);
    for (int w = t; w < (int)sizeof(s.g3) / 16; w += 128) reinterpret_cast<uint4*>(s.g3)[w] = make_uint4(0, 0, 0, 0);
    if (t < 32) tc::tmem_alloc(&s.net.tmem, 128);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t lane = (uint32_t)((warp & 3) * 32) << 16;
    uint32_t phase = 0;
    bool ok = true, first_tile = true;
    for (int base = blockIdx.x * kRows; base < count; base += gridDim.x * kRows) {
        const int p = base + t;
        const bool live = p < count;
        const Record* r = live ? &recs[order ? order[first + p] : (uint32_t)(first + p)] : nullptr;
        // forward (the layer-1 and layer-2 activations stay in net.a[1], net.a[2])
        float f[kIn];
        for (int i = 0; i < kIn; ++i) f[i] = live ? __half2float(r->f[i]) : 0.f;
        store_row(s.net.a[0][0], t, f);
        float o0 = 0.f, o1 = 0.f;
        ok &= forward(s.net, 1, phase, o0, o1);
        // loss and output gradient
        float d0 = 0.f, d1 = 0.f, loss = 0.f;
        if (live) loss = record_loss(*r, o0, o1, d0, d1);
        // the gradients travel as FP16 operands: round them the same way here
        d0 = __half2float(__float2half_rn(d0));
        d1 = __half2float(__float2half_rn(d1));
        {
            __half2 h = __floats2half2_rn(d0, d1);
            *reinterpret_cast<__half2*>(s.g3 + tc::canon(t, 0, 16)) = h;
        }
        float h2[32], h1[32], g[32];
        load_row(s.net.a[2][0], t, h2);
        load_row(s.net.a[1][0], t, h1);
        // dH2 = dO . W3 (K = 16), masked by the ReLU
        sync_for_mma();
        if (t == 0) {
            tc::mma_f16(s.net.tmem, tc::smem_desc(s.g3, 128, 256), tc::smem_desc(s.net.blob + Blob::W3T, 128, 256),
                        tc::idesc_f16(128, kHid), false);
            tc::commit(&s.net.bar);
        }
        ok &= wait_bar(&s.net.bar, phase);
        phase ^= 1u;
        tc::fence_after_sync();
        tc::ld32(s.net.tmem + lane, g);
#pragma unroll
        for (int i = 0; i < 32; ++i) g[i] = h2[i] > 0.f ? __half2float(__float2half_rn(g[i])) : 0.f;
        store_row(s.g2, t, g);
        // dW3 += dO^T . H2 and dW2 += dH2^T . H1 (transposed copies, then K = 128 pixels)
        {
            const float v3[2] = {d0, d1};
            tc::fence_before_sync();
            __syncthreads();  // the previous weight-gradient MMAs have read at and bt
            store_col(s.at, t, v3, 2);
            store_col(s.bt, t, h2, kHid);
            ok &= weight_grad(s, 32, first_tile, phase);
            store_col(s.at, t, g, kHid);
            store_col(s.bt, t, h1, kHid);
            ok &= weight_grad(s, 64, first_tile, phase);
        }
        // dH1 = dH2 . W2 (K = 32), masked by the ReLU
        {
            char* tg[1] = {s.g2};
            sync_for_mma();
            ok &= layer(tg, s.net.blob + Blob::W2T, kHid, s.net.tmem, 1, &s.net.bar, phase);
            tc::ld32(s.net.tmem + lane, g);
#pragma unroll
            for (int i = 0; i < 32; ++i) g[i] = h1[i] > 0.f ? __half2float(__float2half_rn(g[i])) : 0.f;
            tc::fence_before_sync();
            __syncthreads();
            store_col(s.at, t, g, kHid);
            store_col(s.bt, t, f, kIn);
            ok &= weight_grad(s, 96, first_tile, phase);
        }
        {
            const float l = warp_sum(loss), c = warp_sum(live ? 1.f : 0.f);
            if ((t & 31) == 0) {
                s.loss[warp] += l;
                s.count[warp] += c;
            }
        }
        first_tile = false;
        tc::fence_before_sync();
        __syncthreads();
    }
    // this CTA's weight gradients out of tensor memory (rows 0..31 are warp 0's lanes)
    __syncthreads();  // the slab's zeros are in place
    if (!first_tile && warp == 0) {
        float acc[32];
        tc::ld32(s.net.tmem + 32, acc);
        if (t < kOut)
            for (int i = 0; i < kHid; ++i) slab[offsetof(Weights, w3) / 4 + t * kHid + i] = acc[i];
        tc::ld32(s.net.tmem + 64, acc);
        for (int i = 0; i < kHid; ++i) slab[offsetof(Weights, w2) / 4 + t * kHid + i] = acc[i];
        tc::ld32(s.net.tmem + 96, acc);
        for (int i = 0; i < kIn; ++i) slab[offsetof(Weights, w1) / 4 + t * kIn + i] = acc[i];
    }
    __syncthreads();
    if (t == 0) {
        slab[kParams] = ((s.loss[0] + s.loss[1]) + s.loss[2]) + s.loss[3];
        slab[kParams + 1] = ((s.count[0] + s.count[1]) + s.count[2]) + s.count[3];
        if (!ok) atomicOr(status, kStatusWindowTimeout);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (t < 32) tc::tmem_free(s.net.tmem, 128);
}

// The effective matrices of the FP32 masters: column 31 carries the bias,
// rows 31 of layers 1 and 2 make the constant unit.
__device__ __forceinline__ float eff1(const Weights& w, int h, int x) {
    if (h == kConst) return x == kConst ? 1.f : 0.f;
    return x == kConst ? w.b1[h] : w.w1[h * kIn + x];
}
__device__ __forceinline__ float eff2(const Weights& w, int o, int x) {
    if (o == kConst) return x == kConst ? 1.f : 0.f;
    return x == kConst ? w.b2[o] : w.w2[o * kHid + x];
}
__device__ __forceinline__ float eff3(const Weights& w, int o, int x) {
    if (o >= kOut) return 0.f;
    return x == kConst ? w.b3[o] : w.w3[o * kHid + x];
}

// The FP16 blob from FP32 master weights.
__device__ __forceinline__ void build_blob(const Weights& w, char* blob, int t, int nt) {
    auto put = [&](int base, int r, int k, int K, float v) {
        *reinterpret_cast<__half*>(blob + base + tc::canon(r, k, K)) = __float2half_rn(v);
    };
    // the warp network's padded row-major image: w1, w2 [32][40], w3 [8][40]
    auto put_row = [&](int mat, int r, int k, float v) {
        *reinterpret_cast<__half*>(blob + Blob::WARP + ((mat * 32 + r) * 40 + k) * 2) = __float2half_rn(v);
    };
    for (int i = t; i < kHid * kIn; i += nt) {
        const int h = i / kIn, x = i % kIn;
        put(Blob::W1, h, x, kIn, eff1(w, h, x));
        put(Blob::W2, h, x, kHid, eff2(w, h, x));
        put(Blob::W2T, x, h, kHid, eff2(w, h, x));
        put_row(0, h, x, eff1(w, h, x));
        put_row(1, h, x, eff2(w, h, x));
    }
    for (int i = t; i < kOutPad * kHid; i += nt) {
        const int o = i / kHid, h = i % kHid;
        put(Blob::W3, o, h, kHid, eff3(w, o, h));
        put(Blob::W3T, h, o, kOutPad, eff3(w, o, h));
        if (o < 8) put_row(2, o, h, eff3(w, o, h));
    }
    // the image's padding columns (never read) written too, so the blob is fully defined
    for (int i = t; i < 72 * 8; i += nt) {
        const int r = i / 8, k = 32 + i % 8;
        *reinterpret_cast<__half*>(blob + Blob::WARP + (r * 40 + k) * 2) = __float2half_rn(0.f);
    }
}

// Gradients of the effective matrices -> gradients of the masters: column 31
// is the bias, the constant rows and the unused columns have none.
__device__ __forceinline__ void map_grads(float* g, int t, int nt) {
    Weights& G = *reinterpret_cast<Weights*>(g);
    for (int i = t; i < kHid; i += nt) {
        G.b1[i] = i == kConst ? 0.f : G.w1[i * kIn + kConst];
        G.b2[i] = i == kConst ? 0.f : G.w2[i * kHid + kConst];
    }
    for (int i = t; i < kOut; i += nt) G.b3[i] = G.w3[i * kHid + kConst];
    __syncthreads();
    for (int i = t; i < kHid; i += nt) {
        G.w1[i * kIn + kConst] = 0.f;
        G.w2[i * kHid + kConst] = 0.f;
        G.w1[kConst * kIn + i] = 0.f;
        G.w2[kConst * kHid + i] = 0.f;
    }
    for (int i = t; i < kOut; i += nt) G.w3[i * kHid + kConst] = 0.f;
    __syncthreads();
}

// grads[i] += the CTAs' slab values, added in CTA order.
__global__ void mlp_sum_partials(const float* __restrict__ partial, int nslabs, float* __restrict__ grads) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kGradFloats) return;
    float sum = 0.f;
    for (int b = 0; b < nslabs; ++b) sum += partial[(size_t)b * kGradFloats + i];
    grads[i] += sum;
}

__global__ void mlp_build_blob(const Weights* w, char* blob) { build_blob(*w, blob, threadIdx.x, blockDim.x); }
__global__ void mlp_map_grads(float* grads) { map_grads(grads, threadIdx.x, blockDim.x); }

// Adam on the FP32 masters from the summed gradients (divided by the record
// count), then the blob; the gradient buffer is cleared for the next step.
__global__ void mlp_adam(Weights* w, float* m, float* v, float* grads, int step, float lr, char* blob) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;  // lr is this step's rate (the host decays it)
    const float n = fmaxf(grads[kParams + 1], 1.f);
    float* p = reinterpret_cast<float*>(w);
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    map_grads(grads, threadIdx.x, blockDim.x);
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
        const float g = grads[i] / n;
        m[i] = b1 * m[i] + (1.f - b1) * g;
        v[i] = b2 * v[i] + (1.f - b2) * g * g;
        p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
    }
    __syncthreads();
    build_blob(*w, blob, threadIdx.x, blockDim.x);
    __syncthreads();
    for (int i = threadIdx.x; i < kGradFloats; i += blockDim.x) grads[i] = 0.f;
}

}  // namespace learned

// ---------------------------------------------------------------- launchers

using learned::Record;

size_t learned_record_bytes() { return sizeof(Record); }
int learned_param_count() { return learned::kParams; }
int learned_blob_bytes() { return learned::Blob::ALL_BYTES; }

cudaError_t launch_mlp_map_grads(float* grads, cudaStream_t s) {
    learned::mlp_map_grads<<<1, 256, 0, s>>>(grads);
    return cudaGetLastError();
}

cudaError_t launch_mlp_build_blob(const float* weights, char* blob, cudaStream_t s) {
    learned::mlp_build_blob<<<1, 256, 0, s>>>(reinterpret_cast<const learned::Weights*>(weights), blob);
    return cudaGetLastError();
}

cudaError_t launch_mlp_forward(const char* blob, const float* feat, float* out, int n, unsigned int* status,
                               cudaStream_t s) {
    const int grid = (n + learned::kRows - 1) / learned::kRows;
    const int smem = (int)sizeof(learned::InferSmem);
    cudaError_t e = cudaFuncSetAttribute(learned::mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    learned::mlp_forward<<<grid < 1 ? 1 : grid, 128, smem, s>>>(blob, feat, out, n, status);
    return cudaGetLastError();
}

int learned_grad_floats() { return learned::kGradFloats; }

cudaError_t launch_mlp_train(const char* blob, const void* records, const uint32_t* order, int first, int count,
                             float* grads, float* partial, unsigned int* status, int grid, cudaStream_t s) {
    const size_t smem = sizeof(learned::TrainSmem) + 128;
    cudaError_t e = cudaFuncSetAttribute(learned::mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    learned::mlp_train<<<grid, 128, smem, s>>>(blob, reinterpret_cast<const Record*>(records), order, first, count,
                                                partial, status);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    learned::mlp_sum_partials<<<(learned::kGradFloats + 255) / 256, 256, 0, s>>>(partial, grid, grads);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* weights, float* m, float* v, float* grads, int step, float lr, char* blob,
                            cudaStream_t s) {
    learned::mlp_adam<<<1, 1024, 0, s>>>(reinterpret_cast<learned::Weights*>(weights), m, v, grads, step, lr, blob);
    return cudaGetLastError();
}

cudaError_t launch_resolve_learned(int history_fmt, int motion_ch, bool collect, bool tcgen05, const taa_uniforms_t& U,
                                   const FrameArgs& a, const char* blob, void* records, uint32_t* count,
                                   uint32_t capacity, uint32_t seed, uint32_t call, float sample_fraction,
                                   const Img& truth,
                                   cudaStream_t s) {
    using S = learned::S;
    dim3 grid((a.out_w + S::TX - 1) / S::TX, (a.out_h + S::TY - 1) / S::TY);
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int tma_ok = a.history.p && a.history.w >= tiled::Win<S, 0>::W && a.history.h >= S::WH &&
                       history_fmt == 0 && encode_history_map(a.history, 0, tiled::Win<S, 0>::W, S::WH, &map);
    learned::CollectArgs col{reinterpret_cast<Record*>(records), count, capacity, seed, call,
                             (uint32_t)fminf(fmaxf(sample_fraction, 0.f) * 4294967040.f, 4294967040.f), truth};
    if (history_fmt != 0) return cudaErrorInvalidValue;
    const int smem = collect ? 0 : (int)(tcgen05 ? sizeof(learned::InferSmem) : sizeof(learned::WarpNet));
    auto go = [&](auto kernel) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        kernel<<<grid, S::NT, smem, s>>>(U, a, map, tma_ok, blob, col);
        return cudaGetLastError();
    };
    if (collect)
        return motion_ch == 4 ? go(learned::resolve_learned<0, 4, true, false>)
                              : go(learned::resolve_learned<0, 2, true, false>);
    if (tcgen05)
        return motion_ch == 4 ? go(learned::resolve_learned<0, 4, false, true>)
                              : go(learned::resolve_learned<0, 2, false, true>);
    return motion_ch == 4 ? go(learned::resolve_learned<0, 4, false, false>)
                          : go(learned::resolve_learned<0, 2, false, false>);
}

}  // namespace taa_dev
