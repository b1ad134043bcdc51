// learned.cuh - the learned history rectifier: a per-pixel MLP
// (32 features -> 32 -> 32 -> 2, ReLU) that predicts the blend weight and the
// scale of the variance clip box, run on the tensor cores (tcgen05.cuh).
//
// Features (taa.comp's own quantities, in YCoCg, normalised by the 3x3 mean
// luma): the 3x3 mean, standard deviation, minimum and maximum; the filtered
// history; the current colour; the history's deviation from the mean in
// standard deviations; velocity length; depth difference against the
// culling threshold; the rejection flag; the clip ratio of the plain box;
// log luma; the box's luma range; current minus mean; history minus current
// luma; a constant.  Outputs: alpha = sigmoid(o0), box scale s = 2^o1.  The
// rectified pixel is the variance clip of taa.comp:323-345 with the box
// mean +- s * gamma * sigma and the blend taa.comp:900 with alpha; a rejected
// pixel (taa.comp:787-823) blends with the rejection alpha as the shader does;
// a scale outside [0.5, 2] falls back to the plain variance clip and alpha; a
// current sample that is an outlier of its neighbourhood (current_outlier)
// blends with no more than the plain alpha.
#pragma once
#include <cuda_fp16.h>
#include <stddef.h>
#include <stdint.h>

#include "tcgen05.cuh"

namespace taa_dev {
namespace learned {

constexpr int kIn = 32, kHid = 32, kOut = 2, kOutPad = 16;
constexpr int kRows = 128;  // pixels per tensor-core block (the MMA's M)

// The weights as FP32 masters (row-major [out][in]), the layout of
// taa_mlp_weights_t (include/taa_gb300.h).  Unit 31 of each hidden layer is
// the constant 1 that carries the next layer's bias (input 31 is the constant
// feature): rows 31 of w1 and w2 and columns 31 of w1, w2 and w3 are not used.
struct Weights {
    float w1[kHid * kIn], b1[kHid];
    float w2[kHid * kHid], b2[kHid];
    float w3[kOut * kHid], b3[kOut];
};
constexpr int kConst = 31;

// The device blob the kernels copy into shared memory: the FP16 effective
// matrices (biases in column 31, the constant units' rows) in the canonical
// K-major layout as MMA B operands ([N rows][K columns]) for inference, then
// the transposes the backward pass multiplies by.
struct Blob {
    static constexpr int W1 = 0;                          // [32 hid][32 in]
    static constexpr int W2 = W1 + kHid * kIn * 2;        // [32 hid][32 hid]
    static constexpr int W3 = W2 + kHid * kHid * 2;       // [16 out (2 used)][32 hid]
    static constexpr int INFER_BYTES = W3 + kOutPad * kHid * 2;
    static constexpr int W3T = INFER_BYTES;               // [32 hid][16 out (2 used)]
    static constexpr int W2T = W3T + kHid * kOutPad * 2;  // [32 in of layer 2][32 out of layer 2]
    static constexpr int BYTES = W2T + kHid * kHid * 2;   // what the training kernels copy
    // the inference matrices once more as the warp network's padded row-major
    // image (WarpNetN's w1, w2, w3: [32][40], [32][40], [8][40] halves), which a
    // CTA copies in 16-byte words
    static constexpr int WARP = BYTES;
    static constexpr int WARP_BYTES = (2 * 32 + 8) * 40 * 2;
    static constexpr int ALL_BYTES = WARP + WARP_BYTES;  // the allocation
};
static_assert(Blob::BYTES % 16 == 0 && Blob::INFER_BYTES % 16 == 0 && Blob::WARP_BYTES % 16 == 0,
              "blob copied as 16-byte words");

// Features of one pixel (see the file comment).  All colours YCoCg.
struct FeatureIn {
    float mean[3], sigma[3], mn[3], mx[3], hist[3], cur[3];
    float vel_px;      // velocity length in pixels
    float depth_rel;   // (previous depth - expected depth) / (0.1 * (1 - previous depth)), 0 without culling
    bool rejected;
};

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// Fast approximate divisions and logarithm: the features only need to be the
// same in training and inference, which run this same code.
__device__ __forceinline__ void features(const FeatureIn& p, float (&f)[kIn]) {
    const float lum = fmaxf(p.mean[0], 0.f) + 0.05f;
    const float inv = __fdividef(1.0f, lum);
    float ma = 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        f[0 + c] = p.mean[c] * inv;
        f[3 + c] = p.sigma[c] * inv;
        f[6 + c] = p.mn[c] * inv;
        f[9 + c] = p.mx[c] * inv;
        f[12 + c] = p.hist[c] * inv;
        f[15 + c] = p.cur[c] * inv;
        const float dev = __fdividef(p.hist[c] - p.mean[c], p.sigma[c] + 1e-3f * lum);
        f[18 + c] = clampf(dev, -8.f, 8.f) * 0.25f;
        ma = fmaxf(ma, __fdividef(fabsf(p.hist[c] - p.mean[c]), p.sigma[c] + 1e-7f));
        f[27 + c] = (p.cur[c] - p.mean[c]) * inv;
    }
    f[21] = fminf(p.vel_px, 64.f) * (1.f / 16.f);
    f[22] = clampf(p.depth_rel, -8.f, 8.f) * 0.125f;
    f[23] = p.rejected ? 1.f : 0.f;
    f[24] = fminf(ma, 8.f) * 0.125f;
    f[25] = __log2f(fmaxf(p.mean[0], 0.f) + 1e-3f) * 0.125f;
    f[26] = (p.mx[0] - p.mn[0]) * inv;
    f[30] = (p.hist[0] - p.cur[0]) * inv;
    f[31] = 1.f;
    // every feature stays far inside the FP16 range: colours over a luma of
    // at least 0.05, clamped deviations and ratios, velocity capped at 64 px
}

// Hardware approximations (MUFU): the learned form only needs training and
// inference to agree, and both run these same functions.
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float exp2_approx(float x) {
    float r;
    asm("ex2.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
// Whether the current sample is an outlier of its own 3x3 neighbourhood in
// luma: farther from the box mean than K times the plain box's half extent
// gamma * sigma.  The centre texel is one of the nine, so at K = 2 only an
// isolated sample gets there (one bright texel among eight dark ones sits at
// 2.83 sigma); its blend weight is held to the plain variance clip's (the
// plain method judges the learned one), in inference and in the training
// loss alike.  Measured on the C5 sequence (trained in each case): without
// the cap +6.48 dB over the variance clip with a largest error of 53.5
// against its 22.6; K = 1.25 +6.63 dB, 28.1; K = 1.5 +6.39 dB, 55.3; K = 2
// +5.33 dB, 22.6.
#ifndef TAA_LEARNED_OUTLIER_K
#define TAA_LEARNED_OUTLIER_K 2.0f
#endif
__device__ __forceinline__ bool current_outlier(const float (&mean)[3], const float (&sigma)[3], const float (&cur)[3],
                                                float gamma) {
    return fabsf(cur[0] - mean[0]) > TAA_LEARNED_OUTLIER_K * gamma * sigma[0] + 1e-7f;
}
// The network's outputs turned into the blend weight and the box scale.
__device__ __forceinline__ float out_alpha(float o0) { return __fdividef(1.0f, 1.0f + __expf(-o0)); }
__device__ __forceinline__ float out_scale(float o1) { return exp2_approx(o1); }

// Variance clip towards the mean with the box mean +- e (e = s*gamma*sigma +
// 1e-7, taa.comp:323-345), then the blend (taa.comp:900).  YCoCg in and out.
__device__ __forceinline__ void rectify_blend(const float (&mean)[3], const float (&e)[3], const float (&hist)[3],
                                              const float (&cur)[3], float alpha, float (&out)[3]) {
    float d[3], ma = 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        d[c] = hist[c] - mean[c];
        ma = fmaxf(ma, fabsf(__fdividef(d[c], e[c])));
    }
    const float k = ma > 1.f ? __fdividef(1.f, ma) : 1.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float hc = mean[c] + d[c] * k;
        out[c] = hc * (1.f - alpha) + cur[c] * alpha;
    }
}

// The first `bytes` of the device blob into shared memory (16-byte words).
__device__ __forceinline__ void copy_blob(char* dst, const char* src, int bytes) {
    for (int w = threadIdx.x; w < bytes / 16; w += blockDim.x)
        reinterpret_cast<uint4*>(dst)[w] = __ldg(reinterpret_cast<const uint4*>(src) + w);
}

// Writes one pixel's 32 FP16 values as row r of a canonical [128][32] A tile.
__device__ __forceinline__ void store_row(char* tile, int r, const float (&v)[32]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        __half2 h0 = __floats2half2_rn(v[8 * j + 0], v[8 * j + 1]), h1 = __floats2half2_rn(v[8 * j + 2], v[8 * j + 3]);
        __half2 h2 = __floats2half2_rn(v[8 * j + 4], v[8 * j + 5]), h3 = __floats2half2_rn(v[8 * j + 6], v[8 * j + 7]);
        uint4 w;
        w.x = *reinterpret_cast<uint32_t*>(&h0);
        w.y = *reinterpret_cast<uint32_t*>(&h1);
        w.z = *reinterpret_cast<uint32_t*>(&h2);
        w.w = *reinterpret_cast<uint32_t*>(&h3);
        *reinterpret_cast<uint4*>(tile + tc::canon(r, 8 * j, 32)) = w;
    }
}
// Row r of a canonical [128][32] A tile from 32 FP32 accumulators, through the
// ReLU (applied to the FP16 values: rounding keeps the sign).
__device__ __forceinline__ void store_row_relu(char* tile, int r, const float (&v)[32]) {
    const __half2 zero = __float2half2_rn(0.f);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        __half2 h[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) h[q] = __hmax2(__floats2half2_rn(v[8 * j + 2 * q], v[8 * j + 2 * q + 1]), zero);
        uint4 w;
        w.x = *reinterpret_cast<uint32_t*>(&h[0]);
        w.y = *reinterpret_cast<uint32_t*>(&h[1]);
        w.z = *reinterpret_cast<uint32_t*>(&h[2]);
        w.w = *reinterpret_cast<uint32_t*>(&h[3]);
        *reinterpret_cast<uint4*>(tile + tc::canon(r, 8 * j, 32)) = w;
    }
}
// Reads row r of a canonical [128][32] FP16 tile as floats.
__device__ __forceinline__ void load_row(const char* tile, int r, float (&v)[32]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        uint4 w = *reinterpret_cast<const uint4*>(tile + tc::canon(r, 8 * j, 32));
        const uint32_t u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float2 f = __half22float2(*reinterpret_cast<const __half2*>(&u[q]));
            v[8 * j + 2 * q] = f.x;
            v[8 * j + 2 * q + 1] = f.y;
        }
    }
}

// Polls of an MMA-completion barrier before a wait gives up; each poll
// suspends the thread in hardware until the phase completes or kPollNs pass,
// so a waiting warp issues a handful of instructions, not a spin loop.
constexpr uint32_t kMmaPolls = 1u << 16;
#ifndef TAA_MMA_POLL_NS
#define TAA_MMA_POLL_NS 20000
#endif
constexpr uint32_t kPollNs = TAA_MMA_POLL_NS;
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity) {
    for (uint32_t i = 0; i < kMmaPolls; ++i) {
        uint32_t done;
        if constexpr (kPollNs > 0) {
            asm volatile(
                "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(tc::saddr(bar)), "r"(parity), "r"(kPollNs)
                : "memory");
        } else {
            asm volatile(
                "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(tc::saddr(bar)), "r"(parity)
                : "memory");
        }
        if (done) return true;
    }
    return false;
}

// All threads: make this CTA's shared-memory writes visible to the tensor
// core and order them before the MMAs one thread issues next.
__device__ __forceinline__ void sync_for_mma() {
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}
// The same for the 128 threads of one warpgroup (named barrier 1 + wg).
__device__ __forceinline__ void sync_group_for_mma(int wg) {
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    if (wg == 0) asm volatile("bar.sync 1, 128;" ::: "memory");
    else asm volatile("bar.sync 2, 128;" ::: "memory");
    tc::fence_after_sync();
}

// One dense layer for one 128-row block issued by one thread of its
// warpgroup: D = A . W^T with K = 32 (two MMAs) and N = n.  Returns false if
// the wait gave up.
__device__ __forceinline__ bool layer_block(const char* a_tile, const char* w, int n, uint32_t d_tmem, bool issuer,
                                            uint64_t* bar, uint32_t& phase) {
    if (issuer) {
        const uint32_t idesc = tc::idesc_f16(128, n);
        for (int ks = 0; ks < 2; ++ks)
            tc::mma_f16(d_tmem, tc::smem_desc(a_tile + ks * 256, 128, 512), tc::smem_desc(w + ks * 256, 128, 512),
                        idesc, ks > 0);
        tc::commit(bar);
    }
    const bool ok = wait_bar(bar, phase);
    phase ^= 1u;
    tc::fence_after_sync();
    return ok;
}

// One dense layer for `nblocks` blocks of 128 rows: D[b] = A[b] . W^T with
// K = 32 (two MMAs per block) and N = n; thread 0 issues, everyone waits.
// Returns false if the wait gave up.
__device__ __forceinline__ bool layer(char* const* a_tiles, const char* w, int n, uint32_t tmem, int nblocks,
                                      uint64_t* bar, uint32_t& phase) {
    if (threadIdx.x == 0) {
        const uint32_t idesc = tc::idesc_f16(128, n);
        for (int b = 0; b < nblocks; ++b)
            for (int ks = 0; ks < 2; ++ks)
                tc::mma_f16(tmem + (uint32_t)(b * 32), tc::smem_desc(a_tiles[b] + ks * 256, 128, 512),
                            tc::smem_desc(w + ks * 256, 128, 512), idesc, ks > 0);
        tc::commit(bar);
    }
    const bool ok = wait_bar(bar, phase);
    phase ^= 1u;
    tc::fence_after_sync();
    return ok;
}

// ---------------------------------------------------------------- the network per warp

// Inference without block barriers: each warp runs its own 32 pixels through
// the network with warp-wide MMAs (mma.sync m16n8k16, FP16 in, FP32 out).  A
// layer's accumulator fragments are, packed to FP16 after the ReLU, exactly
// the next layer's A fragments, so the activations never leave registers.
// Weights and the warp's feature rows sit in shared memory row-major with
// 80-byte rows (conflict-free ldmatrix).
constexpr int kPad = 40;  // halves per padded row
template <int NW> struct WarpNetN {
    alignas(16) __half w1[kHid][kPad];
    alignas(16) __half w2[kHid][kPad];
    alignas(16) __half w3[8][kPad];
    alignas(16) __half feat[NW][32][kPad];  // one 32-row tile per warp of the CTA
};
using WarpNet = WarpNetN<8>;  // 256-thread CTAs

// The padded row-major weights (w1, w2, w3 laid out back to back from w1)
// from the blob's image of them (all threads, then a barrier).
__device__ __forceinline__ void copy_warp_weights(__half* w1, const char* blob) {
    copy_blob(reinterpret_cast<char*>(w1), blob + Blob::WARP, Blob::WARP_BYTES);
}
template <int NW> __device__ __forceinline__ void load_warp_weights(WarpNetN<NW>& s, const char* blob) {
    static_assert(offsetof(WarpNetN<NW>, w2) == offsetof(WarpNetN<NW>, w1) + 2560 &&
                      offsetof(WarpNetN<NW>, w3) == offsetof(WarpNetN<NW>, w1) + 5120,
                  "w1, w2, w3 back to back as in the blob's image");
    copy_warp_weights(&s.w1[0][0], blob);
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(tc::saddr(p)));
}
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack_relu(float a, float b) {
    __half2 h = __hmax2(__floats2half2_rn(a, b), __float2half2_rn(0.f));
    return *reinterpret_cast<uint32_t*>(&h);
}

// One hidden layer of a 16-row m-tile: A (two k16 fragments) times W ([32][32]
// padded) -> the ReLU'd FP16 A fragments of the next layer.
__device__ __forceinline__ void warp_layer(const uint32_t (&a)[2][4], const __half (*w)[kPad], uint32_t (&h)[2][4]) {
    const int lane = threadIdx.x & 31;
    float acc[4][4];
#pragma unroll
    for (int nj = 0; nj < 4; ++nj) {
        acc[nj][0] = acc[nj][1] = acc[nj][2] = acc[nj][3] = 0.f;
        uint32_t b[4];  // (k 0-7, 8-15, 16-23, 24-31) of rows nj*8 .. nj*8+7
        ldsm_x4(b, &w[nj * 8 + (lane & 7)][(lane >> 3) * 8]);
        mma16816(acc[nj], a[0], b[0], b[1]);
        mma16816(acc[nj], a[1], b[2], b[3]);
    }
#pragma unroll
    for (int kj = 0; kj < 2; ++kj) {
        h[kj][0] = pack_relu(acc[2 * kj][0], acc[2 * kj][1]);
        h[kj][1] = pack_relu(acc[2 * kj][2], acc[2 * kj][3]);
        h[kj][2] = pack_relu(acc[2 * kj + 1][0], acc[2 * kj + 1][1]);
        h[kj][3] = pack_relu(acc[2 * kj + 1][2], acc[2 * kj + 1][3]);
    }
}

// The network on this thread's 32 features; every thread of the warp calls it.
template <int NW>
__device__ __forceinline__ void forward_warp(WarpNetN<NW>& s, const float (&f)[kIn], float& o0, float& o1) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __half* row = s.feat[warp][lane];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        __half2 q0 = __floats2half2_rn(f[8 * j + 0], f[8 * j + 1]), q1 = __floats2half2_rn(f[8 * j + 2], f[8 * j + 3]);
        __half2 q2 = __floats2half2_rn(f[8 * j + 4], f[8 * j + 5]), q3 = __floats2half2_rn(f[8 * j + 6], f[8 * j + 7]);
        uint4 w;
        w.x = *reinterpret_cast<uint32_t*>(&q0);
        w.y = *reinterpret_cast<uint32_t*>(&q1);
        w.z = *reinterpret_cast<uint32_t*>(&q2);
        w.w = *reinterpret_cast<uint32_t*>(&q3);
        *reinterpret_cast<uint4*>(row + 8 * j) = w;
    }
    __syncwarp();
    float res[2][4];
#pragma unroll
    for (int mi = 0; mi < 2; ++mi) {
        uint32_t a[2][4], h1[2][4], h2[2][4];
#pragma unroll
        for (int kj = 0; kj < 2; ++kj) ldsm_x4(a[kj], &s.feat[warp][mi * 16 + (lane & 15)][kj * 16 + (lane >> 4) * 8]);
        warp_layer(a, s.w1, h1);
        warp_layer(h1, s.w2, h2);
        float o[4] = {0.f, 0.f, 0.f, 0.f};
        uint32_t b[4];
        ldsm_x4(b, &s.w3[lane & 7][(lane >> 3) * 8]);
        mma16816(o, h2[0], b[0], b[1]);
        mma16816(o, h2[1], b[2], b[3]);
#pragma unroll
        for (int i = 0; i < 4; ++i) res[mi][i] = o[i];
    }
    __syncwarp();  // the feature rows are free for the next call
    // pixel `lane` is row lane % 16 of m-tile lane / 16: its outputs (columns 0
    // and 1) are in lane (lane % 8) * 4, registers 0-1 (rows 0-7) or 2-3 (8-15)
    const int src = (lane & 7) * 4;
    float v[2][4];
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int i = 0; i < 4; ++i) v[mi][i] = __shfl_sync(0xffffffffu, res[mi][i], src);
    const int mi = lane >> 4, hi = (lane >> 3) & 1;
    o0 = mi ? (hi ? v[1][2] : v[1][0]) : (hi ? v[0][2] : v[0][0]);
    o1 = mi ? (hi ? v[1][3] : v[1][1]) : (hi ? v[0][3] : v[0][1]);
}


}  // namespace learned
}  // namespace taa_dev
