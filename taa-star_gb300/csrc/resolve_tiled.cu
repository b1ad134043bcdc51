// resolve_tiled.cu - the latency-hiding FP32 tiled resolve (no fused sharpen).
//
// One 256-thread CTA resolves a 32x8 tile, one pixel per thread.  The work is
// ordered so that the three dependent memory round trips of a pixel overlap
// instead of following each other:
//   1. the pixel's velocity and depth are requested first;
//   2. the tile's source colour plus a 1-pixel halo is requested next (one or
//      two texels per thread);
//   3. as soon as the velocity arrives the history position and the filter
//      taps are known, and the 16 history texels (and the previous-depth
//      texel for depth culling) are requested with cp.async straight into
//      this thread's slots in shared memory - in flight without holding
//      registers;
//   4. the staged colour is converted once to the working colour space and the
//      3x3 moments / box are computed from shared memory while the history
//      gather is still in flight;
//   5. the thread waits for its own copies only and finishes the pixel.
// Arithmetic is the oracle's FP32 order (this unit is compiled with
// -fmad=false, explicit FMAs only where the oracle has them), so results are
// bit-identical to the plain form.  The benchmark's parameter mode (variance
// clip in YCoCg, clip towards the box centre, velocity for every pixel,
// simple velocity sampling, no tonemap/luma weighting/near-clamp reduction)
// is compiled as a specialisation; other modes keep runtime switches.
#include <atomic>

#include "common.cuh"
#include "kernels.h"
#include "../../include/taa_gb300.h"

namespace taa_dev {
namespace {

constexpr int TX = 32, TY = 8, NT = TX * TY;
constexpr int SX = TX + 2, SY = TY + 2;  // staged colour with halo
constexpr int NTAP = 16;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
template <int BYTES>
__device__ __forceinline__ void cp_async_ca(void* dst_smem, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(smem_addr(dst_smem)), "l"(src), "n"(BYTES)
                 : "memory");
}

// compile-time view of the parameter block: Hot = the benchmark mode
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
};

struct C3 { float x, y, z; };

__device__ __forceinline__ float4 to_working(float4 c, bool tonemap, bool ycocg) {
    if (tonemap) {
        float l = 1.0f + gmax(gmax(c.x, c.y), c.z);
        c.x = c.x / l;
        c.y = c.y / l;
        c.z = c.z / l;
    }
    if (ycocg) {
        // products by powers of two are exact: fusing rounds like the oracle's mul + add
        float y = __fmaf_rn(.25f, c.z, __fmaf_rn(.25f, c.x, .5f * c.y));
        float co = __fmaf_rn(-.5f, c.z, .5f * c.x);
        float cg = __fmaf_rn(-.25f, c.z, __fmaf_rn(-.25f, c.x, .5f * c.y));
        return make_float4(y, co, cg, 0.f);
    }
    return make_float4(c.x, c.y, c.z, 0.f);
}

// Filter taps of the history sample at (u, v): texel coordinates (already
// clamped) and weights.  Catmull-Rom: 4x4 separable taps (taa.comp:441-514 as
// the 16-tap form).  Bilinear: 2x2.  The oracle's order of operations.
struct Taps {
    int xs[4], ys[4];
    float wx[4], wy[4];
};
__device__ __forceinline__ void catmullrom_taps(float u, float v, int w, int h, Taps& t) {
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
    int kx = trunc_index(bx), ky = trunc_index(by);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        t.xs[i] = clampi(kx - 1 + i, 0, w - 1);
        t.ys[i] = clampi(ky - 1 + i, 0, h - 1);
    }
}
__device__ __forceinline__ void bilinear_taps(float u, float v, int w, int h, Taps& t) {
    float px = u * (float)w - 0.5f, py = v * (float)h - 0.5f;
    float fx0 = floorf(px), fy0 = floorf(py);
    float fx = px - fx0, fy = py - fy0;
    if (!(fx == fx)) fx = 0.f;
    if (!(fy == fy)) fy = 0.f;
    int x0 = trunc_index(fx0), y0 = trunc_index(fy0);
    t.xs[0] = clampi(x0, 0, w - 1);
    t.xs[1] = clampi(x0 + 1 < x0 ? x0 : x0 + 1, 0, w - 1);
    t.ys[0] = clampi(y0, 0, h - 1);
    t.ys[1] = clampi(y0 + 1 < y0 ? y0 : y0 + 1, 0, h - 1);
    t.wx[0] = 1.0f - fx;
    t.wx[1] = fx;
    t.wy[0] = 1.0f - fy;
    t.wy[1] = fy;
}

template <int HF, int MC, int INTERP, bool HOT>
__global__ void __launch_bounds__(NT, 3) resolve_tiled_v2(const taa_uniforms_t U, const FrameArgs a) {
    extern __shared__ float4 smem[];
    float4* s_col = smem;                          // SY x SX staged colour (working space)
    float4* s_his = smem + SY * SX;                // NTAP x NT history taps (RGBA32F) ...
    uint2* s_his16 = reinterpret_cast<uint2*>(s_his);  // ... or (RGBA16F)
    float* s_pd = reinterpret_cast<float*>(s_his + (HF == 0 ? NTAP * NT : NTAP * NT / 2));  // NT previous depths

    const taa_parameters_t& P = U.param[0];
    const Mode<HOT> M{P};
    const int tid = threadIdx.x;
    const int lx = tid % TX, ly = tid / TX;
    const int W = a.out_w, H = a.out_h;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int x = x0 + lx, y = y0 + ly;
    const bool inside = x < W && y < H;
    const int cx = min(x, W - 1), cy = min(y, H - 1);

    // 1. the pixel's own depth and velocity
    float depth = __ldg(texel_ptr<float>(a.depth, cx, cy));
    float4 vs = fetch_velocity<MC>(a.velocity, cx, cy);

    // 2. staged colour: texels tid and tid + NT of the (SX x SY) halo tile
    constexpr int NS = SX * SY;
    uint2 st0, st1 = make_uint2(0u, 0u);
    {
        int sy = tid / SX, sx = tid - sy * SX;
        st0 = __ldg(texel_ptr<uint2>(a.color, clampi(x0 - 1 + sx, 0, W - 1), clampi(y0 - 1 + sy, 0, H - 1)));
        if (tid + NT < NS) {
            int i = tid + NT;
            int sy1 = i / SX, sx1 = i - sy1 * SX;
            st1 = __ldg(texel_ptr<uint2>(a.color, clampi(x0 - 1 + sx1, 0, W - 1), clampi(y0 - 1 + sy1, 0, H - 1)));
        }
    }

    // 3. history position (taa.comp:391-438), then the gather in flight
    float u = div_const_rn((float)cx + 0.5f, (float)W, a.inv_out_w);
    float v = div_const_rn((float)cy + 0.5f, (float)H, a.inv_out_h);
    float hu, hv, ehd;
    bool can = !(M.use_velocity() == 0 || (M.use_velocity() == 1 && vs.w < 0.5f));
    if (can) {
        if (M.velocity_sample() == 2) {
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
        float cs0 = u * 2.0f - 1.0f, cs1 = v * 2.0f - 1.0f;
        const float* A = U.mInverseViewProjMatrix;
        const float* B = U.mHistoryViewProjMatrix;
        float ws[4], hs[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) ws[i] = A[i] * cs0 + A[4 + i] * cs1 + A[8 + i] * depth + A[12 + i];
#pragma unroll
        for (int i = 0; i < 4; ++i) hs[i] = B[i] * ws[0] + B[4 + i] * ws[1] + B[8 + i] * ws[2] + B[12 + i] * ws[3];
        hu = (hs[0] / hs[3]) * 0.5f + 0.5f;
        hv = (hs[1] / hs[3]) * 0.5f + 0.5f;
        ehd = hs[2] / hs[3];
    }

    Taps tp;
    const Img& hi = a.history;
    const bool have_hist = hi.p != nullptr;
    if (INTERP == 2) catmullrom_taps(hu, hv, hi.w, hi.h, tp);
    else bilinear_taps(hu, hv, hi.w, hi.h, tp);
    // b-spline mode (1): four bilinear taps at computed positions (taa.comp:517-543)
    float bs_s0[2], bs_s1[2];
    Taps bt[4];
    if (INTERP == 1) {
        float it[2] = {hu * (float)hi.w, hv * (float)hi.h};
        float inv[2] = {1.0f / (float)hi.w, 1.0f / (float)hi.h};
        float t0[2], t1[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            float tc = floorf(it[k] - 0.5f) + 0.5f;
            float f = it[k] - tc, f2 = f * f, f3 = f2 * f;
            float w0 = f2 - 0.5f * (f3 + f);
            float w1 = 1.5f * f3 - 2.5f * f2 + 1.0f;
            float w3 = 0.5f * (f3 - f2);
            float w2 = 1.0f - w0 - w1 - w3;
            bs_s0[k] = w0 + w1;
            bs_s1[k] = w2 + w3;
            t0[k] = (tc - 1.0f + w1 / (w0 + w1)) * inv[k];
            t1[k] = (tc + 1.0f + w3 / (w2 + w3)) * inv[k];
        }
        bilinear_taps(t0[0], t0[1], hi.w, hi.h, bt[0]);
        bilinear_taps(t1[0], t0[1], hi.w, hi.h, bt[1]);
        bilinear_taps(t0[0], t1[1], hi.w, hi.h, bt[2]);
        bilinear_taps(t1[0], t1[1], hi.w, hi.h, bt[3]);
    }
    if (have_hist && inside) {
        constexpr int TB = HF == 0 ? 16 : 8;
        auto issue = [&](int slot, int tx_, int ty_) {
            const char* src = hi.p + (size_t)ty_ * hi.pitch + (size_t)tx_ * TB;
            if (HF == 0) cp_async_ca<16>(&s_his[slot * NT + tid], src);
            else cp_async_ca<8>(&s_his16[slot * NT + tid], src);
        };
        if (INTERP == 2) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int i = 0; i < 4; ++i) issue(j * 4 + i, tp.xs[i], tp.ys[j]);
        } else if (INTERP == 0) {
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int i = 0; i < 2; ++i) issue(j * 2 + i, tp.xs[i], tp.ys[j]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
#pragma unroll
                for (int j = 0; j < 2; ++j)
#pragma unroll
                    for (int i = 0; i < 2; ++i) issue(k * 4 + j * 2 + i, bt[k].xs[i], bt[k].ys[j]);
        }
    }
    const bool depth_cull = P.mDepthCulling != 0;
    if (depth_cull && inside && a.history_depth.p) {
        int tx_ = clampi(trunc_index(hu * (float)a.color.w), 0, a.color.w - 1);
        int ty_ = clampi(trunc_index(hv * (float)a.color.h), 0, a.color.h - 1);
        cp_async_ca<4>(&s_pd[tid], texel_ptr<float>(a.history_depth, tx_, ty_));
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");

    // 4. working-space colour into shared memory, then the 3x3 box
    const bool tm = M.tonemap(), yc = M.ycocg();
    s_col[tid] = to_working(half4_to_float4(st0), tm, yc);
    if (tid + NT < NS) s_col[tid + NT] = to_working(half4_to_float4(st1), tm, yc);
    __syncthreads();
    if (!inside) {
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        return;
    }

    const float4* nb = &s_col[(ly + 1) * SX + lx + 1];
    const C3 c0{nb[0].x, nb[0].y, nb[0].z};
    auto ld = [&](int o) { float4 t = nb[o]; return C3{t.x, t.y, t.z}; };
    const C3 c1 = ld(-SX - 1), c2 = ld(-SX), c3 = ld(-SX + 1), c4 = ld(-1), c5 = ld(1), c6 = ld(SX - 1),
             c7 = ld(SX), c8 = ld(SX + 1);
    C3 mn, mx, ct = c0;
    if (M.variance()) {
        const float N = 9.0f, rN = 1.0f / 9.0f;
        auto m1f = [](float p0, float p1, float p2, float p3, float p4, float p5, float p6, float p7, float p8) {
            return p0 + p1 + p2 + p3 + p4 + p5 + p6 + p7 + p8;
        };
        auto m2f = [](float p0, float p1, float p2, float p3, float p4, float p5, float p6, float p7, float p8) {
            float m = __fmul_rn(p0, p0);
            m = __fmaf_rn(p1, p1, m); m = __fmaf_rn(p2, p2, m); m = __fmaf_rn(p3, p3, m);
            m = __fmaf_rn(p4, p4, m); m = __fmaf_rn(p5, p5, m); m = __fmaf_rn(p6, p6, m);
            m = __fmaf_rn(p7, p7, m); m = __fmaf_rn(p8, p8, m);
            return m;
        };
        float g = P.mVarClipGamma;
        auto box = [&](float p0, float p1, float p2, float p3, float p4, float p5, float p6, float p7, float p8,
                       float& lo, float& hi_, float& mean) {
            float m1 = m1f(p0, p1, p2, p3, p4, p5, p6, p7, p8);
            float m2 = m2f(p0, p1, p2, p3, p4, p5, p6, p7, p8);
            mean = div_const_rn(m1, N, rN);
            float var = __fmaf_rn(-mean, mean, div_const_rn(m2, N, rN));
            float s = g * sqrtf(gmax(0.f, var));
            lo = mean - s;
            hi_ = mean + s;
        };
        box(c0.x, c1.x, c2.x, c3.x, c4.x, c5.x, c6.x, c7.x, c8.x, mn.x, mx.x, ct.x);
        box(c0.y, c1.y, c2.y, c3.y, c4.y, c5.y, c6.y, c7.y, c8.y, mn.y, mx.y, ct.y);
        box(c0.z, c1.z, c2.z, c3.z, c4.z, c5.z, c6.z, c7.z, c8.z, mn.z, mx.z, ct.z);
    } else {
        auto mn9 = [](float a0, float a1, float a2, float a3, float a4, float a5, float a6, float a7, float a8) {
            return gmin(gmin(gmin(gmin(gmin(gmin(gmin(gmin(a0, a1), a2), a3), a4), a5), a6), a7), a8);
        };
        auto mx9 = [](float a0, float a1, float a2, float a3, float a4, float a5, float a6, float a7, float a8) {
            return gmax(gmax(gmax(gmax(gmax(gmax(gmax(gmax(a0, a1), a2), a3), a4), a5), a6), a7), a8);
        };
        mn = {mn9(c0.x, c1.x, c2.x, c3.x, c4.x, c5.x, c6.x, c7.x, c8.x), mn9(c0.y, c1.y, c2.y, c3.y, c4.y, c5.y, c6.y, c7.y, c8.y),
              mn9(c0.z, c1.z, c2.z, c3.z, c4.z, c5.z, c6.z, c7.z, c8.z)};
        mx = {mx9(c0.x, c1.x, c2.x, c3.x, c4.x, c5.x, c6.x, c7.x, c8.x), mx9(c0.y, c1.y, c2.y, c3.y, c4.y, c5.y, c6.y, c7.y, c8.y),
              mx9(c0.z, c1.z, c2.z, c3.z, c4.z, c5.z, c6.z, c7.z, c8.z)};
        if (M.shaped()) {
            auto mn5 = [](float a0, float a2, float a4, float a5, float a7) { return gmin(gmin(gmin(gmin(a0, a2), a4), a5), a7); };
            auto mx5 = [](float a0, float a2, float a4, float a5, float a7) { return gmax(gmax(gmax(gmax(a0, a2), a4), a5), a7); };
            mn = {(mn.x + mn5(c0.x, c2.x, c4.x, c5.x, c7.x)) * 0.5f, (mn.y + mn5(c0.y, c2.y, c4.y, c5.y, c7.y)) * 0.5f,
                  (mn.z + mn5(c0.z, c2.z, c4.z, c5.z, c7.z)) * 0.5f};
            mx = {(mx.x + mx5(c0.x, c2.x, c4.x, c5.x, c7.x)) * 0.5f, (mx.y + mx5(c0.y, c2.y, c4.y, c5.y, c7.y)) * 0.5f,
                  (mx.z + mx5(c0.z, c2.z, c4.z, c5.z, c7.z)) * 0.5f};
        }
    }
    if (M.shrink()) {
        C3 hs{0.5f * (mx.x - mn.x), 0.25f * (mx.y - mn.y), 0.25f * (mx.z - mn.z)};
        C3 ce{(mn.x + mx.x) * 0.5f, (mn.y + mx.y) * 0.5f, (mn.z + mx.z) * 0.5f};
        mn = {ce.x - hs.x, ce.y - hs.y, ce.z - hs.z};
        mx = {ce.x + hs.x, ce.y + hs.y, ce.z + hs.z};
        if (ct.x < mn.x || ct.y < mn.y || ct.z < mn.z || ct.x > mx.x || ct.y > mx.y || ct.z > mx.z) ct = ce;
    }

    // 5. the history gather has landed in this thread's slots
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    auto tap = [&](int slot) -> float4 {
        if (HF == 0) return s_his[slot * NT + tid];
        return half4_to_float4(s_his16[slot * NT + tid]);
    };
    float4 hraw = make_float4(0.f, 0.f, 0.f, 0.f);
    if (have_hist) {
        if (INTERP == 2) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float rx = 0.f, ry = 0.f, rz = 0.f;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    float4 s = tap(j * 4 + i);
                    rx = __fmaf_rn(tp.wx[i], s.x, rx);
                    ry = __fmaf_rn(tp.wx[i], s.y, ry);
                    rz = __fmaf_rn(tp.wx[i], s.z, rz);
                }
                hraw.x = __fmaf_rn(tp.wy[j], rx, hraw.x);
                hraw.y = __fmaf_rn(tp.wy[j], ry, hraw.y);
                hraw.z = __fmaf_rn(tp.wy[j], rz, hraw.z);
            }
        } else {
            auto bil = [&](int base, const Taps& t) {
                float4 A = tap(base + 0), B = tap(base + 1), C = tap(base + 2), D = tap(base + 3);
                float gx = t.wx[0], fx = t.wx[1], gy = t.wy[0], fy = t.wy[1];
                float4 tt = make_float4(A.x * gx + B.x * fx, A.y * gx + B.y * fx, A.z * gx + B.z * fx, 0.f);
                float4 bb = make_float4(C.x * gx + D.x * fx, C.y * gx + D.y * fx, C.z * gx + D.z * fx, 0.f);
                return make_float4(tt.x * gy + bb.x * fy, tt.y * gy + bb.y * fy, tt.z * gy + bb.z * fy, 0.f);
            };
            if (INTERP == 0) {
                hraw = bil(0, tp);
            } else {
                float4 A = bil(0, bt[0]), B = bil(4, bt[1]), C = bil(8, bt[2]), D = bil(12, bt[3]);
                hraw = make_float4((A.x * bs_s0[0] + B.x * bs_s1[0]) * bs_s0[1] + (C.x * bs_s0[0] + D.x * bs_s1[0]) * bs_s1[1],
                                   (A.y * bs_s0[0] + B.y * bs_s1[0]) * bs_s0[1] + (C.y * bs_s0[0] + D.y * bs_s1[0]) * bs_s1[1],
                                   (A.z * bs_s0[0] + B.z * bs_s1[0]) * bs_s0[1] + (C.z * bs_s0[0] + D.z * bs_s1[0]) * bs_s1[1],
                                   0.f);
            }
        }
    }
    C3 hc{hraw.x, hraw.y, hraw.z};
    if (yc)
        hc = {.25f * hraw.x + .5f * hraw.y + .25f * hraw.z, .5f * hraw.x - .5f * hraw.z,
              -.25f * hraw.x + .5f * hraw.y - .25f * hraw.z};

    bool rejected = false;
    if (P.mRejectOutside && (hu < 0.f || hv < 0.f || hu >= 1.f || hv >= 1.f)) rejected = true;
    if (depth_cull) {
        float hd = a.history_depth.p ? s_pd[tid] : 0.f;
        if (fabsf(hd - ehd) > 0.1f * (1.0f - hd)) rejected = true;
    }

    const C3 orig = hc;
    switch (M.clip()) {
        case 1:
            hc = {gmin(gmax(hc.x, mn.x), mx.x), gmin(gmax(hc.y, mn.y), mx.y), gmin(gmax(hc.z, mn.z), mx.z)};
            break;
        case 2: {
            C3 p{0.5f * (mx.x + mn.x), 0.5f * (mx.y + mn.y), 0.5f * (mx.z + mn.z)};
            C3 e{0.5f * (mx.x - mn.x) + 1e-7f, 0.5f * (mx.y - mn.y) + 1e-7f, 0.5f * (mx.z - mn.z) + 1e-7f};
            C3 d{hc.x - p.x, hc.y - p.y, hc.z - p.z};
            float ma = gmax(fabsf(d.x / e.x), gmax(fabsf(d.y / e.y), fabsf(d.z / e.z)));
            if (ma > 1.0f) hc = {p.x + d.x / ma, p.y + d.y / ma, p.z + d.z / ma};
            break;
        }
        case 3: {
            C3 r{hc.x - ct.x, hc.y - ct.y, hc.z - ct.z};
            C3 rmax{mx.x - ct.x, mx.y - ct.y, mx.z - ct.z}, rmin{mn.x - ct.x, mn.y - ct.y, mn.z - ct.z};
            const float eps = 1e-7f;
            auto sc = [&](float s) { r = {r.x * s, r.y * s, r.z * s}; };
            if (r.x > rmax.x + eps) sc(rmax.x / r.x);
            if (r.y > rmax.y + eps) sc(rmax.y / r.y);
            if (r.z > rmax.z + eps) sc(rmax.z / r.z);
            if (r.x < rmin.x - eps) sc(rmin.x / r.x);
            if (r.y < rmin.y - eps) sc(rmin.y / r.y);
            if (r.z < rmin.z - eps) sc(rmin.z / r.z);
            hc = {ct.x + r.x, ct.y + r.y, ct.z + r.z};
            break;
        }
        default: break;
    }

    float alpha = P.mAlpha;
    if (rejected) {
        alpha = P.mRejectionAlpha;
    } else {
        if (M.vel_alpha()) {
            float du = u - hu, dv = v - hv;
            float t = gclamp(sqrtf(du * du + dv * dv) * P.mVelBasedAlphaFactor, 0.f, 1.f);
            alpha = gmax(alpha, alpha * (1.0f - t) + P.mVelBasedAlphaMax * t);
        }
        auto lum = [&](C3 c) { return yc ? c.x : .25f * c.x + .5f * c.y + .25f * c.z; };
        if (M.lottes()) {
            float lc = lum(c0), lh = lum(hc);
            float w = 1.0f - fabsf(lc - lh) / gmax(gmax(lc, lh), 0.2f);
            float ww = w * w;
            alpha = P.mMaxAlpha * (1.0f - ww) + P.mMinAlpha * ww;
        }
        if (M.near_clamp()) {
            float lmn = lum(mn), lmx = lum(mx), lh = lum(orig);
            float dist = 2.0f * fabsf(gmin(lh - lmn, lmx - lh)) / (lmx - lmn);
            if (lmx - lmn < 0.001f) dist = 1.0f;
            alpha = alpha * gclamp(4.0f * dist, 0.f, 1.f);
        }
    }
    if (U.mResetHistory) alpha = 1.0f;
    float t = 1.0f - alpha;
    C3 o{hc.x * t + c0.x * alpha, hc.y * t + c0.y * alpha, hc.z * t + c0.z * alpha};
    if (yc) {
        float tmp = o.x - o.z;
        o = {tmp + o.y, o.x + o.z, tmp - o.y};
    }
    store_history<HF>(a.history_out, x, y, make_float4(o.x, o.y, o.z, 0.f));
    if (a.result.p) {
        if (tm) {
            float l = 1.0f - gmax(gmax(o.x, o.y), o.z);
            o = {o.x / l, o.y / l, o.z / l};
        }
        store_rgba16f(a.result, x, y, make_float4(o.x, o.y, o.z, 1.0f));
    }
}

template <int HF, int MC, int INTERP, bool HOT>
cudaError_t launch_v2(const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    constexpr size_t hist_bytes = HF == 0 ? NTAP * NT * 16 : NTAP * NT * 8;
    constexpr size_t smem = SY * SX * 16 + hist_bytes + NT * 4;
    // the dynamic shared-memory opt-in is per device; remember it per device id
    static std::atomic<unsigned long long> configured{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(configured.load(std::memory_order_relaxed) & bit)) {
        e = cudaFuncSetAttribute(resolve_tiled_v2<HF, MC, INTERP, HOT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return e;
        configured.fetch_or(bit, std::memory_order_relaxed);
    }
    dim3 grid((a.out_w + TX - 1) / TX, (a.out_h + TY - 1) / TY);
    resolve_tiled_v2<HF, MC, INTERP, HOT><<<grid, NT, smem, s>>>(U, a);
    return cudaGetLastError();
}

bool is_hot(const taa_parameters_t& P) {
    return P.mUseYCoCg && !P.mToneMapLumaKaris && P.mVarianceClipping && !P.mShrinkChromaAxis &&
           P.mColorClampingOrClipping == 2 && P.mUseVelocityVectors == 2 && P.mVelocitySampleMode == 0 &&
           !P.mVelBasedAlpha && !P.mLumaWeightingLottes && !P.mReduceBlendNearClamp;
}

template <int HF, int MC, int INTERP>
cudaError_t pick_hot(const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    return is_hot(U.param[0]) ? launch_v2<HF, MC, INTERP, true>(U, a, s) : launch_v2<HF, MC, INTERP, false>(U, a, s);
}
template <int HF, int MC>
cudaError_t pick_interp(int interp, const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    switch (interp) {
        case 0: return pick_hot<HF, MC, 0>(U, a, s);
        case 1: return pick_hot<HF, MC, 1>(U, a, s);
        default: return pick_hot<HF, MC, 2>(U, a, s);
    }
}

}  // namespace

cudaError_t launch_resolve_tiled(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U,
                                 const FrameArgs& a, cudaStream_t s) {
    if (history_fmt == 0)
        return motion_ch == 4 ? pick_interp<0, 4>(interp, U, a, s) : pick_interp<0, 2>(interp, U, a, s);
    return motion_ch == 4 ? pick_interp<1, 4>(interp, U, a, s) : pick_interp<1, 2>(interp, U, a, s);
}

}  // namespace taa_dev
