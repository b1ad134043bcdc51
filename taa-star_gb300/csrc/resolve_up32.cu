// resolve_up32.cu - TAA_FORM_FAST for upsampling (TAAU: a loW x loH source
// resolved into a W x H history, taa.comp:222-257 and 740-755) on the strip
// body: 128-thread CTAs per 32x16 target tile, each thread a vertical strip
// of four target pixels.
//   1. the source texels under the tile and a 1-texel ring (at most 35 x 19
//      for any ratio >= 1) are loaded and staged as (Y, Co, Cg, Cg^2) in FP32;
//      per target pixel its source texel's depth and the source velocity
//      sampled bilinearly at its uv (taa.comp:391-438);
//   2. the target-size history window is placed and copied exactly as the
//      single-size strip body does (strip_body.cuh, steps 3-5: the reference
//      pixel's taps widened by the tile, one 2-D TMA copy on an mbarrier with
//      bounded waits, cp.async at the border, shared rows for a coherent strip);
//   3. per target pixel: the 3x3 variance box around its source texel from
//      staged row sums (a strip's pixels on one source row share it: the
//      test is the same for every lane of a warp), the jittered source sample
//      that lands in it (upsample_axis / upsampled_pick, as the exact forms,
//      the row axis once per tile row in shared memory; beta 0 when none
//      does), the clip toward the box centre, the blend
//      mix(history, current, alpha * beta).
// The arithmetic is the fast form's (contracted FMAs, hardware square root
// and reciprocal approximations): within 1e-4 relative L2 of the FP64 oracle
// and of the exact tiled form's upsampling path.
#include <cstring>

#include "strip_body.cuh"

namespace taa_dev {
namespace fast32 {

// What the upsampling kernel reads besides Args (whose W, H are the target size).
struct UpArgs {
    int loW, loH;     // source size
    float jx, jy;     // the jitter in source texels per axis (upsample_jitter)
    float scx, scy;   // target / source size per axis
};

constexpr int UMW = TX + 3, UMH = TY + 3, UNS = UMW * UMH;  // staged source texels: the tile's and a ring
constexpr int UNSPT = (UNS + NT - 1) / NT;

// Resident CTAs per SM the register budget is sized for (a tuning constant:
// 8 measured 167 us per 1080p -> 4K frame, 7 177 us, 6 183 us; staging the
// source velocity in shared memory for the bilinear taps cost an eighth CTA
// and measured 175 us).  Measured by parts (variants with a part removed,
// 170 us in all): the history filter 53 us, the landing-sample search and
// the current colour 30 us (the rows' candidates once per tile row in
// shared memory: 170 -> 166.5 us, the same bits), the bilinear velocity
// 9 us, the previous-depth gather 10 us; the rest 78 us.
#ifndef TAA_FAST_UP_MIN_BLOCKS
#define TAA_FAST_UP_MIN_BLOCKS 8
#endif

struct UpSmem {
    float4 col[UNS];                   // staged source texels (Y, Co, Cg, Cg^2), row length rw
    alignas(128) float4 win[WW * WH];  // the target-size history window
    UpAxis yaxis[TY];                  // the landing-sample candidates of the tile's target rows
    uint64_t bar;
    int org[3];
};

// The staged source texel (ix, iy) of the tile, or - never for a sample that
// lands within a texel of its target pixel, which the staged ring covers -
// the texel read and converted from global memory.
__device__ __forceinline__ float4 staged_or_global(const Args& a, const float4* col, int rw, int rh, int ix, int iy,
                                                 int gx, int gy, int loW, int loH) {
    if (ix >= 0 && iy >= 0 && ix < rw && iy < rh) return col[iy * rw + ix];
    return F32Pol::stage(__ldg(at<uint2>(a.color, a.color_pitch, clampi(gx, 0, loW - 1), clampi(gy, 0, loH - 1))));
}


template <int INTERP, int MC>
__global__ void __launch_bounds__(NT, TAA_FAST_UP_MIN_BLOCKS)
    resolve_strips_up(const Args a, const __grid_constant__ CUtensorMap hmap, const int tma_ok,
                      const __grid_constant__ UpArgs up) {
    using RawVel = typename std::conditional<MC == 4, uint2, uint32_t>::type;
    constexpr int SPAN = INTERP == 2 ? 4 : 2;
    __shared__ UpSmem sm;
    const int tid = threadIdx.x, lx = tid & 31, sy = tid >> 5;
    const int W = a.W, H = a.H, loW = up.loW, loH = up.loH;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int x = x0 + lx, cx = min(x, W - 1);
    const int ya = y0 + NPX * sy;
    const bool have_hist = a.hist != nullptr;
    // a target column's / row's source texel: int(uv * source size) with uv = (t + 0.5) / size
    auto src_x = [&](int t) { return trunc_index(div_const_rn((float)t + 0.5f, (float)W, a.inv_w) * (float)loW); };
    auto src_y = [&](int t) { return trunc_index(div_const_rn((float)t + 0.5f, (float)H, a.inv_h) * (float)loH); };
    const int rx0 = src_x(x0) - 1, ry0 = src_y(y0) - 1;
    const int rw = min(src_x(min(x0 + TX - 1, W - 1)) - rx0 + 2, UMW);
    const int rh = min(src_y(min(y0 + TY - 1, H - 1)) - ry0 + 2, UMH);

    // 1. loads: the staged source texels; per pixel its source depth and bilinear velocity
    uint2 st[UNSPT];
#pragma unroll
    for (int j = 0; j < UNSPT; ++j) {
        const int i = tid + j * NT;
        st[j] = make_uint2(0u, 0u);
        if (i < rw * rh) {
            const int ry = i / rw, rx = i - ry * rw;
            st[j] = __ldg(at<uint2>(a.color, a.color_pitch, clampi(rx0 + rx, 0, loW - 1), clampi(ry0 + ry, 0, loH - 1)));
        }
    }
    const uint32_t polls = first_wait_polls(a.status);
    PixelInfo px;
    float (&hu)[NPX] = px.hu, (&hv)[NPX] = px.hv, (&ehd)[NPX] = px.ehd, (&pd)[NPX] = px.pd;
    int srow[NPX];
    const int scol = src_x(cx);
    px.u = div_const_rn((float)cx + 0.5f, (float)W, a.inv_w);
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        const int cy = min(ya + k, H - 1);
        px.v[k] = div_const_rn((float)cy + 0.5f, (float)H, a.inv_h);
        srow[k] = src_y(cy);
        const float depth = __ldg(at<float>(a.depth, a.depth_pitch, scol, srow[k]));
        const float4 vel = bilinear_uv(loW, loH, px.u, px.v[k], [&](int xx, int yy) {
            return tiled::velocity_of<MC>(__ldg(at<RawVel>(a.vel, a.vel_pitch, xx, yy)));
        });
        hu[k] = px.u - vel.x;
        hv[k] = px.v[k] - vel.y;
        ehd[k] = depth - vel.z;
        pd[k] = 0.f;
        if (a.depth_cull && a.hdepth)
            pd[k] = __ldg(at<float>(a.hdepth, a.hdepth_pitch, clampi(trunc_index(hu[k] * (float)loW), 0, loW - 1),
                                    clampi(trunc_index(hv[k] * (float)loH), 0, loH - 1)));
    }
    // 2. the history window (the single-size strip body's steps 3-5)
    if (tid == REF_TID && have_hist) {
        float f;
        const int rux = axis_first<INTERP>(__fmul_rn(hu[0], (float)W), f);
        const int ruy = axis_first<INTERP>(__fmul_rn(hv[0], (float)H), f);
        const int wx0 = rux - (cx - x0) - MARGIN, wy0 = ruy - (min(ya, H - 1) - y0) - MARGIN;
        const bool interior = wx0 >= 0 && wy0 >= 0 && wx0 <= W - WW && wy0 <= H - WH;
        const int mode = tma_ok && interior ? 1 : 2;
        sm.org[0] = wx0;
        sm.org[1] = wy0;
        sm.org[2] = mode;
        if (mode == 1) {
            mbar_init(&sm.bar, 1);
            mbar_expect_tx(&sm.bar, (uint32_t)(sizeof(float4) * WW * WH));
            tiled::tma_load_2d(sm.win, &hmap, 4 * wx0, wy0, &sm.bar);
        }
    }
#pragma unroll
    for (int j = 0; j < UNSPT; ++j) {
        const int i = tid + j * NT;
        if (i < rw * rh) sm.col[i] = F32Pol::stage(st[j]);
    }
    // the tile's rows' landing-sample candidates, once per row (the shader's arithmetic per axis)
    if (tid < TY) sm.yaxis[tid] = upsample_axis(min(y0 + tid, H - 1), H, loH, up.jy, up.scy);
    __syncthreads();
    int wx0 = 0, wy0 = 0, mode = 0;
    if (have_hist) {
        wx0 = sm.org[0];
        wy0 = sm.org[1];
        mode = sm.org[2];
    }
    if (mode == 2) {
        const int warp = tid >> 5;
        for (int r = warp; r < WH; r += NT / 32) {
            const int gy = clampi(wy0 + r, 0, H - 1);
            for (int c = lx; c < WW; c += 32)
                cp_async<16>(&sm.win[r * WW + c], at<float4>(a.hist, a.hist_pitch, clampi(wx0 + c, 0, W - 1), gy));
        }
        cp_async_commit();
    }
    unsigned rej = 0;
#pragma unroll
    for (int k = 0; k < NPX; ++k)
        if ((a.reject_outside && (hu[k] < 0.f || hv[k] < 0.f || hu[k] >= 1.f || hv[k] >= 1.f)) ||
            (a.depth_cull && fabsf(pd[k] - ehd[k]) > 0.1f * (1.0f - pd[k])))
            rej |= 1u << k;
    bool landed = true;
    if (mode == 1) {
        landed = mbar_wait_bounded(&sm.bar, 0u, polls);
        if (!landed) {
            atomicOr(a.status, kStatusWindowTimeout);
            mbar_wait_bounded(&sm.bar, 0u);  // the copy may still land in this CTA's memory
        }
    } else if (mode == 2) {
        cp_async_wait_all();
        __syncthreads();
    }
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
        coherent = coherent && (unsigned)bx <= (unsigned)(WW - SPAN) && (unsigned)by <= (unsigned)(WH - SPAN - NPX + 1);
        if (coherent) {
            float wx[4], wy[NPX][4];
            axis_weights<INTERP>(fx, wx);
#pragma unroll
            for (int k = 0; k < NPX; ++k) axis_weights<INTERP>(fy[k], wy[k]);
            const float4* wp = &sm.win[by * WW + bx];
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
                    const float4 t = lds128(&wp[j * WW + i]);
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
                if ((unsigned)tbx <= (unsigned)(WW - SPAN) && (unsigned)tby <= (unsigned)(WH - SPAN)) {
                    const float4* wp = &sm.win[tby * WW + tbx];
                    h[k] = filter<SPAN>(t, [&](int i, int j) { return lds128(&wp[j * WW + i]); });
                } else {
                    h[k] = filter<SPAN>(t, [&](int i, int j) {
                        return __ldg(at<float4>(a.hist, a.hist_pitch, clampi(t.ux + i, 0, W - 1),
                                                clampi(t.uy + j, 0, H - 1)));
                    });
                }
            }
        }
    }
    // 3. per pixel: box, the landing source sample, clip, blend, stores
    const UpAxis uxa = upsample_axis(cx, W, loW, up.jx, up.scx);
    Box b{};
    int box_row = -1;
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        const int y = ya + k;
        if (srow[k] != box_row) {  // the same for every lane of the warp (one target row)
            box_row = srow[k];
            const float4* sp = &sm.col[(srow[k] - ry0 - 1) * rw + (scol - rx0 - 1)];
            const Row s = add(add(row_sums(sp), row_sums(sp + rw)), row_sums(sp + 2 * rw));
            b = box_of(s, a.gamma);
        }
        if (!(x < W && y < H && landed)) continue;
        int fxs, fys;
        float cur[3] = {0.f, 0.f, 0.f};
        float beta = 0.f;
        if (upsampled_pick(uxa, sm.yaxis[y - y0], fxs, fys)) {
            beta = 1.f;
            const float4 c = staged_or_global(a, sm.col, rw, rh, fxs - rx0, fys - ry0, fxs, fys, loW, loH);
            cur[0] = c.x;
            cur[1] = c.y;
            cur[2] = c.z;
        }
        float hc[3];
        hist_ycocg(h[k], hc);
        float ma = 0.f;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) ma = fmaxf(ma, fabsf(hc[ch] - b.m[ch]) * rcp_approx(b.e[ch]));
        const bool rejected = (rej >> k) & 1u;
        float alpha = rejected ? a.rejection_alpha : a.alpha;
        if (a.reset) alpha = 1.0f;
        if (rejected || a.reset) beta = 1.0f;  // taa.comp:852 and 898
        store_out(a, x, y, clip_blend(hc, b.m, ma, cur, alpha * beta));
    }
}

}  // namespace fast32

bool fast32_up_supported(const taa_uniforms_t& U, int history_fmt, int in_w, int in_h, int out_w, int out_h) {
    const taa_parameters_t& P = U.param[0];
    // up_path_supported: upsampling on, source no larger than the target on either axis
    // (so that a tile's source texels and ring fit 35 x 19)
    return history_fmt == 0 && tiled::is_hot(P) && (P.mInterpolationMode == 0 || P.mInterpolationMode == 2) &&
           up_path_supported(U, in_w, in_h, out_w, out_h);
}

cudaError_t launch_resolve_fast32_up(int motion_ch, const taa_uniforms_t& U, const FrameArgs& f, cudaStream_t s) {
    using namespace fast32;
    const taa_parameters_t& P = U.param[0];
    const Args a = make_args(U, f);
    UpArgs up;
    up.loW = f.color.w;
    up.loH = f.color.h;
    up.jx = upsample_jitter(U.mJitterNdc[0], P.mUnjitterFactor, up.loW);
    up.jy = upsample_jitter(U.mJitterNdc[1], P.mUnjitterFactor, up.loH);
    up.scx = (float)a.W / (float)up.loW;
    up.scy = (float)a.H / (float)up.loH;
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int tma_ok = a.hist && f.history.w >= WW && f.history.h >= WH && encode_history_map(f.history, 2, WW, WH, &map);
    const dim3 grid((a.W + TX - 1) / TX, (a.H + TY - 1) / TY);
    auto go = [&](auto kernel) {
        kernel<<<grid, NT, 0, s>>>(a, map, tma_ok, up);
        return cudaGetLastError();
    };
    const bool cr = P.mInterpolationMode == 2, m4 = motion_ch == 4;
    if (cr) return m4 ? go(resolve_strips_up<2, 4>) : go(resolve_strips_up<2, 2>);
    return m4 ? go(resolve_strips_up<0, 4>) : go(resolve_strips_up<0, 2>);
}

}  // namespace taa_dev
