// tiled_up.cuh - the upsampling (TAAU) path of the tiled FP32 form
// (taa.comp:222-257 and 750-755): source images loW x loH, history and
// outputs hiW x hiH with hiW >= loW and hiH >= loH.
//
// One 256-thread CTA per 32x16 target tile, two vertically adjacent pixels
// per thread (the tile of the single-size tiled form):
//   1. the source texels under the tile and a 1-texel ring - at most
//      (32 + 3) x (16 + 3) for any ratio >= 1 - are staged in shared memory in
//      the working colour space, edge-clamped; warp 0 places the target-size
//      history window at the tile's centre (TMA, or cp.async at the border);
//   2. per target pixel: its source texel (int(uv * lo size)), the 3x3 box on
//      the staged neighbourhood, the jittered source sample that lands in the
//      pixel (upsample_axis / upsampled_pick, shared with the plain form; the
//      column's half once per thread) as the current
//      colour with beta = 1, else beta = 0; velocity sampled bilinearly at the
//      pixel's uv, the history position and sample, rejection, and the
//      policy's rectification with the blend mix(history, current,
//      alpha * beta).
// The arithmetic is the plain form's in its order (compiled with
// -fmad=false), so the result has the FP32 oracle's bits.  Parameter modes
// the path does not implement (velocity sampling other than the simple one,
// anti-ghosting, the segmentation mask, debug output, split screen, a
// non-zero unjittered neighbourhood) take the plain form (up_path_supported).
#pragma once
#include "tiled_skeleton.cuh"

namespace taa_dev {
namespace tiled {

template <class Pol, class S, int HF> struct UpSmem {
    static constexpr int MAXW = S::TX + 3, MAXH = S::TY + 3;  // source texels under a tile and its ring
    typename Pol::Staged col[MAXW * MAXH];
    alignas(128) typename HistTexel<HF>::T win[Win<S, HF>::W * S::WH];
    uint64_t bar;  // completion of the window's TMA copy
    int org[3];    // window origin x, y and how it is copied (1 TMA, 2 cp.async)
};

template <class Pol, class S, int HF, int MC, int INTERP>
__global__ void __launch_bounds__(S::NT, TAA_MULTI_MIN_BLOCKS * 256 / S::NT)
    resolve_tile_up(const taa_uniforms_t U, const FrameArgs a, const __grid_constant__ CUtensorMap hmap,
                    const int tma_ok) {
    using SM = UpSmem<Pol, S, HF>;
    constexpr int TX = S::TX, NT = S::NT, NPX = S::NPX, WH = S::WH;
    constexpr int WWS = Win<S, HF>::W;
    __shared__ SM sm;
    const int tid = threadIdx.x;
    if (tid == 0) mbar_init(&sm.bar, 1);
    const taa_parameters_t& P = U.param[0];
    const Mode<false> M{P};
    const int tile_x = blockIdx.x, tile_y = blockIdx.y;
    const int lx = tid % TX, ly = tid / TX;
    const int W = a.out_w, H = a.out_h, loW = a.color.w, loH = a.color.h;
    const int x0 = tile_x * TX, y0 = tile_y * S::TY;
    const f2 z{a.neg_zero2};
    // the source texel of a target column / row: int(uv * source size) with
    // uv = (t + 0.5) / target size (taa.comp:131-136)
    auto src_x = [&](int x) { return trunc_index(div_const_rn((float)x + 0.5f, (float)W, a.inv_out_w) * (float)loW); };
    auto src_y = [&](int y) { return trunc_index(div_const_rn((float)y + 0.5f, (float)H, a.inv_out_h) * (float)loH); };
    // 1. the staged source neighbourhood: texels rx0 .. rx0 + rw - 1 (and rows), edge-clamped
    const int rx0 = src_x(x0) - 1, ry0 = src_y(y0) - 1;
    const int rw = min(src_x(min(x0 + TX - 1, W - 1)) - rx0 + 2, SM::MAXW);
    const int rh = min(src_y(min(y0 + S::TY - 1, H - 1)) - ry0 + 2, SM::MAXH);
    const bool tm = M.tonemap(), yc = M.ycocg();
    for (int i = tid; i < rw * rh; i += NT) {
        const int sy = i / rw, sx = i - sy * rw;
        const int gx = clampi(rx0 + sx, 0, loW - 1), gy = clampi(ry0 + sy, 0, loH - 1);
        sm.col[i] = Pol::stage(__ldg(texel_ptr<uint2>(a.color, gx, gy)), tm, yc);
    }
    // warp 0 places the target-size history window at the tile's centre (its
    // source texel's velocity and depth: the window is only a cache, a pixel
    // whose taps leave it reads global memory)
    const Img& hi = a.history;
    const bool have_hist = hi.p != nullptr;
    const bool windowed = have_hist && INTERP != 1;
    if (windowed && tid < 32) {
        int rx, ry;
        reference_pixel<S>(a, tile_x, tile_y, rx, ry);
        const int sx = clampi(src_x(rx), 0, loW - 1), sy = clampi(src_y(ry), 0, loH - 1);
        const float rdepth = __ldg(texel_ptr<float>(a.depth, sx, sy));
        const float4 rvs = fetch_velocity<MC>(a.velocity, sx, sy);
        place_window<Pol, S, HF, MC, INTERP, false>(U, a, M, &hmap, tma_ok != 0, tile_x, tile_y, rdepth, rvs, sm.win,
                                                   &sm.bar, sm.org, tid == 0);
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
    // 2. per pixel: box, current sample, history position (before the window wait)
    const bool depth_cull = P.mDepthCulling != 0;
    const int x = x0 + lx, cx = min(x, W - 1);
    // this thread's column of the upsampled-sample search (its pixels share it)
    const UpAxis ux = upsample_axis(cx, W, loW, upsample_jitter(U.mJitterNdc[0], P.mUnjitterFactor, loW),
                                    (float)W / (float)loW);
    const float jy = upsample_jitter(U.mJitterNdc[1], P.mUnjitterFactor, loH), scy = (float)H / (float)loH;
    typename Pol::Box box[NPX];
    C3 cur[NPX];
    float beta[NPX], u[NPX], v[NPX], hu[NPX], hv[NPX], ehd[NPX], prev_depth[NPX];
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        const int cy = min(y0 + NPX * ly + k, H - 1);
        const f2 uv = div_const_rn2(add2(pk((float)cx, (float)cy), dup(0.5f)), pk(-(float)W, -(float)H),
                                    pk(a.inv_out_w, a.inv_out_h), z);
        u[k] = f2lo(uv);
        v[k] = f2hi(uv);
        const int sx = trunc_index(u[k] * (float)loW), sy = trunc_index(v[k] * (float)loH);
        Pol::template box<false>(&sm.col[(sy - ry0) * rw + (sx - rx0)], rw, M, P.mVarClipGamma, box[k], z);
        // the source sample that lands in this target texel (taa.comp:222-257)
        int fx, fy;
        cur[k] = C3{0.f, 0.f, 0.f};
        beta[k] = 0.f;
        if (upsampled_pick(ux, upsample_axis(cy, H, loH, jy, scy), fx, fy)) {
            beta[k] = 1.f;
            const int ix = fx - rx0, iy = fy - ry0;
            const float4 c = ix >= 0 && iy >= 0 && ix < rw && iy < rh
                                 ? sm.col[iy * rw + ix]
                                 : Pol::stage(__ldg(texel_ptr<uint2>(a.color, clampi(fx, 0, loW - 1),
                                                                     clampi(fy, 0, loH - 1))),
                                              tm, yc);
            cur[k] = C3{c.x, c.y, c.z};
        }
        // the history position: velocity sampled bilinearly at uv (taa.comp:391-438)
        const float depth = fetch_r32f(a.depth, sx, sy);
        const float4 vs = bilinear_uv(a.velocity.w, a.velocity.h, u[k], v[k],
                                      [&](int xx, int yy) { return fetch_velocity<MC>(a.velocity, xx, yy); });
        const bool can = !(M.use_velocity() == 0 || (M.use_velocity() == 1 && vs.w < 0.5f));
        if (can) {
            hu[k] = u[k] - vs.x;
            hv[k] = v[k] - vs.y;
            ehd[k] = depth - vs.z;
        } else {
            Pol::reproject(U, u[k], v[k], depth, hu[k], hv[k], ehd[k]);
        }
        prev_depth[k] = 0.f;
        if (depth_cull && a.history_depth.p) {
            const int tx_ = clampi(trunc_index(hu[k] * (float)loW), 0, loW - 1);
            const int ty_ = clampi(trunc_index(hv[k] * (float)loH), 0, loH - 1);
            prev_depth[k] = __ldg(texel_ptr<float>(a.history_depth, tx_, ty_));
        }
    }
    bool landed = true;
    if (mode == 1) {
        landed = mbar_wait_bounded(&sm.bar, 0u, first_wait_polls(a.status));
        if (!landed) {
            atomicOr(a.status, kStatusWindowTimeout);
            mbar_wait_bounded(&sm.bar, 0u);  // the copy may still land in this CTA's memory
        }
    } else if (mode == 2) {
        cp_async_wait_all();
        __syncthreads();
    }
    // 3. per pixel: rejection, history sample, rectification, blend, stores
#pragma unroll
    for (int k = 0; k < NPX; ++k) {
        const int y = y0 + NPX * ly + k;
        if (!(x < W && y < H && landed)) continue;
        bool rejected = false;
        if (P.mRejectOutside && (hu[k] < 0.f || hv[k] < 0.f || hu[k] >= 1.f || hv[k] >= 1.f)) rejected = true;
        if (depth_cull) {
            const float hd = prev_depth[k];
            if (fabsf(hd - ehd[k]) > 0.1f * (1.0f - hd)) rejected = true;
        }
        float4 hraw = make_float4(0.f, 0.f, 0.f, 0.f);
        if (have_hist) {
            HistoryTaps<Pol, INTERP> taps;
            taps.setup(hu[k], hv[k], hi.w, hi.h, z);
            const int span = INTERP == 2 ? 4 : 2;
            const int bx = taps.t[0].ux - wx0, by = taps.t[0].uy - wy0;
            const bool in_win = windowed && bx >= 0 && by >= 0 && bx + span <= WWS && by + span <= WH;
            if (in_win) {
                hraw = Pol::template filter_window<INTERP, HF>(taps, &sm.win[by * WWS + bx], WWS);
            } else {
                hraw = Pol::template filter<INTERP>(
                    taps, hi.w, hi.h, [&](int tx_, int ty_) { return fetch_history<HF>(hi, tx_, ty_); });
            }
        }
        float4 o = Pol::template finish<false, true>(U, P, M, box[k], cur[k], hraw, u[k], v[k], hu[k], hv[k],
                                                     rejected, beta[k]);
        store_history<HF>(a.history_out, x, y, make_float4(o.x, o.y, o.z, 0.f));
        if (a.result.p) {
            if (tm) o = Pol::un_tonemap(o);
            store_rgba16f(a.result, x, y, make_float4(o.x, o.y, o.z, 1.0f));
        }
    }
}

template <class Pol, int HF, int MC, int INTERP>
cudaError_t launch_tile_up(const taa_uniforms_t& U, const FrameArgs& a, cudaStream_t s) {
    using S = MultiShape<32, 8, 2>;
    const dim3 grid((a.out_w + S::TX - 1) / S::TX, (a.out_h + S::TY - 1) / S::TY);
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int tma_ok = INTERP != 1 && a.history.p && a.history.w >= Win<S, HF>::W && a.history.h >= S::WH &&
                       encode_history_map(a.history, HF, Win<S, HF>::W, S::WH, &map);
    resolve_tile_up<Pol, S, HF, MC, INTERP><<<grid, S::NT, 0, s>>>(U, a, map, tma_ok);
    return cudaGetLastError();
}

template <class Pol>
cudaError_t launch_form_up(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U, const FrameArgs& a,
                           cudaStream_t s) {
    auto by_interp = [&](auto hf, auto mc) {
        constexpr int HF = decltype(hf)::value, MC = decltype(mc)::value;
        return interp == 0 ? launch_tile_up<Pol, HF, MC, 0>(U, a, s)
               : interp == 1 ? launch_tile_up<Pol, HF, MC, 1>(U, a, s)
                             : launch_tile_up<Pol, HF, MC, 2>(U, a, s);
    };
    using I0 = std::integral_constant<int, 0>;
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    using I4 = std::integral_constant<int, 4>;
    if (history_fmt == 0) return motion_ch == 4 ? by_interp(I0{}, I4{}) : by_interp(I0{}, I2{});
    return motion_ch == 4 ? by_interp(I1{}, I4{}) : by_interp(I1{}, I2{});
}

}  // namespace tiled
}  // namespace taa_dev
