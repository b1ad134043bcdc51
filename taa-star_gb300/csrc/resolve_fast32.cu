// resolve_fast32.cu - TAA_FORM_FAST: the strip body (strip_body.cuh) with the
// FP32 policy, for one view (launch_resolve_fast32), for one view with a
// fused sharpener (launch_resolve_fast32_sharpen) and for many views in one
// launch (launch_fast32_batch, the batch's tile shape 5).
#include <cstring>

#include "strip_body.cuh"

namespace taa_dev {
bool fast32_supported(const taa_uniforms_t& U, int history_fmt, int in_w, int in_h, int out_w, int out_h) {
    const taa_parameters_t& P = U.param[0];
    return history_fmt == 0 && tiled::is_hot(P) && (P.mInterpolationMode == 0 || P.mInterpolationMode == 2) &&
           fast_path_supported(U, in_w, in_h, out_w, out_h);
}

// The reference's default parameter block and its relatives: RGB, 3x3
// minimum/maximum box, clamp; velocity for every pixel, for movers only, or
// reprojection; nothing that changes the blend weight.
static bool clamp_rgb_mode(const taa_parameters_t& P) {
    return !P.mUseYCoCg && !P.mToneMapLumaKaris && !P.mVarianceClipping && !P.mShapedNeighbourhood &&
           P.mColorClampingOrClipping == 1 && P.mUseVelocityVectors >= 0 && P.mUseVelocityVectors <= 2 &&
           P.mVelocitySampleMode == 0 && !P.mVelBasedAlpha && !P.mLumaWeightingLottes && !P.mReduceBlendNearClamp &&
           !P.mAddNoise && !P.mDynamicAntiGhosting && !P.mRayTraceAugment;
}

bool fast32_single_supported(const taa_uniforms_t& U, int history_fmt, int in_w, int in_h, int out_w, int out_h) {
    const taa_parameters_t& P = U.param[0];
    return (history_fmt == 0 || history_fmt == 1) && (tiled::is_hot(P) || clamp_rgb_mode(P)) &&
           (P.mInterpolationMode == 0 || P.mInterpolationMode == 2) && fast_path_supported(U, in_w, in_h, out_w, out_h);
}

namespace {
// The kernel for the mode, filter, velocity channels and history format.
template <int HF>
cudaError_t launch_single(const taa_parameters_t& P, const taa_uniforms_t& U, const fast32::Args& a,
                          const CUtensorMap& map, int tma_ok, int motion_ch, cudaStream_t s) {
    using namespace fast32;
    const dim3 grid((a.W + TX - 1) / TX, (a.H + TY - 1) / TY);
    auto go = [&](auto kernel) {
        kernel<<<grid, NT, 0, s>>>(a, map, tma_ok);
        return cudaGetLastError();
    };
    const bool cr = P.mInterpolationMode == 2, m4 = motion_ch == 4;
    if (!tiled::is_hot(P)) {  // the clamp RGB mode
        const Reproj rp = make_reproj(U);
        auto go_rp = [&](auto kernel) {
            kernel<<<grid, NT, 0, s>>>(a, map, tma_ok, rp);
            return cudaGetLastError();
        };
        if (cr)
            return m4 ? go_rp(resolve_strips_reproj<ClampRgbPol, 2, 4, HF>)
                      : go_rp(resolve_strips_reproj<ClampRgbPol, 2, 2, HF>);
        return m4 ? go_rp(resolve_strips_reproj<ClampRgbPol, 0, 4, HF>)
                  : go_rp(resolve_strips_reproj<ClampRgbPol, 0, 2, HF>);
    }
    if (cr) return m4 ? go(resolve_strips<F32Pol, 2, 4, HF>) : go(resolve_strips<F32Pol, 2, 2, HF>);
    return m4 ? go(resolve_strips<F32Pol, 0, 4, HF>) : go(resolve_strips<F32Pol, 0, 2, HF>);
}
}  // namespace

cudaError_t launch_resolve_fast32(int motion_ch, int history_fmt, const taa_uniforms_t& U, const FrameArgs& f,
                                  cudaStream_t s) {
    using namespace fast32;
    const taa_parameters_t& P = U.param[0];
    Args a = make_args(U, f);
    a.hout_half = history_fmt == 1;
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int ww = history_fmt == 1 ? WinOf<1>::W : WW;
    const int tma_ok = a.hist && f.history.w >= ww && f.history.h >= WH &&
                       encode_history_map(f.history, history_fmt == 1 ? 1 : (TAA_FAST_TMA2D ? 2 : 0), ww, WH, &map);
    if (history_fmt == 1) return launch_single<1>(P, U, a, map, tma_ok, motion_ch, s);
    return launch_single<0>(P, U, a, map, tma_ok, motion_ch, s);
}

cudaError_t launch_resolve_fast32_sharpen(int motion_ch, int sharpener, const taa_uniforms_t& U, const FrameArgs& f,
                                          cudaStream_t s) {
    using namespace fast32;
    const taa_parameters_t& P = U.param[0];
    const Args a = make_args(U, f);
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const int tma_ok = a.hist && f.history.w >= WW && f.history.h >= WH &&
                       encode_history_map(f.history, TAA_FAST_TMA2D ? 2 : 0, WW, WH, &map);
    const bool cas = sharpener == TAA_SHARPEN_CAS;
    float peak;
    std::memcpy(&peak, &f.cas_peak_bits, sizeof peak);
    const float k = cas ? peak : f.sharpen_factor;
    char* const sp = f.sharpened.p;
    const uint32_t pitch = (uint32_t)f.sharpened.pitch;
    // 30x14 output tiles, each resolved with its 1-pixel ring
    const dim3 grid((a.W + TX - 3) / (TX - 2), (a.H + TY - 3) / (TY - 2));
    auto go = [&](auto kernel) {
        kernel<<<grid, NT, 0, s>>>(a, map, tma_ok, sp, pitch, k);
        return cudaGetLastError();
    };
    const bool cr = P.mInterpolationMode == 2, m4 = motion_ch == 4;
    if (cas) {
        if (cr) return m4 ? go(resolve_strips_sharpen<2, 2, 4>) : go(resolve_strips_sharpen<2, 2, 2>);
        return m4 ? go(resolve_strips_sharpen<2, 0, 4>) : go(resolve_strips_sharpen<2, 0, 2>);
    }
    if (cr) return m4 ? go(resolve_strips_sharpen<1, 2, 4>) : go(resolve_strips_sharpen<1, 2, 2>);
    return m4 ? go(resolve_strips_sharpen<1, 0, 4>) : go(resolve_strips_sharpen<1, 0, 2>);
}

void fast32_window(int* w, int* h) {
    *w = fast32::WW;
    *h = fast32::WH;
}

namespace {
template <int INTERP, int MC> const void* fast32_batch_kernel() {
    return reinterpret_cast<const void*>(&fast32::resolve_strips_batch<fast32::F32Pol, INTERP, MC>);
}
const void* fast32_batch_fn(int interp, int motion_ch) {
    if (interp == 2) return motion_ch == 4 ? fast32_batch_kernel<2, 4>() : fast32_batch_kernel<2, 2>();
    if (interp == 0) return motion_ch == 4 ? fast32_batch_kernel<0, 4>() : fast32_batch_kernel<0, 2>();
    return nullptr;
}
}  // namespace

cudaError_t fast32_batch_occupancy(int interp, int motion_ch, int* ctas_per_sm) {
    const void* fn = fast32_batch_fn(interp, motion_ch);
    if (!fn) return cudaErrorInvalidValue;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, fast32::NT, 0);
}

cudaError_t launch_fast32_batch(int interp, int motion_ch, const BatchView* views, const CUtensorMap* maps,
                                const int* tma_ok, const uint32_t* jobs, int njobs, int grid, cudaStream_t stream) {
    const void* fn = fast32_batch_fn(interp, motion_ch);
    if (!fn) return cudaErrorInvalidValue;
    void* args[] = {(void*)&views, (void*)&maps, (void*)&tma_ok, (void*)&jobs, (void*)&njobs};
    return cudaLaunchKernel(fn, dim3(grid), dim3(fast32::NT), args, 0, stream);
}

}  // namespace taa_dev
