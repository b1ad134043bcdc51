// resolve_half_guard.cu - the FP16 resolve form (policy_half.cuh) with
// TAA_FLAG_FP16_GUARD: a pixel whose clip engages on a box ill-conditioned for
// FP16 is finished in FP32 from its source texels.
#include "policy_half.cuh"

namespace taa_dev {

cudaError_t launch_resolve_half_guarded(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U,
                                        const FrameArgs& a, cudaStream_t s) {
    return tiled::launch_form<half_form::HalfPol<true>>(history_fmt, motion_ch, interp, U, a, s);
}

}  // namespace taa_dev
