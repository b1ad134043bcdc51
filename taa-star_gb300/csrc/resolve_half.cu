// resolve_half.cu - the FP16 resolve form (policy_half.cuh) on the tiled
// pipeline (tiled_skeleton.cuh): the fast variant, every pixel in FP16.
#include "policy_half.cuh"

namespace taa_dev {

cudaError_t launch_resolve_half(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U,
                                const FrameArgs& a, cudaStream_t s) {
    return tiled::launch_form<half_form::HalfPol<false>>(history_fmt, motion_ch, interp, U, a, s);
}

}  // namespace taa_dev
