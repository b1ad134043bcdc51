// resolve_tiled.cu - the tiled FP32 resolve form: the CTA pipeline of
// tiled_skeleton.cuh with the oracle's FP32 arithmetic (policy_f32.cuh).
// Compiled with -fmad=false.
#include "kernels.h"
#include "policy_f32.cuh"

namespace taa_dev {

cudaError_t launch_resolve_tiled(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U,
                                 const FrameArgs& a, cudaStream_t s) {
    return tiled::launch_form<tiled::ExactF32>(history_fmt, motion_ch, interp, U, a, s);
}

}  // namespace taa_dev
