// resolve_tiled.cu - the tiled FP32 resolve form: the CTA pipeline of
// tiled_skeleton.cuh with the oracle's FP32 arithmetic (policy_f32.cuh), and
// its upsampling path (tiled_up.cuh).
// Compiled with -fmad=false.
#include "kernels.h"
#include "policy_f32.cuh"
#include "tiled_up.cuh"

namespace taa_dev {

cudaError_t launch_resolve_tiled(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U,
                                 const FrameArgs& a, cudaStream_t s) {
    if (a.color.w != a.out_w || a.color.h != a.out_h)  // upsampling (up_path_supported)
        return tiled::launch_form_up<tiled::ExactF32>(history_fmt, motion_ch, interp, U, a, s);
    return tiled::launch_form<tiled::ExactF32>(history_fmt, motion_ch, interp, U, a, s);
}

}  // namespace taa_dev
