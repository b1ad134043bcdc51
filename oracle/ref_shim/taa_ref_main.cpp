// taa_ref_main.cpp - the reference's shaders/taa.comp and shaders/sharpen.comp,
// compiled as C++ through glsl_shim.hpp (test infrastructure: the pin of the
// oracle's restatement).  oracle/ref_build.py rewrites the shader sources
// mechanically (drops #version/#extension, turns `out T x` parameters into
// `T& x`) and compiles this file once with REAL = float (GLSL FP32) and once
// with REAL = double.
#include <vector>

#include "glsl_shim.hpp"
#include "taa_params.h"

// the shader's common header defines the same flag names as taa_params.h
#undef TAA_RTFLAG_OUT
#undef TAA_RTFLAG_DIS
#undef TAA_RTFLAG_NRM
#undef TAA_RTFLAG_DPT
#undef TAA_RTFLAG_MID
#undef TAA_RTFLAG_LUM
#undef TAA_RTFLAG_CNT
#undef TAA_RTFLAG_ALL
#undef TAA_RTFLAG_FXD
#undef TAA_RTFLAG_FXA

namespace glsl {
namespace taa_shader {
uvec3 gl_GlobalInvocationID;  // set per invocation by the dispatch loop below
#define layout(...)
#define uniform struct
#define writeonly
#define readonly
#define restrict
#define in
#define float GReal
#include TAA_COMP_SOURCE
#undef float
#undef in
#undef restrict
#undef readonly
#undef writeonly
#undef uniform
#undef layout
}  // namespace taa_shader

namespace sharpen_shader {
uvec3 gl_GlobalInvocationID;
#define layout(...)
#define uniform struct
#define writeonly
#define readonly
#define restrict
#define in
#define float GReal
#include SHARPEN_SOURCE
#undef float
#undef in
#undef restrict
#undef readonly
#undef writeonly
#undef uniform
#undef layout
}  // namespace sharpen_shader
}  // namespace glsl

namespace {
using namespace glsl;

// uniforms_for_taa field by field into the shader's block (bools from VkBool32)
template <class P> void copy_params(P& d, const taa_parameters_t& s) {
#define F(n) d.n = s.n;
#define B(n) d.n = s.n != 0;
    F(mAlpha) F(mColorClampingOrClipping) B(mDepthCulling) B(mUnjitterNeighbourhood) B(mUnjitterCurrentSample)
    F(mUnjitterFactor) B(mPassThrough) B(mUseYCoCg) B(mShrinkChromaAxis) B(mVarianceClipping) B(mShapedNeighbourhood)
    B(mLumaWeightingLottes) F(mVarClipGamma) F(mMinAlpha) F(mMaxAlpha) F(mRejectionAlpha) B(mRejectOutside)
    F(mUseVelocityVectors) F(mVelocitySampleMode) F(mInterpolationMode) B(mToneMapLumaKaris) B(mAddNoise)
    F(mNoiseFactor) B(mReduceBlendNearClamp) B(mDynamicAntiGhosting) B(mVelBasedAlpha) F(mVelBasedAlphaMax)
    F(mVelBasedAlphaFactor) B(mRayTraceAugment) F(mRayTraceAugmentFlags) F(mRayTraceAugment_WNrm)
    F(mRayTraceAugment_WDpt) F(mRayTraceAugment_WMId) F(mRayTraceAugment_WLum) F(mRayTraceAugment_Thresh)
    F(mRayTraceHistoryCount) F(mDebugMode) F(mDebugScale) B(mDebugCenter) B(mDebugToScreenOutput)
#undef F
#undef B
    d.mDebugMask = vec4(s.mDebugMask[0], s.mDebugMask[1], s.mDebugMask[2], s.mDebugMask[3]);
}

mat4 to_mat4(const float* m) {
    mat4 r;
    for (int c = 0; c < 4; ++c) r.c[c] = vec4(m[c * 4 + 0], m[c * 4 + 1], m[c * 4 + 2], m[c * 4 + 3]);
    return r;
}
}  // namespace

extern "C" {

// One frame of the reference resolve.  Images as in the oracle's C entry
// point: float texels, 4 channels except depth (1) ; velocity widened to 4.
int ref_taa_resolve(const taa_uniforms_t* u, int in_w, int in_h, int out_w, int out_h, const float* color,
                    const float* depth, const float* history, const float* history_depth, const float* velocity4,
                    const uint32_t* material, const uint32_t* prev_material, const uint32_t* prev_segmask,
                    const float* uvnrm, double* out_history, double* out_screen, double* out_debug,
                    uint32_t* out_segmask) {
    namespace S = glsl::taa_shader;
    std::vector<double> dbg_scratch;
    if (!out_debug) {
        dbg_scratch.assign((size_t)out_w * out_h * 4, 0.0);
        out_debug = dbg_scratch.data();
    }
    S::uCurrentFrame = texture2D{color, in_w, in_h, 4};
    S::uCurrentDepth = texture2D{depth, in_w, in_h, 1};
    S::uCurrentVelocity = texture2D{velocity4, in_w, in_h, 4};
    S::uCurrentUvNrm = texture2D{uvnrm, in_w, in_h, 4};
    S::uHistoryFrame = texture2D{history, out_w, out_h, 4};
    S::uHistoryDepth = texture2D{history_depth, in_w, in_h, 1};
    S::uCurrentMaterial = uimage2D{const_cast<uint32_t*>(material), in_w, in_h};
    S::uPreviousMaterial = uimage2D{const_cast<uint32_t*>(prev_material), in_w, in_h};
    S::uPreviousSegMask = uimage2D{const_cast<uint32_t*>(prev_segmask), out_w, out_h};
    S::uResultScreen = image2D{out_screen, out_w, out_h};
    S::uResultHistory = image2D{out_history, out_w, out_h};
    S::uDebug = image2D{out_debug, out_w, out_h};
    S::uSegMask = uimage2D{out_segmask, out_w, out_h};
    S::ubo.mHistoryViewProjMatrix = to_mat4(u->mHistoryViewProjMatrix);
    S::ubo.mInverseViewProjMatrix = to_mat4(u->mInverseViewProjMatrix);
    copy_params(S::ubo.param[0], u->param[0]);
    copy_params(S::ubo.param[1], u->param[1]);
    S::ubo.mJitterNdc = vec4(u->mJitterNdc[0], u->mJitterNdc[1], u->mJitterNdc[2], u->mJitterNdc[3]);
    S::ubo.mSinTime = vec4(u->mSinTime[0], u->mSinTime[1], u->mSinTime[2], u->mSinTime[3]);
    S::ubo.splitScreen = u->splitScreen != 0;
    S::ubo.splitX = u->splitX;
    S::ubo.mUpsampling = u->mUpsampling != 0;
    S::ubo.mBypassHistoryUpdate = u->mBypassHistoryUpdate != 0;
    S::ubo.mResetHistory = u->mResetHistory != 0;
    S::ubo.mCamNearPlane = u->mCamNearPlane;
    S::ubo.mCamFarPlane = u->mCamFarPlane;
    for (int y = 0; y < out_h; ++y)
        for (int x = 0; x < out_w; ++x) {
            // one invocation: the shader's globals start from their initialisers
            S::gDebugValue = vec4(0);
            S::gl_GlobalInvocationID = uvec3{uvec2{(uint)x, (uint)y}, 0u};
            S::main();
        }
    return 0;
}

// shaders/sharpen.comp over an RGBA image.
int ref_sharpen(const float* in, int w, int h, float factor, double* out) {
    namespace S = glsl::sharpen_shader;
    S::uInputFrame = texture2D{in, w, h, 4};
    S::uOutput = image2D{out, w, h};
    S::pushConstants.sharpeningFactor = factor;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            S::gl_GlobalInvocationID = uvec3{uvec2{(uint)x, (uint)y}, 0u};
            S::main();
        }
    return 0;
}

}  // extern "C"
