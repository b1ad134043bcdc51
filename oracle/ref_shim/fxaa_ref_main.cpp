// fxaa_ref_main.cpp - the reference's FXAA passes of the ray-trace-assist path
// (shaders/antialias_fxaa_prepare.comp, shaders/antialias_fxaa.comp with
// shaders/Fxaa3_11_mod.h), compiled as C++ through glsl_shim.hpp (test
// infrastructure: the pin of the oracle's FXAA restatement).
// oracle/ref_build.py rewrites the two shader sources mechanically (drops
// #version/#extension) and compiles this file once with REAL = float and once
// with REAL = double, with GLSL_SNAP = 1/512 texel (the oracle's FXAA sampler).
#include "glsl_shim.hpp"

namespace glsl {
namespace fxaa_prepare_shader {
uvec3 gl_GlobalInvocationID;
#define layout(...)
#define uniform struct
#define writeonly
#define readonly
#define restrict
#define in
#define float GReal
#include FXAA_PREPARE_SOURCE
#undef float
#undef in
#undef restrict
#undef readonly
#undef writeonly
#undef uniform
#undef layout
}  // namespace fxaa_prepare_shader

namespace fxaa_shader {
uvec3 gl_GlobalInvocationID;
#define layout(...)
#define uniform struct
#define writeonly
#define readonly
#define restrict
#define in
#define float GReal
#include FXAA_SOURCE
#undef float
#undef in
#undef restrict
#undef readonly
#undef writeonly
#undef uniform
#undef layout
}  // namespace fxaa_shader
}  // namespace glsl

using namespace glsl;

extern "C" {

// antialias_fxaa_prepare.comp over an RGBA image: rgb and luma, unrounded.
int ref_fxaa_prepare(const float* in, int w, int h, double* out) {
    namespace S = glsl::fxaa_prepare_shader;
    S::uInput = texture2D{in, w, h, 4};
    S::uOutput = image2D{out, w, h};
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            S::gl_GlobalInvocationID = uvec3{uvec2{(uint)x, (uint)y}, 0u};
            S::main();
        }
    return 0;
}

// antialias_fxaa.comp over a prepared RGBA image (as the RGBA16F temp image
// holds it) and a segmentation mask; the push constants as given.
int ref_fxaa(const float* prepared, const uint32_t* segmask, int w, int h, float rcp_x, float rcp_y, float subpix,
             float edge_threshold, float edge_threshold_min, double* out) {
    namespace S = glsl::fxaa_shader;
    static texture2D tex;
    tex = texture2D{prepared, w, h, 4};
    S::texInput = sampler2D(&tex);
    S::uOutput = image2D{out, w, h};
    S::taaSegMask = uimage2D{const_cast<uint32_t*>(segmask), w, h};
    S::pushConstants.fxaaQualityRcpFrame = vec2(rcp_x, rcp_y);
    S::pushConstants.fxaaQualitySubpix = subpix;
    S::pushConstants.fxaaQualityEdgeThreshold = edge_threshold;
    S::pushConstants.fxaaQualityEdgeThresholdMin = edge_threshold_min;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            S::gl_GlobalInvocationID = uvec3{uvec2{(uint)x, (uint)y}, 0u};
            S::main();
        }
    return 0;
}

}  // extern "C"
