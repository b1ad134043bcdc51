// post_ref_main.cpp - the reference's post-process pass (shaders/post_process.comp:
// split-screen line, zoom box and magnified inset, debug image on either side
// of the split) compiled as C++ through glsl_shim.hpp (test infrastructure: the
// pin of the oracle's restatement).  oracle/ref_build.py rewrites the shader
// source mechanically (drops #version/#extension) and compiles this file once
// with REAL = float and once with REAL = double.
#include "glsl_shim.hpp"

namespace glsl {
namespace post_shader {
uvec3 gl_GlobalInvocationID;
#define layout(...)
#define uniform struct
#define writeonly
#define readonly
#define restrict
#define in
#define float GReal
#include POST_SOURCE
#undef float
#undef in
#undef restrict
#undef readonly
#undef writeonly
#undef uniform
#undef layout
}  // namespace post_shader
}  // namespace glsl

using namespace glsl;

extern "C" {

// post_process.comp over an RGBA input and debug image (w x h), the push
// constants as given (ivec4s, vec4 masks, VkBool32 flags as 0/1); writes the
// RGBA output unrounded.
int ref_post_process(const float* input, const float* debug, int w, int h, const int* zoom_src, const int* zoom_dst,
                     const float* mask_l, const float* mask_r, int zoom, int show_zoom_box, int split_x, int show_l,
                     int show_r, double* out) {
    namespace S = glsl::post_shader;
    S::uInputFrame = texture2D{input, w, h, 4};
    S::uDebugFrame = texture2D{debug, w, h, 4};
    S::uOutput = image2D{out, w, h};
    auto& pc = S::pushConstants;
    pc.zoomSrcLTWH = ivec4(zoom_src[0], zoom_src[1], zoom_src[2], zoom_src[3]);
    pc.zoomDstLTWH = ivec4(zoom_dst[0], zoom_dst[1], zoom_dst[2], zoom_dst[3]);
    pc.debugL_mask = vec4(mask_l[0], mask_l[1], mask_l[2], mask_l[3]);
    pc.debugR_mask = vec4(mask_r[0], mask_r[1], mask_r[2], mask_r[3]);
    pc.zoom = zoom != 0;
    pc.showZoomBox = show_zoom_box != 0;
    pc.splitX = split_x;
    pc.debugL_show = show_l != 0;
    pc.debugR_show = show_r != 0;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            S::gl_GlobalInvocationID = uvec3{uvec2{(uint)x, (uint)y}, 0u};
            S::main();
        }
    return 0;
}

}  // extern "C"
