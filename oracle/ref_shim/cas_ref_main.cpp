// cas_ref_main.cpp - the reference's shaders/sharpen_cas.comp (FidelityFX CAS,
// sharpen only: CasFilter of shaders/ffx_cas.h on the GLSL half of
// shaders/ffx_a.h) compiled as C++ through ffx_glsl.hpp, FP32 only (the
// filter's reciprocal and square-root approximations act on FP32 bit
// patterns).  Test infrastructure: the pin of the oracle's CAS restatement.
// oracle/ref_build.py rewrites sharpen_cas.comp and ffx_cas.h mechanically
// (drops #version/#extension, turns `out T x` / `inout T x` parameters into
// `T& x`); ffx_a.h compiles as it lies.
#include "ffx_glsl.hpp"

namespace ffx_glsl {
namespace cas_shader {
// the dispatch's built-ins, set per invocation by the loop below
uvec3 gl_LocalInvocationID, gl_WorkGroupID;
// the push-constant block's members are globals of the shader
uvec4 pc_const0, pc_const1;
#define const0 pc_const0
#define const1 pc_const1
#define layout(...)
#define uniform struct
#define writeonly
#define readonly
#define restrict
#define in
#include CAS_SOURCE
#undef in
#undef restrict
#undef readonly
#undef writeonly
#undef uniform
#undef layout
#undef const1
#undef const0
}  // namespace cas_shader
}  // namespace ffx_glsl

extern "C" {

// sharpen_cas.comp over an RGBA image of w x h FP32 texels with the CasSetup
// constants const0/const1; writes RGBA doubles (the FP32 results).  The
// dispatch is the reference's: ceil(w/16) x ceil(h/16) work groups of 64
// invocations (source/taa.hpp:1134), each filtering four pixels 8 apart.
int ref_cas(const float* in, int w, int h, const uint32_t* c0, const uint32_t* c1, double* out) {
    namespace S = ffx_glsl::cas_shader;
    using ffx_glsl::uvec3;
    using ffx_glsl::uvec4;
    S::imgSrc = ffx_glsl::image2D{in, nullptr, w, h};
    S::imgDst = ffx_glsl::image2D{nullptr, out, w, h};
    S::pc_const0 = uvec4(c0[0], c0[1], c0[2], c0[3]);
    S::pc_const1 = uvec4(c1[0], c1[1], c1[2], c1[3]);
    for (int gy = 0; gy < (h + 15) / 16; ++gy)
        for (int gx = 0; gx < (w + 15) / 16; ++gx)
            for (uint32_t l = 0; l < 64; ++l) {
                S::gl_WorkGroupID = uvec3(gx, gy, 0);
                S::gl_LocalInvocationID = uvec3(l, 0, 0);
                S::main();
            }
    return 0;
}

}  // extern "C"
