// taa_oracle.hpp - CPU restatement of the reference TAA resolve (test infrastructure).
//
// THIS IS THE ORACLE.  It is test infrastructure only: the tests, the smoke
// check and the CPU-baseline leg of the benchmark use it as the checker.  The
// product library never links it.
//
// It restates shaders/taa.comp:131-960 (resolve), shaders/ffx_cas.h:424-537 with
// shaders/ffx_a.h:1455-1457 (CAS sharpen-only) and shaders/sharpen.comp:24-38
// (simple sharpen), templated on the arithmetic type:
//   R = float  : "FP32 GLSL semantics" - every operation rounded to FP32 in the
//                shader's order, no contraction (built with -ffp-contract=off).
//                The four accumulations that are numerically fragile in FP32
//                (the second moment sum of the 3x3 neighbourhood) are written
//                as explicit fused multiply-adds in source order, which is what
//                a contracting GLSL compiler emits; the CUDA kernels do the same.
//   R = double : FP64 transliteration, the truth against which errors are reported.
//
// Sampler semantics (Vulkan behaviour that is not in the reference source):
//   * texelFetch outside the image clamps to the edge (undefined in GLSL; the
//     shader itself notes this at taa.comp:41).
//   * texture() at a coordinate that is, by construction in the shader, the
//     centre of a texel (the 3x3 neighbourhood without unjitter, velocity at the
//     pixel centre, the 3x3 closest-depth taps, the anti-ghosting taps - all
//     only when source and target sizes are equal) returns that texel exactly,
//     as the hardware sampler does with its 8-bit sub-texel precision.
//   * texture() elsewhere is exact-weight bilinear with clamp-to-edge
//     (taa.hpp:274 creates a bilinear clamp-to-edge sampler).
//   * The 9-tap Catmull-Rom history filter (taa.comp:496-512) is evaluated as
//     the 16-tap form it equals under an exact bilinear sampler (taa.comp:469-495
//     with the edge clamp at size-1); the "b-spline" 4-tap filter
//     (taa.comp:517-543) is evaluated literally with exact bilinear taps.
#pragma once
#include <cstdint>
#include <cstddef>
#include "../include/taa_params.h"

namespace taa_oracle {

// Images handed to the oracle: float arrays (exact copies of the FP16/FP32
// texels), `ch` channels per texel, rows tightly packed.
struct ImageF {
    const float* p = nullptr;
    int w = 0, h = 0, ch = 4;
};
struct ImageU {
    const uint32_t* p = nullptr;
    int w = 0, h = 0;
};

struct ResolveInputs {
    ImageF color;          // binding 1, RGBA, source size
    ImageF depth;          // binding 2, 1 channel, source size
    ImageF history;        // binding 3, RGBA, target size (p==nullptr reads zeros)
    ImageF history_depth;  // binding 4, 1 channel, source size
    ImageF velocity;       // binding 7, 4 channels (RG inputs are widened with z=w=0)
    ImageU material;       // binding 10
    ImageU prev_material;  // binding 11
    ImageU prev_segmask;   // binding 12
    ImageF uvnrm;          // binding 13, RGBA
    int out_w = 0, out_h = 0;
};

// Outputs (target size, 4 doubles per texel holding the value computed in R,
// before any FP16 store).  Any pointer may be null.
struct ResolveOutputs {
    double* history = nullptr;
    double* screen = nullptr;
    double* debug = nullptr;
    uint32_t* segmask = nullptr;
};

// Resolve one frame.  precision: 32 or 64.  Returns 0 or -1 on bad arguments.
int resolve(int precision, const taa_uniforms_t& u, const ResolveInputs& in,
            const ResolveOutputs& out, int nthreads);

// CAS sharpen-only on an RGBA image (3 channels used); `peak_bits` is const1.x
// of CasSetup.  Output alpha is 1.  precision 32 or 64.
int cas(int precision, const float* in, int w, int h, uint32_t peak_bits, double* out, int nthreads);

// shaders/sharpen.comp.
int sharpen(int precision, const float* in, int w, int h, float factor, double* out, int nthreads);

// The FXAA pass of the ray-trace-assist path (source/taa.hpp:1063-1104):
// shaders/antialias_fxaa_prepare.comp and antialias_fxaa.comp (FXAA 3.11
// quality preset 12) as one, on an RGBA image (alpha unused) and a segmentation
// mask (NULL: every pixel is marked).  Output: rgb and the FP16-stored luma.
// rcp_frame = 1 / image size in FP32 (source/taa.hpp:953).  precision 32 or 64.
int fxaa(int precision, const float* in, const uint32_t* segmask, int w, int h, const float rcp_frame[2],
         float subpix, float edge_threshold, float edge_threshold_min, double* out, int nthreads);

// The post-process pass (shaders/post_process.comp; push constants of
// source/taa.hpp:101-111): split line, zoom box and inset, debug image per side
// of the split (its alpha made visible in red and blue when the side's mask .w
// is positive).  `debug` may be NULL when neither side shows it.  precision 32
// or 64.
struct PostParams {
    int zoom_src[4], zoom_dst[4];  // left, top, width, height
    float mask_l[4], mask_r[4];
    int zoom, show_zoom_box, split_x, show_l, show_r;
};
int post_process(int precision, const float* in, const float* debug, int w, int h, const PostParams& pp, double* out,
                 int nthreads);

// CasSetup, restated (ffx_cas.h:375-394).
void cas_setup(float sharpness, float in_w, float in_h, float out_w, float out_h,
               uint32_t const0[4], uint32_t const1[4]);

// helpers::halton (helper_functions.hpp:9-17) and the jitter table selection of
// taa::get_jitter_offset_for_frame (taa.hpp:150-233).
float halton(int i, int b);
void jitter_offset(int sample_distribution, uint64_t frame_id, int in_w, int in_h,
                   int fixed_index, int slow_motion, float rotate_degrees, float extra_scale,
                   float out[2], int* num_samples);

// Round-to-nearest-even float -> binary16 -> float (what an RGBA16F store keeps).
float quantize_half(float x);

}  // namespace taa_oracle
