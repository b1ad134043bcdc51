// post_api.cpp - the passes that follow the resolve in the reference's frame
// (source/taa.hpp:1028-1139): FXAA on the segmentation mask and the sharpen
// pass on its own.  Validation and launch only; the kernels are in fxaa.cu
// and resolve_fast.cu.
#include <cuda_runtime.h>

#include <cstring>

#include "../../include/taa_gb300.h"
#include "host_util.h"
#include "kernels.h"

using namespace taa_host;
using taa_dev::Img;
using taa_dev::ImgW;

namespace {

bool overlaps(const char* alo, const char* ahi, const char* blo, const char* bhi) { return alo < bhi && blo < ahi; }

int check_size(int32_t w, int32_t h, const char* who) {
    if (w <= 0 || h <= 0 || w > 32768 || h > 32768) return fail(TAA_E_INVAL, "%s: image size %dx%d", who, w, h);
    return ok();
}

}  // namespace

extern "C" {

// push_constants_for_fxaa (source/taa.hpp:93-98)
int taa_fxaa_default_params(taa_fxaa_params_t* out) {
    if (!out) return fail(TAA_E_INVAL, "taa_fxaa_default_params: NULL argument");
    out->subpix = 0.75f;
    out->edge_threshold = 0.116f;
    out->edge_threshold_min = 0.0833f;
    return ok();
}

// source/taa.hpp:1063-1104 (prepare + FXAA dispatches), one kernel.
int taa_fxaa(taa_ctx* ctx, void* stream, const void* input, size_t input_pitch, const void* segmask,
             size_t segmask_pitch, void* output, size_t output_pitch, int32_t width, int32_t height,
             const taa_fxaa_params_t* params) {
    static const char* who = "taa_fxaa";
    int rc;
    if ((rc = check_size(width, height, who))) return rc;
    taa_fxaa_params_t p;
    taa_fxaa_default_params(&p);
    if (params) p = *params;
    if (!finite(p.subpix) || !finite(p.edge_threshold) || !finite(p.edge_threshold_min))
        return fail(TAA_E_INVAL, "%s: parameters must be finite", who);
    const char *ilo = nullptr, *ihi = nullptr, *olo = nullptr, *ohi = nullptr;
    if ((rc = check_image("input", input, input_pitch, width, height, 8, true, &ilo, &ihi))) return rc;
    if ((rc = check_image("segmask", segmask, segmask_pitch, width, height, 4, false))) return rc;
    if ((rc = check_image("output", output, output_pitch, width, height, 8, true, &olo, &ohi))) return rc;
    if (overlaps(ilo, ihi, olo, ohi)) return fail(TAA_E_INVAL, "%s: output overlaps input", who);
    // the reference's push constant: 1 / output resolution in FP32 (source/taa.hpp:953)
    const float rcp[2] = {1.f / (float)width, 1.f / (float)height};
    Img in{(const char*)input, input_pitch, width, height};
    Img seg{(const char*)segmask, segmask_pitch, width, height};
    ImgW out{(char*)output, output_pitch};
    // the context's work list when it holds every pixel of this image
    uint32_t* list = nullptr;
    if (ctx && ctx->fxaa_list && (size_t)width * (size_t)height <= ctx->fxaa_cap) list = ctx->fxaa_list;
    cudaError_t e = taa_dev::launch_fxaa(in, seg, out, rcp, p.subpix, p.edge_threshold, p.edge_threshold_min, list,
                                         (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return ok();
}

// source/taa.hpp:1111-1139 on an arbitrary input image.
int taa_sharpen(void* stream, uint32_t sharpener, float factor, const void* input, size_t input_pitch, void* output,
                size_t output_pitch, int32_t width, int32_t height) {
    static const char* who = "taa_sharpen";
    int rc;
    if ((rc = check_size(width, height, who))) return rc;
    if (sharpener != TAA_SHARPEN_SIMPLE && sharpener != TAA_SHARPEN_CAS)
        return fail(TAA_E_INVAL, "%s: sharpener %u (1 simple, 2 CAS)", who, sharpener);
    if (!finite(factor)) return fail(TAA_E_INVAL, "%s: factor not finite", who);
    const char *ilo = nullptr, *ihi = nullptr, *olo = nullptr, *ohi = nullptr;
    if ((rc = check_image("input", input, input_pitch, width, height, 8, true, &ilo, &ihi))) return rc;
    if ((rc = check_image("output", output, output_pitch, width, height, 8, true, &olo, &ohi))) return rc;
    if (overlaps(ilo, ihi, olo, ohi)) return fail(TAA_E_INVAL, "%s: output overlaps input", who);
    uint32_t c0[4], c1[4];
    if ((rc = taa_cas_setup(factor, (float)width, (float)height, (float)width, (float)height, c0, c1))) return rc;
    taa_dev::FrameArgs a;
    std::memset(&a, 0, sizeof a);
    a.result = ImgW{(char*)input, input_pitch};
    a.sharpened = ImgW{(char*)output, output_pitch};
    a.out_w = width;
    a.out_h = height;
    a.cas_peak_bits = c1[0];
    a.sharpen_factor = factor;
    cudaError_t e = taa_dev::launch_sharpen((int)sharpener, a, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return ok();
}

}  // extern "C"
