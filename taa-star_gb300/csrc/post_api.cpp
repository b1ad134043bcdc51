// post_api.cpp - the passes that follow the resolve in the reference's frame
// (source/taa.hpp:1028-1158): FXAA on the segmentation mask, the sharpen pass
// on its own and the post-process visualisation.  Validation and launch only;
// the kernels are in fxaa.cu, resolve_fast.cu and post_process.cu.
#include <cmath>
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

static_assert(sizeof(taa_post_process_params_t) == 84, "push_constants_for_postprocess is 84 bytes");

// push_constants_for_postprocess (source/taa.hpp:101-111) and the zoom boxes of
// set_source_image_views (source/taa.hpp:352-359; w is unsigned there)
int taa_post_process_default_params(int32_t width, int32_t height, taa_post_process_params_t* out) {
    if (!out) return fail(TAA_E_INVAL, "taa_post_process_default_params: NULL argument");
    int rc;
    if ((rc = check_size(width, height, "taa_post_process_default_params"))) return rc;
    const uint32_t w = (uint32_t)width, h = (uint32_t)height;
    const int src = (int)std::round((float)w / 96.f);
    const int dst = (int)std::round((float)w / 9.6f);
    const int brd = (int)std::round((float)w / (96.f * 2.f));
    const int32_t zs[4] = {(int32_t)((w - (uint32_t)src) / 2u), (int32_t)((h - (uint32_t)src) / 2u), src, src};
    const int32_t zd[4] = {(int32_t)(w - (uint32_t)dst - (uint32_t)brd), brd, dst, dst};
    for (int i = 0; i < 4; ++i) {
        out->zoom_src_ltwh[i] = zs[i];
        out->zoom_dst_ltwh[i] = zd[i];
        out->debug_l_mask[i] = out->debug_r_mask[i] = i < 3 ? 1.f : 0.f;
    }
    out->zoom = 0;
    out->show_zoom_box = 1;
    out->split_x = -1;
    out->debug_l_show = 0;
    out->debug_r_show = 0;
    return ok();
}

// source/taa.hpp:1141-1158: the post-process dispatch.
int taa_post_process(void* stream, const taa_post_process_params_t* params, const void* input, size_t input_pitch,
                     const void* debug, size_t debug_pitch, void* output, size_t output_pitch, int32_t width,
                     int32_t height) {
    static const char* who = "taa_post_process";
    int rc;
    if ((rc = check_size(width, height, who))) return rc;
    if (!params) return fail(TAA_E_INVAL, "%s: NULL params", who);
    const taa_post_process_params_t& p = *params;
    const int32_t lim = 1 << 24;
    for (int i = 0; i < 4; ++i)
        if (p.zoom_src_ltwh[i] < -lim || p.zoom_src_ltwh[i] > lim || p.zoom_dst_ltwh[i] < -lim ||
            p.zoom_dst_ltwh[i] > lim)
            return fail(TAA_E_INVAL, "%s: zoom box coordinates beyond +-2^24", who);
    if (std::isnan(p.debug_l_mask[3]) || std::isnan(p.debug_r_mask[3]))
        return fail(TAA_E_INVAL, "%s: debug mask .w is NaN", who);
    const bool need_debug = p.debug_l_show || p.debug_r_show;
    const char *ilo = nullptr, *ihi = nullptr, *dlo = nullptr, *dhi = nullptr, *olo = nullptr, *ohi = nullptr;
    if ((rc = check_image("input", input, input_pitch, width, height, 8, true, &ilo, &ihi))) return rc;
    if ((rc = check_image("debug", debug, debug_pitch, width, height, 8, need_debug, &dlo, &dhi))) return rc;
    if ((rc = check_image("output", output, output_pitch, width, height, 8, true, &olo, &ohi))) return rc;
    if (overlaps(ilo, ihi, olo, ohi)) return fail(TAA_E_INVAL, "%s: output overlaps input", who);
    if (debug && overlaps(dlo, dhi, olo, ohi)) return fail(TAA_E_INVAL, "%s: output overlaps debug", who);
    taa_dev::PostArgs a;
    std::memset(&a, 0, sizeof a);
    a.in = Img{(const char*)input, input_pitch, width, height};
    a.debug = Img{(const char*)debug, debug_pitch, width, height};
    a.out = ImgW{(char*)output, output_pitch};
    a.w = width;
    a.h = height;
    for (int i = 0; i < 4; ++i) {
        a.zoom_src[i] = p.zoom_src_ltwh[i];
        a.zoom_dst[i] = p.zoom_dst_ltwh[i];
    }
    a.mask_l_w = p.debug_l_mask[3];
    a.mask_r_w = p.debug_r_mask[3];
    a.zoom = p.zoom != 0;
    a.show_zoom_box = p.show_zoom_box != 0;
    a.split_x = p.split_x;
    a.show_l = p.debug_l_show != 0;
    a.show_r = p.debug_r_show != 0;
    cudaError_t e = taa_dev::launch_post_process(a, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return ok();
}

}  // extern "C"
