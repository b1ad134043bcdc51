// host_util.h - host-side helpers shared by the C ABI units (internal to the library).
#pragma once
#include <cuda_runtime.h>

#include "../../include/taa_gb300.h"
#include "kernels.h"

// A resolve context (taa_create): the description, the uniform block of the
// next resolves, CasSetup constants and the few device buffers it owns.
struct taa_ctx {
    taa_desc_t desc;
    taa_uniforms_t uniforms;
    bool have_uniforms = false;
    uint32_t cas_const0[4] = {0, 0, 0, 0};
    uint32_t cas_const1[4] = {0, 0, 0, 0};
    int device = 0;
    // RGBA16F screen image for the plain form's separate sharpen pass when the
    // caller does not bind a result image; allocated when a sharpener is set.
    void* scratch_screen = nullptr;
    size_t scratch_pitch = 0;
    // the learned form's weights (TAA_FORM_LEARNED): FP32 masters and the FP16 blob
    float* mlp_weights = nullptr;
    char* mlp_blob = nullptr;
    bool have_mlp = false;
    // TAA_FLAG_FXAA: the FXAA pass's work list, a counter then fxaa_cap entries
    uint32_t* fxaa_list = nullptr;
    size_t fxaa_cap = 0;
};

namespace taa_host {

// Records the message of a failing call (taa_last_error) and returns `code`.
int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int cuda_fail(cudaError_t e, const char* what);
bool finite(float v);
int ok();
// Validates one image binding: alignment to the texel, pitch, and (when lo/hi
// are given) the byte range [lo, hi) it spans.  NULL is an error if required.
int check_image(const char* name, const void* p, size_t pitch, int w, int h, size_t texel, bool required,
                const char** lo = nullptr, const char** hi = nullptr);
// Validation of a context description and of a uniform block.
int check_desc(const taa_desc_t& d, const char* who);
int check_uniforms(const taa_uniforms_t& u, const char* who);
// Validates one frame's bindings against a description (sizes, formats,
// alignment, aliasing) and fills the kernel arguments.
int frame_args(const taa_desc_t& d, const taa_uniforms_t& U, uint32_t cas_peak_bits, const taa_frame_io_t* io,
               const char* who, taa_dev::FrameArgs* out);
// Whether the learned form runs these parameters and bindings (TAA_OK, or a
// TAA_E_UNSUPPORTED failure naming what it does not run).
int learned_supported(const taa_desc_t& d, const taa_uniforms_t& U, const taa_frame_io_t* io, const char* who);

}  // namespace taa_host
