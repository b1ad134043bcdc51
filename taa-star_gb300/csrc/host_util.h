// host_util.h - host-side helpers shared by the C ABI units (internal to the library).
#pragma once
#include <cuda_runtime.h>

#include "../../include/taa_gb300.h"
#include "kernels.h"

namespace taa_host {

// Records the message of a failing call (taa_last_error) and returns `code`.
int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int cuda_fail(cudaError_t e, const char* what);
bool finite(float v);
// Validation of a context description and of a uniform block.
int check_desc(const taa_desc_t& d, const char* who);
int check_uniforms(const taa_uniforms_t& u, const char* who);
// Validates one frame's bindings against a description (sizes, formats,
// alignment, aliasing) and fills the kernel arguments.
int frame_args(const taa_desc_t& d, const taa_uniforms_t& U, uint32_t cas_peak_bits, const taa_frame_io_t* io,
               const char* who, taa_dev::FrameArgs* out);

}  // namespace taa_host
