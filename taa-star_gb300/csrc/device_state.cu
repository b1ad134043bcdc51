// device_state.cu - per-device state of the library and the host side of its
// TMA copies.
//
//  * the device status word: kernels that wait on an mbarrier give up after a
//    bounded number of polls and set a bit here instead of hanging; the host
//    reads it with taa_device_status (include/taa_gb300.h).  The word after
//    it holds the poll count of the first window wait (a test hook);
//  * the id of the current CUDA context (cuCtxGetId), with which the host
//    keeps addresses of __device__ variables valid across cudaDeviceReset;
//  * tensor maps for the history window copy (cp.async.bulk.tensor), encoded
//    through the driver's cuTensorMapEncodeTiled, reached with
//    cudaGetDriverEntryPointByVersion so the library needs no link to libcuda.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/taa_gb300.h"
#include "kernels.h"

// [0]: the status bits; [1]: polls of the first bounded wait for a
// history-window copy (taa_debug_set_window_wait)
static __device__ unsigned int status_word[2] = {0u, TAA_WINDOW_WAIT_POLLS};

namespace taa_dev {

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_lock;
// the status word's address per device, with the id of the context it was looked up in
unsigned int* g_status[kMaxDevices] = {};
unsigned long long g_status_ctx[kMaxDevices] = {};
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
bool g_encode_looked_up = false;
using PFN_ctx_get_current = CUresult (*)(CUcontext*);
using PFN_ctx_get_id = CUresult (*)(CUcontext, unsigned long long*);
PFN_ctx_get_current g_ctx_get_current = nullptr;
PFN_ctx_get_id g_ctx_get_id = nullptr;
bool g_ctx_looked_up = false;
}  // namespace

cudaError_t current_context_id(unsigned long long* id) {
    {
        std::lock_guard<std::mutex> hold(g_lock);
        if (!g_ctx_looked_up) {
            g_ctx_looked_up = true;
            cudaDriverEntryPointQueryResult q{};
            void* fn = nullptr;
            if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) == cudaSuccess &&
                q == cudaDriverEntryPointSuccess)
                g_ctx_get_current = reinterpret_cast<PFN_ctx_get_current>(fn);
            fn = nullptr;
            if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
                q == cudaDriverEntryPointSuccess)
                g_ctx_get_id = reinterpret_cast<PFN_ctx_get_id>(fn);
        }
    }
    if (!g_ctx_get_current || !g_ctx_get_id) return cudaErrorNotSupported;
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
    if (!ctx) {
        // no context yet on this thread (nothing has touched the device, or
        // cudaDeviceReset destroyed it): the runtime makes the device's
        // primary context current.  Queries of an existing context stay free
        // of runtime calls that stream capture forbids.
        const cudaError_t e = cudaFree(nullptr);
        if (e != cudaSuccess) return e;
        if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return cudaErrorDeviceUninitialized;
    }
    return g_ctx_get_id(ctx, id) == CUDA_SUCCESS ? cudaSuccess : cudaErrorDeviceUninitialized;
}

// The status word's device address, looked up again whenever the current
// context is not the one of the cached address (after cudaDeviceReset the
// module is loaded anew, at another address).
cudaError_t device_status_word(unsigned int** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    unsigned long long ctx = 0;
    if ((e = current_context_id(&ctx)) != cudaSuccess) return e;
    std::lock_guard<std::mutex> hold(g_lock);
    if (!g_status[dev] || g_status_ctx[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, status_word);
        if (e != cudaSuccess) return e;
        g_status[dev] = static_cast<unsigned int*>(p);
        g_status_ctx[dev] = ctx;
    }
    *out = g_status[dev];
    return cudaSuccess;
}

bool encode_history_map(const Img& h, int history_fmt, int box_w, int box_h, CUtensorMap* map) {
    {
        std::lock_guard<std::mutex> hold(g_lock);
        if (!g_encode_looked_up) {
            g_encode_looked_up = true;
            cudaDriverEntryPointQueryResult q{};
            void* fn = nullptr;
            if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                    cudaSuccess &&
                q == cudaDriverEntryPointSuccess)
                g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        }
    }
    if (!g_encode || !h.p) return false;
    // a TMA source must start on a 16-byte boundary with rows a multiple of 16 bytes apart
    if (reinterpret_cast<uintptr_t>(h.p) % 16 != 0 || h.pitch % 16 != 0) return false;
    const cuuint32_t elem[3] = {1, 1, 1};
    CUresult r;
    if (history_fmt == 0) {
        // RGBA32F as (channel, x, y): the innermost box extent is one 16-byte texel
        const cuuint64_t dim[3] = {4, (cuuint64_t)h.w, (cuuint64_t)h.h};
        const cuuint64_t stride[2] = {16, (cuuint64_t)h.pitch};
        const cuuint32_t box[3] = {4, (cuuint32_t)box_w, (cuuint32_t)box_h};
        r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<char*>(h.p), dim, stride, box, elem,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    } else if (history_fmt == 2) {
        // RGBA32F as (float, y): a box row of box_w texels is one contiguous
        // run of 16 * box_w bytes (the x coordinate, 4 floats per texel, is
        // always a 16-byte multiple), fetched as a few wide requests instead
        // of one 16-byte request per texel
        if (4 * box_w > 256) return false;
        const cuuint64_t dim[2] = {4 * (cuuint64_t)h.w, (cuuint64_t)h.h};
        const cuuint64_t stride[1] = {(cuuint64_t)h.pitch};
        const cuuint32_t box[2] = {(cuuint32_t)(4 * box_w), (cuuint32_t)box_h};
        r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<char*>(h.p), dim, stride, box, elem,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    } else {
        // RGBA16F as (half, y): a box row of box_w texels is 8 * box_w bytes,
        // and the x coordinate (4 halves per texel) must be a multiple of 8
        // halves, so box_w and the window origin are even
        if (box_w % 2 != 0 || 4 * box_w > 256) return false;
        const cuuint64_t dim[2] = {4 * (cuuint64_t)h.w, (cuuint64_t)h.h};
        const cuuint64_t stride[1] = {(cuuint64_t)h.pitch};
        const cuuint32_t box[2] = {(cuuint32_t)(4 * box_w), (cuuint32_t)box_h};
        r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<char*>(h.p), dim, stride, box, elem,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    }
    return r == CUDA_SUCCESS;
}

}  // namespace taa_dev
