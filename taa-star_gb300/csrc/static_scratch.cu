// static_scratch.cu - the fixed device buffer behind taa_resolve_static_scratch.
//
// When a resolve runs with a sharpener as a pass of its own after it and the
// caller binds no result image, the resolved screen image has to live
// somewhere between the resolve
// kernel and the sharpen kernel.  taa_resolve keeps it in an image the context
// allocates with cudaMallocPitch; taa_resolve_static_scratch keeps it here, in
// a file-scope device array that the CUDA runtime sets aside when it loads this
// library's device code, so that call allocates nothing.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/taa_gb300.h"
#include "kernels.h"

// One RGBA16F screen image of up to TAA_STATIC_SCRATCH_MAX_TEXELS texels.
// Nothing in it has to start at zero: the resolve writes every texel of the
// out_width x out_height image before the sharpen pass reads any.
static __device__ __align__(256) unsigned char screen_scratch[(size_t)TAA_STATIC_SCRATCH_MAX_TEXELS * 8];

namespace taa_dev {

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_lock;
void* g_address[kMaxDevices] = {};
unsigned long long g_context[kMaxDevices] = {};  // id of the context each address belongs to
}  // namespace

// Device address of screen_scratch on the current device.  The first call on
// each device looks it up with cudaGetSymbolAddress (with that device current,
// which loads the device code there if the runtime has not yet); later calls
// return the cached address while the device's context is the same one.  A
// new context (after cudaDeviceReset the runtime creates one, and loads this
// library's device code into it at another address) is looked up again.
cudaError_t static_screen_scratch(void** address, size_t* bytes) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    unsigned long long ctx = 0;
    if ((e = current_context_id(&ctx)) != cudaSuccess) return e;
    std::lock_guard<std::mutex> hold(g_lock);
    if (!g_address[dev] || g_context[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, screen_scratch);
        if (e != cudaSuccess) return e;
        if (!p) return cudaErrorInvalidSymbol;
        g_address[dev] = p;
        g_context[dev] = ctx;
    }
    *address = g_address[dev];
    *bytes = sizeof screen_scratch;
    return cudaSuccess;
}

}  // namespace taa_dev
