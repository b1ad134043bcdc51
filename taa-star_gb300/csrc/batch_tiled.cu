// batch_tiled.cu - the batched resolve: many views of any size in one
// persistent launch of the tiled FP32 form (tiled_skeleton.cuh, resolve_batch),
// for each tile shape the autotuner chooses from.  Compiled with -fmad=false,
// so every view gets the same bits as its own taa_resolve in TAA_FORM_TILED.
// Shape 5 dispatches to TAA_FORM_FAST's strip body (resolve_fast32.cu), whose
// views get the bits of their own taa_resolve in TAA_FORM_FAST.
#include "kernels.h"
#include "policy_f32.cuh"

namespace taa_dev {

namespace {
using tiled::ExactF32;
using tiled::Shape;

// tile shapes by id (include/taa_gb300.h lists them for the tuning record)
using S0 = Shape<32, 8>;
using S1 = tiled::MultiShape<16, 8, 2>;  // 16x16, two pixels per thread
using S2 = tiled::MultiShape<32, 8, 2>;  // 32x16, two pixels per thread
using S3 = Shape<16, 8>;
using S4 = Shape<8, 8>;

template <class S, int MC, int INTERP, bool HOT>
const void* kernel_of() {
    return reinterpret_cast<const void*>(&tiled::resolve_batch<ExactF32, S, 0, MC, INTERP, HOT>);
}

// Calls f(S{}, kernel) for the instantiation the key names; false if none.
template <class S, class F>
bool with_shape(const BatchKey& k, F&& f) {
    const bool hot = k.hot != 0;
    const void* fn = nullptr;
    if (k.motion_ch == 4) {
        if (k.interp == 2) fn = hot ? kernel_of<S, 4, 2, true>() : kernel_of<S, 4, 2, false>();
        else if (k.interp == 0) fn = hot ? kernel_of<S, 4, 0, true>() : kernel_of<S, 4, 0, false>();
    } else if (k.motion_ch == 2) {
        if (k.interp == 2) fn = hot ? kernel_of<S, 2, 2, true>() : kernel_of<S, 2, 2, false>();
        else if (k.interp == 0) fn = hot ? kernel_of<S, 2, 0, true>() : kernel_of<S, 2, 0, false>();
    }
    if (!fn) return false;
    f(S{}, fn);
    return true;
}
template <class F>
bool with_kernel(const BatchKey& k, F&& f) {
    if (k.history_fmt != 0) return false;
    switch (k.shape) {
        case 0: return with_shape<S0>(k, f);
        case 1: return with_shape<S1>(k, f);
        case 2: return with_shape<S2>(k, f);
        case 3: return with_shape<S3>(k, f);
        case 4: return with_shape<S4>(k, f);
        default: return false;
    }
}
}  // namespace

bool hot_parameters(const taa_parameters_t& P) { return tiled::is_hot(P); }

bool batch_shape_info(int shape, int history_fmt, BatchShapeInfo* out) {
    if (shape == kBatchFastShape) {
        if (history_fmt != 0) return false;
        out->tile_w = 32;
        out->tile_h = 16;
        out->threads = 128;
        fast32_window(&out->win_w, &out->win_h);
        return true;
    }
    BatchKey k{shape, history_fmt, 2, 2, 1};
    return with_kernel(k, [&](auto s, const void*) {
        using S = decltype(s);
        out->tile_w = S::TX;
        out->tile_h = S::TY;
        out->threads = S::NT;
        out->win_w = tiled::Win<S, 0>::W;
        out->win_h = S::WH;
    });
}

cudaError_t batch_occupancy(const BatchKey& k, int* ctas_per_sm) {
    if (k.shape == kBatchFastShape) {
        if (k.history_fmt != 0 || !k.hot) return cudaErrorInvalidValue;
        return fast32_batch_occupancy(k.interp, k.motion_ch, ctas_per_sm);
    }
    cudaError_t e = cudaErrorInvalidValue;
    with_kernel(k, [&](auto s, const void* fn) {
        using S = decltype(s);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, S::NT, 0);
    });
    return e;
}

cudaError_t launch_batch(const BatchKey& k, const BatchView* views, const CUtensorMap* maps, const int* tma_ok,
                         const uint32_t* jobs, int njobs, int grid, cudaStream_t stream) {
    if (k.shape == kBatchFastShape) {
        if (k.history_fmt != 0 || !k.hot) return cudaErrorInvalidValue;
        return launch_fast32_batch(k.interp, k.motion_ch, views, maps, tma_ok, jobs, njobs, grid, stream);
    }
    cudaError_t e = cudaErrorInvalidValue;
    with_kernel(k, [&](auto s, const void* fn) {
        using S = decltype(s);
        void* args[] = {(void*)&views, (void*)&maps, (void*)&tma_ok, (void*)&jobs, (void*)&njobs};
        e = cudaLaunchKernel(fn, dim3(grid), dim3(S::NT), args, 0, stream);
    });
    return e;
}

}  // namespace taa_dev
