// sequence.cpp - drives the C++ mirror of taa<CF> (taa-star_gb300/taa.hpp)
// over a short synthetic sequence, the way the reference's renderer drives
// its taa component each frame (source/main.cpp:4122-4123, taa.hpp:894, 974).
//
//   sequence <width> <height> <frames> [fxaa | post]
// prints one line per frame with the resolve time and the result's mean.
// With "fxaa" the ray-trace-assist path runs: the resolve writes the
// segmentation mask, FXAA antialiases the pixels it marks, then the sharpener
// (source/taa.hpp:1031-1139); the line also counts the marked pixels.  With
// "post" the screen is split, the left side shows the debug image (mode 2)
// and the zoom inset is drawn (source/taa.hpp:1141-1158); the line also
// counts the texels of the split column that are black.
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/taa_synth.h"
#include "../taa.hpp"

int main(int argc, char** argv) {
    const int W = argc > 1 ? atoi(argv[1]) : 320, H = argc > 2 ? atoi(argv[2]) : 180;
    const int N = argc > 3 ? atoi(argv[3]) : 8;
    const bool fxaa = argc > 4 && std::string(argv[4]) == "fxaa";
    const bool post = argc > 4 && std::string(argv[4]) == "post";
    constexpr size_t CF = 3;
    taa_synth_scene_t scene;
    if (taa_synth_default_scene(&scene, W, H, 7) != TAA_OK) return 1;
    scene.radius_min = 4.f;
    scene.radius_max = 24.f;
    std::array<taa_gb300::Image, CF> col, dep, mot;
    for (size_t i = 0; i < CF; ++i) {
        cudaMallocPitch(&col[i].ptr, &col[i].pitch, (size_t)W * 8, H);
        cudaMallocPitch(&dep[i].ptr, &dep[i].pitch, (size_t)W * 4, H);
        cudaMallocPitch(&mot[i].ptr, &mot[i].pitch, (size_t)W * 8, H);
    }
    taa_gb300::taa<CF> taa;
    auto& p = taa.mParameters[0];
    p.mInterpolationMode = 2;
    p.mUseYCoCg = 1;
    p.mVarianceClipping = 1;
    p.mColorClampingOrClipping = 2;
    p.mAlpha = 0.1f;
    p.mUseVelocityVectors = 2;
    if (fxaa) {
        p.mRayTraceAugment = 1;
        p.mRayTraceAugmentFlags = TAA_RTFLAG_OUT | TAA_RTFLAG_DIS | TAA_RTFLAG_DPT | TAA_RTFLAG_LUM | TAA_RTFLAG_FXA;
    }
    taa.mSampleDistribution = 2;
    taa.mSharpener = TAA_SHARPEN_CAS;
    taa.set_source_image_views(W, H, W, H, col, dep, mot, TAA_MOTION_RGBA16F);
    if (post) {
        taa.mParameters[1] = p;
        taa.mSplitScreen = true;  // split at W / 2 (set_source_image_views)
        p.mDebugMode = 2;
        p.mDebugScale = 1.f;
        p.mDebugToScreenOutput = 1;
        taa.mPostProcessPushConstants.zoom = 1;
    }
    cudaStream_t s;
    cudaStreamCreate(&s);
    std::vector<__half> host((size_t)W * H * 4);
    std::vector<uint32_t> mask((size_t)W * H);
    for (int f = 0; f < N; ++f) {
        const size_t i = f % CF;
        taa_synth_frame_t out{col[i].ptr, col[i].pitch, dep[i].ptr, dep[i].pitch, mot[i].ptr, mot[i].pitch, 4,
                              nullptr, 0};
        scene.jitter_phase = 0;
        if (taa_synth_render(&scene, f, s, &out) != TAA_OK) return 2;
        double proj[16], view[16];
        taa_synth_camera(&scene, f, proj, view);
        taa_gb300::Mat4 P, V;
        for (int k = 0; k < 16; ++k) {
            P.m[k] = proj[k];
            V.m[k] = view[k];
        }
        (void)taa.get_jittered_projection_matrix(P, f);
        taa.save_history_proj_matrix(P, f);
        taa.update(V, f, f / 60.0);
        taa.render(f, s);
        const taa_gb300::Image& r = taa.result(f);
        cudaMemcpy2DAsync(host.data(), (size_t)W * 8, r.ptr, r.pitch, (size_t)W * 8, H, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        double sum = 0;
        for (size_t k = 0; k < host.size(); k += 4) sum += __half2float(host[k]);
        long marked = 0, split_black = 0;
        if (post) {
            for (int y = 0; y < H; ++y) {
                const __half* t = &host[((size_t)y * W + W / 2) * 4];
                split_black += __half2float(t[0]) == 0.f && __half2float(t[1]) == 0.f && __half2float(t[2]) == 0.f;
            }
        }
        if (fxaa && f > 0) {
            const taa_gb300::Image& m = taa.segmentation_mask(f);
            cudaMemcpy2D(mask.data(), (size_t)W * 4, m.ptr, m.pitch, (size_t)W * 4, H, cudaMemcpyDeviceToHost);
            for (uint32_t v : mask) marked += (v & 3u) == 1u;
        }
        printf("frame %d resolve %.3f ms marked %ld split_black %ld mean_r %.5f\n", f, taa.duration(), marked,
               split_black, sum / (W * H));
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        printf("cuda error %s\n", cudaGetErrorString(e));
        return 3;
    }
    return 0;
}
