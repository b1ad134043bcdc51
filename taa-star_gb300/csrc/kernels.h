// kernels.h - launchers of the device kernels (internal to the library).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include "common.cuh"
#include "f32x2.cuh"
#include "../../include/taa_synth.h"

namespace taa_dev {

// Plain FP32 resolve (resolve_plain.cu).
cudaError_t launch_resolve_plain(const taa_uniforms_t& U, const FrameArgs& a, int history_format,
                                 int motion_channels, cudaStream_t stream);

// Parameters the fast forms specialise on at compile time; everything else in
// the parameter block stays a runtime value.
struct FastKey {
    int form;          // TAA_FORM_TILED or TAA_FORM_FP16
    int history_fmt;   // 0 RGBA32F, 1 RGBA16F
    int motion_ch;     // 2 or 4
    int interp;        // 0 bilinear, 1 b-spline, 2 Catmull-Rom
    int sharpen;       // 0 off, 1 simple, 2 CAS (fused epilogue)
};

// Whether the tiled forms run these parameters and sizes.  The ray-trace-assist
// classification only where rt_augment_ok (the tiled forms without a fused
// sharpener run it; the batch, the learned form and the fused sharpener do
// not); noise, dynamic anti-ghosting and the 3x3-longest velocity only where
// extra_modes_ok (the tiled forms without a fused sharpener and the batch).
bool fast_path_supported(const taa_uniforms_t& U, int in_w, int in_h, int out_w, int out_h, bool rt_augment_ok = false,
                         bool extra_modes_ok = false);
// Whether the tiled FP32 form's upsampling path (tiled_up.cuh) runs these
// parameters and sizes: TAAU (mUpsampling) from a source no larger than the
// target in either axis, simple velocity sampling, no anti-ghosting, no
// segmentation mask, no split screen, pass-through or bypass, and an
// unjittered neighbourhood only with a zero jitter.
bool up_path_supported(const taa_uniforms_t& U, int in_w, int in_h, int out_w, int out_h);

// The reassociating FP32 resolve, TAA_FORM_FAST (resolve_fast32.cu): whether
// it runs these parameters, sizes and history format, and its launch.
bool fast32_supported(const taa_uniforms_t& U, int history_fmt, int in_w, int in_h, int out_w, int out_h);
// TAA_FORM_FAST for one view without a fused sharpener: the benchmark mode or
// the reference's default mode (RGB, minimum/maximum box, clamp, any velocity
// use), RGBA32F or RGBA16F history.
bool fast32_single_supported(const taa_uniforms_t& U, int history_fmt, int in_w, int in_h, int out_w, int out_h);
// TAA_FORM_FAST for upsampling (TAAU) in the benchmark mode, RGBA32F history.
bool fast32_up_supported(const taa_uniforms_t& U, int history_fmt, int in_w, int in_h, int out_w, int out_h);
cudaError_t launch_resolve_fast32_up(int motion_ch, const taa_uniforms_t& U, const FrameArgs& f, cudaStream_t s);
// TAA_FORM_FAST for the other rectification modes (YCoCg or RGB, variance or
// min/max box, clamp or clip toward the centre, any velocity use), one view,
// RGBA32F history, no fused sharpener.
bool fast32_gen_mode(const taa_parameters_t& P);
bool fast32_gen_supported(const taa_uniforms_t& U, int history_fmt, int in_w, int in_h, int out_w, int out_h);
cudaError_t launch_resolve_fast32_gen(int motion_ch, const taa_uniforms_t& U, const FrameArgs& f, cudaStream_t s);
cudaError_t launch_resolve_fast32(int motion_ch, int history_fmt, const taa_uniforms_t& U, const FrameArgs& f,
                                  cudaStream_t s);
// TAA_FORM_FAST and the sharpener (TAA_SHARPEN_SIMPLE or TAA_SHARPEN_CAS) in
// one launch: result (if bound), history and sharpened as the two-pass form.
cudaError_t launch_resolve_fast32_sharpen(int motion_ch, int sharpener, const taa_uniforms_t& U, const FrameArgs& f,
                                          cudaStream_t s);
// The same tile body over many views (resolve_fast32.cu): the history window
// (texels) its 2-D tensor maps cover, its occupancy and its launch (the batch
// arguments as for launch_batch, one CTA of 128 threads per 32x16 tile).
void fast32_window(int* w, int* h);
cudaError_t fast32_batch_occupancy(int interp, int motion_ch, int* ctas_per_sm);
cudaError_t launch_fast32_batch(int interp, int motion_ch, const BatchView* views, const CUtensorMap* maps,
                                const int* tma_ok, const uint32_t* jobs, int njobs, int grid, cudaStream_t stream);

// Tiled FP32 / FP16 resolve, optionally with the fused sharpen (resolve_fast.cu).
cudaError_t launch_resolve_fast(const FastKey& key, const taa_uniforms_t& U, const FrameArgs& a,
                                cudaStream_t stream);

// Tiled resolve without a fused sharpener: exact FP32 (resolve_tiled.cu) and
// packed FP16 neighbourhood (resolve_half.cu), sharing tiled_skeleton.cuh.
cudaError_t launch_resolve_tiled(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U,
                                 const FrameArgs& a, cudaStream_t stream);
cudaError_t launch_resolve_half(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U,
                                const FrameArgs& a, cudaStream_t stream);
// The FP16 form with TAA_FLAG_FP16_GUARD (resolve_half_guard.cu).
cudaError_t launch_resolve_half_guarded(int history_fmt, int motion_ch, int interp, const taa_uniforms_t& U,
                                        const FrameArgs& a, cudaStream_t stream);

// Standalone sharpen passes on an RGBA16F image (used after the plain form).
cudaError_t launch_sharpen(int sharpener, const FrameArgs& a, cudaStream_t stream);
// The FXAA pass (prepare + FXAA 3.11 quality preset 12) on an RGBA16F image;
// segmask.p == nullptr marks every pixel.  `list`: a work list of a counter
// (padded to 16 bytes) and in.w * in.h entries, or nullptr.
cudaError_t launch_fxaa(const Img& in, const Img& segmask, const ImgW& out, const float rcp[2], float subpix,
                        float edge_threshold, float edge_threshold_min, uint32_t* list, cudaStream_t stream);

// The post-process pass (post_process.cu) on RGBA16F images of w x h texels.
struct PostArgs {
    Img in, debug;  // debug.p may be null when neither side shows it
    ImgW out;
    int w, h;
    int zoom_src[4], zoom_dst[4];  // left, top, width, height
    float mask_l_w, mask_r_w;      // .w of each side's debug mask
    int zoom, show_zoom_box, split_x, show_l, show_r;
};
cudaError_t launch_post_process(const PostArgs& a, cudaStream_t stream);

// Device address and size of the fixed screen buffer of static_scratch.cu on
// the current device (looked up once per device).
cudaError_t static_screen_scratch(void** address, size_t* bytes);

// Address of the device status word on the current device (device_state.cu).
cudaError_t device_status_word(unsigned int** out);
// Id of the current CUDA context (cuCtxGetId): unique for the process's
// lifetime, so a cached device address can be checked against the context
// it was looked up in.
cudaError_t current_context_id(unsigned long long* id);

// Tensor map of a history image for box_w x box_h texel window copies;
// false when the image cannot be a TMA source (alignment, driver entry point).
// history_fmt 0: RGBA32F as (channel, x, y); 1: RGBA16F as (half, y);
// 2: RGBA32F as (float, y), rows of the box copied as contiguous runs.
bool encode_history_map(const Img& history, int history_fmt, int box_w, int box_h, CUtensorMap* map);

// The batched persistent resolve (batch_tiled.cu).
struct BatchKey {
    int shape;        // tile shape id: 0 32x8, 1 16x16, 2 32x16, 3 16x8, 4 8x8 (the exact FP32 tiles);
                      // 5 32x16 in four-pixel strips (TAA_FORM_FAST's body)
    int history_fmt;  // 0 (RGBA32F) only
    int motion_ch;    // 2 or 4
    int interp;       // 0 bilinear or 2 Catmull-Rom
    int hot;          // the benchmark-mode specialisation (tiled::is_hot)
};
struct BatchShapeInfo {
    int tile_w, tile_h, threads;
    int win_w, win_h;  // history window (texels) = the TMA box
};
constexpr int kBatchShapes = 6;
constexpr int kBatchFastShape = 5;
bool batch_shape_info(int shape, int history_fmt, BatchShapeInfo* out);
cudaError_t batch_occupancy(const BatchKey& k, int* ctas_per_sm);
cudaError_t launch_batch(const BatchKey& k, const BatchView* views, const CUtensorMap* maps, const int* tma_ok,
                         const uint32_t* jobs, int njobs, int grid, cudaStream_t stream);
// True when the parameters select the benchmark-mode specialisation.
bool hot_parameters(const taa_parameters_t& P);

// The learned rectifier (learned.cu).
size_t learned_record_bytes();
int learned_param_count();
int learned_blob_bytes();
cudaError_t launch_mlp_build_blob(const float* weights, char* blob, cudaStream_t s);
cudaError_t launch_mlp_map_grads(float* grads, cudaStream_t s);
cudaError_t launch_mlp_forward(const char* blob, const float* feat, float* out, int n, unsigned int* status,
                               cudaStream_t s);
// Training over records [first, first + count) (in `order` when given): each of
// the `grid` CTAs writes its gradient sums to its slab of `partial` (grid x
// learned_grad_floats() floats), which are then added to `grads` in CTA order,
// so the result does not depend on scheduling.
int learned_grad_floats();
cudaError_t launch_mlp_train(const char* blob, const void* records, const uint32_t* order, int first, int count,
                             float* grads, float* partial, unsigned int* status, int grid, cudaStream_t s);
cudaError_t launch_mlp_adam(float* weights, float* m, float* v, float* grads, int step, float lr, char* blob,
                            cudaStream_t s);
cudaError_t launch_resolve_learned(int history_fmt, int motion_ch, bool collect, bool tcgen05, const taa_uniforms_t& U,
                                   const FrameArgs& a, const char* blob, void* records, uint32_t* count,
                                   uint32_t capacity, uint32_t seed, uint32_t call, float sample_fraction,
                                   const Img& truth,
                                   cudaStream_t s);

// The learned form's inference in the benchmark mode on the strip body
// (resolve_learned_strips.cu); `blob` is the network's device blob.
cudaError_t launch_resolve_learned_strips_tc(int motion_ch, const taa_uniforms_t& U, const FrameArgs& f,
                                             const char* blob, cudaStream_t s);
cudaError_t launch_resolve_learned_strips(int motion_ch, const taa_uniforms_t& U, const FrameArgs& a, const char* blob,
                                          cudaStream_t s);

// Synthetic renderer (synth.cu).
cudaError_t launch_synth(const taa_synth_scene_t& s, const float* host_spheres, int frame,
                         const taa_synth_frame_t& out, cudaStream_t stream);

}  // namespace taa_dev
