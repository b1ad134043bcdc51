/*
 * taa_gb300.h - C ABI of the GB300-native TAA resolve.
 *
 * This library replaces one dispatch of the reference renderer: the compute
 * pass that source/taa.hpp:1008-1027 records for shaders/taa.comp, plus the
 * optional sharpen pass that follows it in the same command buffer
 * (source/taa.hpp:1111-1139, shaders/sharpen.comp and shaders/sharpen_cas.comp),
 * which this library launches after the resolve (or, with
 * TAA_FLAG_FUSED_SHARPEN, in the same launch).  Everything else in the
 * reference (scene rendering, ray tracing, post-process overlay, GUI) stays
 * outside.
 *
 * Conventions
 *  - All images are headless pitched linear device buffers (no Vulkan images,
 *    no samplers).  `pitch` is the row stride in bytes.  Every pointer and
 *    pitch must be a multiple of its texel size, otherwise TAA_E_ALIGN.
 *  - Texel formats follow the reference (shaders/shader_cpu_common.h:61-76):
 *    colour RGBA16F, depth D32F, result/debug RGBA16F, segmask R32UI.
 *    Velocity is RGBA16F in the reference layout (.xy UV-space motion,
 *    .z depth delta, .w mover id) or RG16F (.xy only; .z and .w read as 0).
 *    History is RGBA32F (default; an FP32 accumulator) or RGBA16F (reference).
 *  - Calls are asynchronous on the given CUDA stream (a cudaStream_t passed
 *    as void*; NULL is the legacy default stream).  No call allocates device
 *    memory after taa_create and no resolve call synchronises the host (only
 *    taa_device_status waits for the device), so a sequence of taa_resolve
 *    calls can be captured into a CUDA graph.
 *  - Return value 0 (TAA_OK) on success, a negative taa_status otherwise; the
 *    message of the last failure on the calling thread is in taa_last_error().
 *    The reference has no error path (it asserts, source/taa.hpp:153,237,903).
 *  - One context per stream; different contexts may be used concurrently.
 */
#ifndef TAA_GB300_H
#define TAA_GB300_H

#include <stdint.h>
#include <stddef.h>
#include "taa_params.h"

#ifdef __cplusplus
extern "C" {
#endif

#define TAA_GB300_ABI_VERSION 1

typedef enum taa_status {
    TAA_OK            = 0,
    TAA_E_INVAL       = -1,  /* bad argument: null, size, enum out of range, aliasing */
    TAA_E_ALIGN       = -2,  /* pointer or pitch not a multiple of the texel size */
    TAA_E_CUDA        = -3,  /* a CUDA runtime call failed (message in taa_last_error) */
    TAA_E_TIMEOUT     = -4,  /* a bounded device-side wait gave up */
    TAA_E_UNSUPPORTED = -5,  /* valid request this build does not implement */
    TAA_E_NOMEM       = -6   /* allocation failure in taa_create */
} taa_status;

/* History texel format. */
#define TAA_HISTORY_RGBA32F 0u
#define TAA_HISTORY_RGBA16F 1u
/* Velocity texel format. */
#define TAA_MOTION_RGBA16F  0u
#define TAA_MOTION_RG16F    1u
/* Kernel form. */
#define TAA_FORM_AUTO   0u  /* fastest FP32 form for the parameters: TAA_FORM_FAST where it runs them, else TILED, else PLAIN */
#define TAA_FORM_PLAIN  1u  /* one thread per pixel, FP32, every parameter honoured */
#define TAA_FORM_TILED  2u  /* FP32, CTA tile staged in shared memory; the FP32 shader's bits */
#define TAA_FORM_FP16   3u  /* packed half2 neighbourhood, clip and sharpen; FP32 history and blend */
#define TAA_FORM_LEARNED 4u /* blend weight and clip-box scale from a per-pixel MLP (taa_set_mlp) */
/* FP32 with the arithmetic reassociated: contracted FMAs, the 3x3 moments from
 * row sums a thread's four pixels share, the history rows filtered
 * horizontally once for them, hardware square-root and reciprocal
 * approximations in the variance box and the clip.  Frame error within 1e-4
 * relative L2 of the FP64 oracle and of TAA_FORM_TILED on the benchmark
 * sequences (measured 2e-5 to 6e-5; the exact FP32 form is 1e-5 to 5e-5 from
 * FP64).  It runs the parameter block's rectification modes without a
 * tonemap, shaped neighbourhood, noise, anti-ghosting or ray-trace assist:
 * YCoCg (with or without chroma-axis shrinking) or RGB, the variance or the
 * 3x3 minimum/maximum box, clamp or the clip toward the box centre, the
 * velocity-based alpha, luma weighting and near-clamp reduction of the blend
 * weight, velocity for every pixel, for movers only or reprojection through
 * the matrices, simple velocity sampling, Catmull-Rom or bilinear history, no
 * debug binding.  The
 * benchmark mode (YCoCg, variance, clip, velocity for every pixel) also runs
 * with a fused sharpener, in a batch and with upsampling (taa_uniforms_t
 * mUpsampling, a source no larger than the target on either axis); the other
 * modes run for one view of equal source and target sizes.  Other parameters
 * run in TAA_FORM_TILED.  RGBA32F history, or RGBA16F (the
 * reference's storage; one resolve within 5e-4 of the exact form after the
 * FP16 store) for one view without the one-launch sharpener. */
#define TAA_FORM_FAST   5u
/* taa_desc_t.flags: run the learned form's network on tcgen05 (128-row blocks
 * whose features and activations stay in tensor memory, one thread issuing
 * per CTA, a CTA-wide barrier per layer) instead of per warp with warp-wide
 * MMAs (the default: no block barriers; at 1080p 68 us a frame against 79 us
 * for tcgen05; the same output bits).  Both run the parameters of
 * TAA_FORM_FAST's benchmark mode on its strip body, others on the tiled body. */
#define TAA_FLAG_LEARNED_TCGEN05 0x1u
/* taa_desc_t.flags: taa_create also sets aside the work list of the FXAA pass
 * (taa_fxaa), 4 bytes per output pixel, so that the pass needs one read of
 * the segmentation mask. */
#define TAA_FLAG_FXAA 0x2u
/* taa_desc_t.flags, with TAA_FORM_FP16: a pixel whose clip toward the box
 * centre engages on a box that FP16 cannot resolve (its tightest channel 16
 * times narrower than its widest, as next to a firefly) is finished in FP32
 * from its source texels.  Frame error of one resolve against the FP64
 * oracle below 1e-3 relative L2 on the benchmark scenes (up to 8.6e-3
 * without); a free-running 64-frame 4K chain reaches 1.06e-3 at its last
 * frame.  The form runs slower. */
#define TAA_FLAG_FP16_GUARD 0x4u
/* taa_desc_t.flags, with a sharpener: one launch resolves each tile and the
 * 1-pixel ring around it (recomputing what the neighbouring tiles resolve,
 * bit for bit) and sharpens the tile from shared memory, so the unsharpened
 * image never reaches device memory.  In TAA_FORM_FAST (and AUTO where it
 * selects it) the tiles are 30x14 outputs of 32x16 strip-body regions, and
 * the three images carry the two-pass fast form's bits; in TAA_FORM_TILED
 * the exact form's.  TAA_FORM_FP16 with the flag runs the fast form's kernel
 * where it runs the parameters (there is no FP16 one-launch kernel: on this
 * GPU the fast FP32 form is the faster and the more precise), else the exact
 * form's.  Without the flag the forms launch the resolve, which
 * writes the RGBA16F result image, and then the sharpen pass on it, as the
 * reference dispatches taa.comp and then the sharpener (source/taa.hpp:1027,
 * 1111-1139).  On 2560x1440 with CAS the fused fast form takes 58 us a frame
 * with bilinear history (two passes: 61 us) and 74 us with Catmull-Rom (two
 * passes: 71 us): the ring's 22% more resolves against the result image's
 * round trip. */
#define TAA_FLAG_FUSED_SHARPEN 0x8u
/* Sharpener (taa<CF>::mSharpener, source/taa.hpp:1418). */
#define TAA_SHARPEN_OFF     0u
#define TAA_SHARPEN_SIMPLE  1u  /* shaders/sharpen.comp */
#define TAA_SHARPEN_CAS     2u  /* shaders/sharpen_cas.comp, FidelityFX CAS sharpen-only */

typedef struct taa_ctx taa_ctx;

/* Context description: the image sizes and formats that
 * taa<CF>::set_source_image_views (source/taa.hpp:263-360) derives from the
 * views it is given. */
typedef struct taa_desc_t {
    uint32_t struct_size;     /* sizeof(taa_desc_t) */
    int32_t  in_width;        /* source size: colour, depth, velocity, history depth */
    int32_t  in_height;
    int32_t  out_width;       /* target size: history, result, debug, segmask */
    int32_t  out_height;
    uint32_t history_format;  /* TAA_HISTORY_* */
    uint32_t motion_format;   /* TAA_MOTION_* */
    uint32_t form;            /* TAA_FORM_* */
    uint32_t sharpener;       /* TAA_SHARPEN_* */
    float    sharpen_factor;  /* mSharpenFactor, default 0.5 (source/taa.hpp:1419) */
    uint32_t flags;           /* TAA_FLAG_FXAA; TAA_FLAG_LEARNED_TCGEN05 with TAA_FORM_LEARNED; TAA_FLAG_FP16_GUARD with TAA_FORM_FP16;
                                 TAA_FLAG_FUSED_SHARPEN with a sharpener */
} taa_desc_t;

/* Per-frame bindings; one field pair per descriptor binding of set 0 in
 * shaders/taa.comp:24-38 (bound at source/taa.hpp:1009-1025).  Optional
 * outputs may be NULL; a NULL history reads as zeros (first frame).
 * Pointers are device-accessible memory.  An output the library only
 * writes (sharpened, debug, and result unless a two-pass sharpener reads it
 * back) may be pinned host memory (cudaHostAlloc, or cudaHostRegister with
 * cudaHostRegisterMapped): the kernel's stores then cross the host link
 * directly, which saves the caller a device image and a device-to-host copy
 * (a frame's copy-in on another stream overlaps them). */
typedef struct taa_frame_io_t {
    const void* color;         size_t color_pitch;          /* binding  1 uCurrentFrame    */
    const void* depth;         size_t depth_pitch;          /* binding  2 uCurrentDepth    */
    const void* history;       size_t history_pitch;        /* binding  3 uHistoryFrame    */
    const void* history_depth; size_t history_depth_pitch;  /* binding  4 uHistoryDepth    (depth culling) */
    void*       result;        size_t result_pitch;         /* binding  5 uResultScreen    (optional) */
    void*       debug;         size_t debug_pitch;          /* binding  6 uDebug           (optional) */
    const void* velocity;      size_t velocity_pitch;       /* binding  7 uCurrentVelocity */
    void*       history_out;   size_t history_out_pitch;    /* binding  8 uResultHistory   */
    void*       segmask;       size_t segmask_pitch;        /* binding  9 uSegMask         (optional) */
    const void* material;      size_t material_pitch;       /* binding 10 uCurrentMaterial (optional) */
    const void* prev_material; size_t prev_material_pitch;  /* binding 11 uPreviousMaterial(optional) */
    const void* prev_segmask;  size_t prev_segmask_pitch;   /* binding 12 uPreviousSegMask (optional) */
    const void* uvnrm;         size_t uvnrm_pitch;          /* binding 13 uCurrentUvNrm    (optional) */
    void*       sharpened;     size_t sharpened_pitch;      /* the sharpen pass's output   (RGBA16F, with a sharpener) */
} taa_frame_io_t;

/* Longest list of debug sample offsets (sample distribution 5, taa_settings_t). */
#define TAA_SETTINGS_MAX_SAMPLE_OFFSETS 64

/* Jitter options: the debugging knobs of taa<CF>::get_jitter_offset_for_frame
 * (source/taa.hpp:219-232, members 1404-1407).  Pass NULL for the defaults. */
typedef struct taa_jitter_opts_t {
    int32_t fixed_index;      /* mFixedJitterIndex, -1 = off */
    int32_t slow_motion;      /* mJitterSlowMotion, 1 = off */
    float   rotate_degrees;   /* mJitterRotateDegrees */
    float   extra_scale;      /* mJitterExtraScale, 1 = off */
} taa_jitter_opts_t;

/* ---- library ---------------------------------------------------------- */

/* Version string of the library and its ABI version number. */
const char* taa_version(int* abi_version);

/* Message of the last failing call on this thread ("" if none). */
const char* taa_last_error(void);

/* ---- host-side helpers (no device work) ------------------------------- */

/* Fill `out` with the reference defaults (source/taa.hpp:31-76). */
int taa_default_parameters(taa_parameters_t* out);

/* Jitter offset in NDC for a frame, taa<CF>::get_jitter_offset_for_frame
 * (source/taa.hpp:150-233) with helpers::halton (source/helper_functions.hpp:9-26).
 * sample_distribution: 0 circular quad, 1 uniform-4 helix, 2 Halton(2,3)x8,
 * 3 Halton(2,3)x16, 4 regular 16.  in_width/in_height: source resolution.
 * out_num_samples may be NULL. */
int taa_get_jitter_offset(int32_t sample_distribution, uint64_t frame_id,
                          int32_t in_width, int32_t in_height,
                          const taa_jitter_opts_t* opts,
                          float out_ndc[2], int32_t* out_num_samples);

/* Sample distribution 5 of the same function (source/taa.hpp:207-211): the
 * frame's entry of `count` (1..TAA_SETTINGS_MAX_SAMPLE_OFFSETS) debug sample
 * offsets given in pixels (taa_settings_t.mDebugSampleOffsets), scaled to NDC,
 * then the same debugging knobs. */
int taa_get_jitter_offset_custom(const float (*offsets_px)[2], int32_t count, uint64_t frame_id,
                                 int32_t in_width, int32_t in_height, const taa_jitter_opts_t* opts,
                                 float out_ndc[2]);

/* translate(jitter.x, jitter.y, 0) * proj, taa<CF>::get_jittered_projection_matrix
 * (source/taa.hpp:243-253).  Column-major 4x4. */
int taa_jittered_projection(const float proj[16], const float jitter_ndc[2], float out[16]);

/* The two per-frame matrices of taa<CF>::render (source/taa.hpp:993-994),
 * composed in FP64 and rounded once to FP32:
 *   inv_view_proj  = inverse(proj_cur * view_cur)
 *   hist_view_proj = proj_prev * view_prev
 * All column-major.  Returns TAA_E_INVAL for a singular proj_cur*view_cur. */
int taa_compose_matrices(const double proj_cur[16], const double view_cur[16],
                         const double proj_prev[16], const double view_prev[16],
                         float inv_view_proj[16], float hist_view_proj[16]);

/* FidelityFX CAS constants, CasSetup (shaders/ffx_cas.h:375-394). */
int taa_cas_setup(float sharpness, float in_w, float in_h, float out_w, float out_h,
                  uint32_t const0[4], uint32_t const1[4]);

/* ---- context ----------------------------------------------------------- */

/* Create a context for one resolution/format set
 * (replaces taa<CF>::set_source_image_views + initialize, source/taa.hpp:263,650).
 * Allocates the small device state it needs; nothing is allocated later. */
int taa_create(const taa_desc_t* desc, taa_ctx** out_ctx);
int taa_destroy(taa_ctx* ctx);

/* Copy the uniform block used by the next taa_resolve calls
 * (replaces mUniformsBuffer[i]->fill, source/taa.hpp:995).  Validates enums. */
int taa_set_uniforms(taa_ctx* ctx, const taa_uniforms_t* uniforms);

/* Change the sharpener and its strength (source/taa.hpp:961-966). */
int taa_set_sharpener(taa_ctx* ctx, uint32_t sharpener, float factor);

/* Kernel form actually used for the current uniforms (TAA_FORM_*). */
int taa_selected_form(const taa_ctx* ctx);

/* Enqueue the resolve (and, with a sharpener, the sharpen pass) on `stream`
 * (replaces the dispatch at source/taa.hpp:1027 and the sharpen dispatch at
 * source/taa.hpp:1125/1134).  `io->history` and `io->history_out` must not
 * overlap. */
int taa_resolve(taa_ctx* ctx, void* stream, const taa_frame_io_t* io);

/* ---- passes after the resolve ------------------------------------------- */

/* FXAA settings: the push constants of the FXAA pass (source/taa.hpp:93-98). */
typedef struct taa_fxaa_params_t {
    float subpix;              /* fxaaQualitySubpix, 0.75: amount of sub-pixel aliasing removal */
    float edge_threshold;      /* fxaaQualityEdgeThreshold, 0.116: local contrast needed */
    float edge_threshold_min;  /* fxaaQualityEdgeThresholdMin, 0.0833: trims darks */
} taa_fxaa_params_t;

/* Fill `out` with the reference's FXAA settings (source/taa.hpp:95-97). */
int taa_fxaa_default_params(taa_fxaa_params_t* out);

/* FXAA on the pixels the segmentation mask marks for it: the prepare and the
 * FXAA dispatches of the ray-trace-assist path (source/taa.hpp:1063-1104,
 * shaders/antialias_fxaa_prepare.comp + shaders/antialias_fxaa.comp with
 * FXAA 3.11 quality preset 12) as one pass.  `input`: the RGBA16F result image
 * of a resolve; `segmask`: the R32UI mask the resolve wrote (pixels with
 * (mask & 3) == 1 are antialiased), or NULL to antialias every pixel;
 * `output`: RGBA16F, rgb and the FP16 luma in alpha as the reference's temp
 * image holds them.  All images width x height; `output` must not overlap
 * `input`.  `params` NULL means the defaults.  Enqueued on `stream`.
 * `ctx`: a context created with TAA_FLAG_FXAA whose output size holds at
 * least width x height pixels lends the pass its work list (the pass streams
 * the images once and antialiases the listed pixels after); NULL, or any
 * other context, runs the pass without it (a second read of the mask).  The
 * results are the same.  Calls sharing a context run on one stream. */
int taa_fxaa(taa_ctx* ctx, void* stream, const void* input, size_t input_pitch, const void* segmask,
             size_t segmask_pitch, void* output, size_t output_pitch, int32_t width, int32_t height,
             const taa_fxaa_params_t* params);

/* The sharpen pass on its own (source/taa.hpp:1111-1139): sharpener
 * TAA_SHARPEN_SIMPLE (shaders/sharpen.comp) or TAA_SHARPEN_CAS
 * (shaders/sharpen_cas.comp, CasSetup of `factor` at this size) from an RGBA16F
 * image into another of the same size.  For chains where the sharpener reads
 * another pass's output (after taa_fxaa); taa_resolve runs it otherwise. */
int taa_sharpen(void* stream, uint32_t sharpener, float factor, const void* input, size_t input_pitch, void* output,
                size_t output_pitch, int32_t width, int32_t height);

/* The post-process pass's push constants (push_constants_for_postprocess,
 * source/taa.hpp:101-111; the same 84-byte layout). */
typedef struct taa_post_process_params_t {
    int32_t zoom_src_ltwh[4];  /* zoomSrcLTWH: left, top, width, height of the magnified box */
    int32_t zoom_dst_ltwh[4];  /* zoomDstLTWH: the inset it is drawn into */
    float debug_l_mask[4];     /* debugL_mask (param[0].mDebugMask): .w > 0 shows alpha in red and blue */
    float debug_r_mask[4];     /* debugR_mask (param[1].mDebugMask) */
    uint32_t zoom;             /* draw the inset */
    uint32_t show_zoom_box;    /* outline the magnified box in red */
    int32_t split_x;           /* column of the split line; -1: no split (the left side is the whole image) */
    uint32_t debug_l_show;     /* left of the split: the debug image instead of the input (param[0].mDebugToScreenOutput) */
    uint32_t debug_r_show;     /* right of the split (param[1].mDebugToScreenOutput) */
} taa_post_process_params_t;

/* Fill `out` with the reference's post-process settings for a width x height
 * output: the struct's defaults (source/taa.hpp:101-111) with the zoom boxes
 * that set_source_image_views derives from the size (source/taa.hpp:352-359). */
int taa_post_process_default_params(int32_t width, int32_t height, taa_post_process_params_t* out);

/* The post-process pass (shaders/post_process.comp, source/taa.hpp:1141-1158)
 * from the last image of the chain (`input`, RGBA16F) and the resolve's debug
 * image (`debug`, RGBA16F; may be NULL when neither debug_*_show is set) into
 * `output` (RGBA16F), all width x height.  `output` must not overlap `input`
 * or `debug`.  Box coordinates beyond +-2^24 are rejected (TAA_E_INVAL); the
 * magnified box reads the input clamped to the image where it leaves it (the
 * reference's texelFetch is undefined there).  Enqueued on `stream`. */
int taa_post_process(void* stream, const taa_post_process_params_t* params, const void* input, size_t input_pitch,
                     const void* debug, size_t debug_pitch, void* output, size_t output_pitch, int32_t width,
                     int32_t height);

/* ---- settings files ------------------------------------------------------ */

/* The settings taa<CF> writes to and reads from its .ini file
 * (writeSettingsToIni / readSettingsFromIni, source/taa.hpp:1198-1339): both
 * parameter sets and the members of the sections TAA_Primary and
 * TAA_Postprocess.  Booleans are 0/1. */
typedef struct taa_settings_t {
    taa_parameters_t param[2];          /* [TAA_Param_0], [TAA_Param_1] */
    /* [TAA_Primary] */
    uint32_t mTaaEnabled;
    int32_t  mSampleDistribution;
    int32_t  mSharpener;
    float    mSharpenFactor;
    uint32_t mSplitScreen;
    int32_t  mSplitX;
    int32_t  mFixedJitterIndex;
    float    mJitterExtraScale;
    int32_t  mJitterSlowMotion;
    float    mJitterRotateDegrees;
    uint32_t mResetHistoryOnChange;
    int32_t  mDebugSampleOffsetsCount;  /* 1..TAA_SETTINGS_MAX_SAMPLE_OFFSETS */
    float    mDebugSampleOffsets[TAA_SETTINGS_MAX_SAMPLE_OFFSETS][2];
    /* [TAA_Postprocess] */
    uint32_t mPostProcessEnabled;
    uint32_t zoom;
    uint32_t showZoomBox;
    int32_t  zoomSrcLTWH[4];
    int32_t  zoomDstLTWH[4];
} taa_settings_t;

/* The reference's initial values of every member above (source/taa.hpp:31-76,
 * 101-111 for the post-processing push constants, 1350-1420 for the others). */
int taa_settings_default(taa_settings_t* out);

/* Write the settings as the reference's .ini text: the sections and keys of
 * writeSettingsToIni, keys lower-cased and `key=value` lines as its INI
 * library writes them, numbers formatted like std::to_string (floats with six
 * decimals, as the reference stores them).  The length of the text (without
 * the terminating NUL) goes to *length; with `text` NULL nothing else happens,
 * otherwise the text and a NUL are written if they fit in `capacity` bytes and
 * TAA_E_INVAL is returned (nothing written) if they do not. */
int taa_settings_write_ini(const taa_settings_t* settings, char* text, size_t capacity, size_t* length);

/* Read .ini text (a whole settings file of the reference, or what
 * taa_settings_write_ini wrote) into *settings: every key readSettingsFromIni
 * reads that is present and non-empty overwrites its member; absent keys
 * leave the member as it was; other sections and keys are ignored.  Section
 * and key names match case-insensitively; ';' starts a comment line.  A value
 * that does not start with a number returns TAA_E_INVAL (the reference's
 * std::stoi/stof throw there) and leaves *settings unchanged. */
int taa_settings_read_ini(taa_settings_t* settings, const char* text, size_t length);

/* ---- batches: many views in one persistent launch --------------------------
 * No counterpart in the reference, which resolves one view per dispatch
 * (source/taa.hpp:1027).  A batch holds up to TAA_BATCH_MAX_VIEWS views of any
 * sizes that share the motion format, the interpolation mode and the
 * parameter mode (all views either in the benchmark mode - YCoCg variance
 * clip towards the box centre, velocity for every pixel - or all not); each
 * view keeps RGBA32F history, has equal source and target sizes and no
 * sharpener, and is resolved with the same bits as its own taa_resolve in
 * the form of the batch's tile body (taa_batch_tuning_t.form: TAA_FORM_TILED,
 * or TAA_FORM_FAST for benchmark-mode views of a batch created with
 * TAA_FORM_AUTO or TAA_FORM_FAST).  Per-view arguments (uniform block, bindings, history
 * tensor maps) live in TAA_BATCH_SLOTS device slots: taa_batch_prepare fills
 * a slot, taa_batch_launch resolves every view of a prepared slot with one
 * launch (a persistent grid of SM count x CTAs per SM taking tiles from a job
 * list, or one CTA per tile, as tuned) and does no host work besides it, so a sequence of launches
 * on prepared slots can be captured into a CUDA graph. */
typedef struct taa_batch taa_batch;
#define TAA_BATCH_MAX_VIEWS 255
#define TAA_BATCH_SLOTS 4
/* Job orders. */
#define TAA_SCHEDULE_VIEW_ORDER    0  /* views in the given order, each tile by tile, row by row */
#define TAA_SCHEDULE_LARGEST_FIRST 1  /* views by decreasing pixel count */
#define TAA_SCHEDULE_INTERLEAVED   2  /* one tile of each view in turn */
#define TAA_BATCH_CTA_PER_TILE    -1  /* taa_batch_tuning_t.ctas_per_sm: a grid of one CTA per tile */
typedef struct taa_batch_tuning_t {
    int32_t tile_w, tile_h;  /* TAA_FORM_TILED: 32x8, 16x16, 32x16, 16x8 or 8x8 pixels;
                                TAA_FORM_FAST: 32x16 (four-pixel strips) */
    int32_t schedule;        /* TAA_SCHEDULE_* */
    int32_t ctas_per_sm;     /* persistent grid = SM count x this; 0 = as many as fit;
                                TAA_BATCH_CTA_PER_TILE = one CTA per tile instead */
    float   ms;              /* one launch, as measured by taa_batch_autotune (0 otherwise) */
    int32_t form;            /* the tile body: TAA_FORM_TILED (0 reads as TILED; each view gets the bits of its
                                own taa_resolve in TAA_FORM_TILED) or TAA_FORM_FAST (views in the benchmark mode
                                of a batch created with TAA_FORM_AUTO or TAA_FORM_FAST; the bits of taa_resolve
                                in TAA_FORM_FAST) */
} taa_batch_tuning_t;

/* Create a batch for n views; allocates its device slots and job list. */
int taa_batch_create(const taa_desc_t* descs, int32_t n, taa_batch** out_batch);
int taa_batch_destroy(taa_batch* batch);
/* The uniform block of one view for the next taa_batch_prepare. */
int taa_batch_set_uniforms(taa_batch* batch, int32_t view, const taa_uniforms_t* uniforms);
/* Validate the n bindings in ios[] (as taa_resolve does) and copy every
 * view's arguments into slot `slot` on `stream`.  Waits on the host only while
 * the slot's previous copy is still in flight. */
int taa_batch_prepare(taa_batch* batch, void* stream, int32_t slot, const taa_frame_io_t* ios);
/* Resolve every view of a prepared slot on `stream` (one launch). */
int taa_batch_launch(taa_batch* batch, void* stream, int32_t slot);
/* Time every tile shape (the exact tiles, and the fast strips where the
 * batch's form and parameters allow them) and job order, each with a
 * persistent grid and with one CTA per tile, on a prepared slot (three
 * interleaved rounds of a warm-up and reps launches each, which rewrite the
 * slot's outputs with the same values; a candidate's time is its best round),
 * keep the fastest and return it.  Synchronises the stream. */
int taa_batch_autotune(taa_batch* batch, void* stream, int32_t slot, int32_t reps, taa_batch_tuning_t* best);
int taa_batch_get_tuning(const taa_batch* batch, taa_batch_tuning_t* out);
int taa_batch_set_tuning(taa_batch* batch, const taa_batch_tuning_t* tuning);

/* ---- the learned rectifier (TAA_FORM_LEARNED) -----------------------------
 * No counterpart in the reference.  A per-pixel MLP (32 features -> 32 -> 32
 * -> 2, ReLU; FP16 weights, FP32 accumulation on the tensor cores) predicts
 * the blend weight (sigmoid of output 0) and the scale of the variance clip
 * box (2 to the power of output 1) from the pixel's 3x3 mean, standard
 * deviation, minimum and maximum, history, current colour, velocity length
 * and depth difference (all in YCoCg, normalised by the mean luma).  Where the
 * scale leaves [0.5, 2] the pixel falls back to the plain variance clip with
 * mAlpha; rejected pixels blend with mRejectionAlpha as in the shader.  The
 * form runs YCoCg variance clipping with Catmull-Rom history, RGBA32F
 * history, equal source and target sizes and no sharpener. */
/* Input 31 and hidden unit 31 of each layer are the constant 1 that carries
 * the next layer's bias: rows 31 of w1 and w2, columns 31 of w1, w2 and w3,
 * b1[31] and b2[31] are not weights (ignored; their gradients are zero). */
typedef struct taa_mlp_weights_t {
    float w1[32 * 32], b1[32];  /* layer 1, row-major [out][in] */
    float w2[32 * 32], b2[32];  /* layer 2 */
    float w3[2 * 32], b3[2];    /* output layer: blend weight, log2 box scale */
} taa_mlp_weights_t;

/* One training record: a pixel of a collected frame. */
typedef struct taa_mlp_record_t {
    uint16_t features[32];      /* FP16 bits, as the network reads them */
    float mean[3], sigma[3];    /* 3x3 variance box, YCoCg */
    float history[3], current[3];
    float truth[3];             /* RGB, 64-spp ground truth */
    float gamma, alpha_fixed;   /* mVarClipGamma; the blend weight when bit 0 of flags is set */
    uint32_t flags;             /* bit 0: rejected or reset (the network does not choose alpha) */
    uint32_t key[2];            /* the trainer's collection call (from 0), the pixel's index y * width + x */
} taa_mlp_record_t;

/* Random starting weights (uniform, Glorot scale; seeded) whose outputs
 * start near alpha0 and box scale 1. */
int taa_mlp_init_weights(taa_mlp_weights_t* w, uint64_t seed, float alpha0);
/* Upload the weights of a TAA_FORM_LEARNED context (waits for the copy). */
int taa_set_mlp(taa_ctx* ctx, const taa_mlp_weights_t* w);
/* The network alone: n rows of 32 FP32 features (device memory) -> n x 2
 * FP32 outputs (device memory), with the context's weights. */
int taa_mlp_forward(taa_ctx* ctx, void* stream, const float* features, float* outputs, int32_t n);

/* Training: records are collected while frames are resolved with the plain
 * variance clip, then the network is trained on them with Adam by the
 * library's tensor-core forward and backward kernels. */
typedef struct taa_mlp_trainer taa_mlp_trainer;
int taa_mlp_trainer_create(int32_t capacity, taa_mlp_trainer** out);
int taa_mlp_trainer_destroy(taa_mlp_trainer* tr);
/* Resolve one frame with the plain variance clip (like taa_resolve on `ctx`,
 * which must fit the learned form) and append a record for each pixel whose
 * hash of (seed, x, y) falls in the given fraction; `truth` is the frame's
 * RGBA32F ground truth (device memory, target size). */
int taa_mlp_collect(taa_mlp_trainer* tr, taa_ctx* ctx, void* stream, const taa_frame_io_t* io, const void* truth,
                    size_t truth_pitch, float fraction, uint32_t seed);
/* Records collected so far (capped at the capacity); waits for the device. */
int taa_mlp_record_count(taa_mlp_trainer* tr, int32_t* count);
/* Copy records [first, first + count) to host memory; waits for the device. */
int taa_mlp_records(taa_mlp_trainer* tr, int32_t first, int32_t count, taa_mlp_record_t* out);
/* Sums over records [first, first + count) of the loss and of its gradient
 * with respect to every weight (taa_mlp_weights_t layout).  The loss of a
 * record: its resolved RGB (variance clip with the predicted box scale, blend
 * with the predicted weight) minus the ground truth, squared and summed over
 * the channels.  Waits for the device. */
int taa_mlp_gradients(taa_mlp_trainer* tr, const taa_mlp_weights_t* w, int32_t first, int32_t count,
                      taa_mlp_weights_t* grad, float* loss_sum);
/* `steps` Adam steps (learning rate lr, cosine-decayed to lr / 10 over the
 * run) on batches of `batch` records drawn
 * without replacement from a seeded shuffle, starting from *w; the trained
 * weights are written back to *w, and the mean loss of the first and last
 * batch to *loss_first / *loss_last.  Waits for the device.
 * Deterministic: the shuffle runs over the records ordered by key (whatever
 * order the collection appended them in) and the gradient sums are added in
 * a fixed order, so the same collections (within the capacity), seed and
 * starting weights give the same trained weights bit for bit. */
int taa_mlp_train(taa_mlp_trainer* tr, taa_mlp_weights_t* w, int32_t steps, int32_t batch, float lr, uint64_t seed,
                  float* loss_first, float* loss_last);

/* Bits of the device status word (taa_device_status). */
#define TAA_DEVICE_WINDOW_TIMEOUT 0x1u /* a history-window copy did not land within its bounded wait */

/* Polls of the first bounded wait for a history-window copy; each poll
 * suspends the waiting thread for at most 20 microseconds (about 80 ms in all). */
#define TAA_WINDOW_WAIT_POLLS 4096u

/* Read (and with clear != 0, reset) the device status word of the current
 * device.  Kernels never spin without bound: a wait that gives up sets a bit
 * here and leaves the affected pixels unwritten instead of hanging.  This
 * call waits for the device (a synchronous read); it has no counterpart in
 * the reference, whose shaders do not wait. */
int taa_device_status(uint32_t* bits, int clear);

/* Test hook, no counterpart in the reference: set on the current device how
 * many polls the first wait for a history-window copy makes before it gives
 * up (TAA_WINDOW_WAIT_POLLS by default).  With 0 every such wait gives up at
 * once, so the failure path runs without a fault: the kernel sets
 * TAA_DEVICE_WINDOW_TIMEOUT, waits for the copy a second time (always with the
 * default bound, so no copy is still in flight when the tile's threads
 * leave) and leaves the tile's pixels unwritten.  Applies to resolves
 * enqueued after the call; waits for the device. */
int taa_debug_set_window_wait(uint32_t first_wait_polls);

/* Largest out_width * out_height that taa_resolve_static_scratch accepts when
 * it needs its buffer: one 3840x2160 RGBA16F screen image, 66,355,200 bytes
 * per device, set aside when the CUDA runtime loads the library's device code. */
#define TAA_STATIC_SCRATCH_MAX_TEXELS (3840 * 2160)

/* taa_resolve with the given sharpener, for callers that may not allocate
 * device memory.  No counterpart in the reference: it exists for hosts that
 * own every byte of device memory themselves - an engine that sizes one pool
 * at load time and hands out only images from it (or images imported from
 * Vulkan), or a frame loop where cudaMalloc/cudaFree would stall or
 * synchronise the device.  taa_create with TAA_SHARPEN_OFF allocates no device
 * memory; with a sharpener it allocates the screen image that a resolve
 * hands to the sharpen pass after it when io->result is NULL.  Create the
 * context with TAA_SHARPEN_OFF and name the sharpener here instead: when the
 * call resolves and then sharpens (every form but the tiled form with
 * TAA_FLAG_FUSED_SHARPEN) with no result binding, that screen image lives in
 * a fixed buffer inside the library, and nothing is allocated.  Otherwise the
 * call is taa_resolve with the sharpener given.
 *  - The first call on each device looks the buffer up (cudaGetSymbolAddress,
 *    on the current device); make it before any stream capture.  The address
 *    is kept with the CUDA context it was looked up in: after a
 *    cudaDeviceReset (a new context, into which the runtime loads the
 *    library's device code at another address) the next call looks it up
 *    again, so make that call before any capture too.
 *  - The buffer holds TAA_STATIC_SCRATCH_MAX_TEXELS texels: a call that needs
 *    it for a larger output returns TAA_E_INVAL (bind io->result instead, or
 *    create a tiled-form context with TAA_FLAG_FUSED_SHARPEN, whose single
 *    launch needs no screen image).
 *  - One buffer per device: calls that overlap on the same device (two
 *    streams, or two host threads) race on it.  Calls queued on one stream
 *    do not.
 *  - Nothing needs to start at zero: the resolve writes the whole screen image
 *    before the sharpen pass reads it. */
int taa_resolve_static_scratch(taa_ctx* ctx, void* stream, const taa_frame_io_t* io,
                               uint32_t sharpener, float factor);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* TAA_GB300_H */
