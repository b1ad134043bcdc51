/*
 * taa_synth.h - seeded analytic scene renderer that feeds the resolve.
 *
 * The reference renders its TAA inputs with a Vulkan rasteriser
 * (source/main.cpp, shaders/fwd_geometry.frag).  This library replaces that
 * with an analytic scene so that every input is exact and reproducible:
 *   - a fronto-parallel backdrop textured with a checkerboard (period
 *     `checker_period` px) times a zone-plate chirp, seen by a camera that
 *     pans by cam(t) = cam_v0*t + 0.5*cam_accel*t^2 px;
 *   - `num_spheres` shaded, striped spheres (movers) with screen velocities,
 *     radii, depths and optional spin about the view axis;
 *   - `firefly_fraction` of the pixels replaced by white fireflies of
 *     radiance in [4, firefly_max];
 *   - Halton(2,3) sub-pixel jitter of period 8 (taa.hpp:195-198) with a
 *     per-view phase.
 * Colour is RGBA16F HDR, depth D32F (Vulkan [0,1], near 0.1, far 1000),
 * motion follows the reference convention (shaders/fwd_geometry.frag:288-295):
 * UV-space, unjittered, history_uv = uv - motion.xy, .z depth delta (0 here:
 * all motion is parallel to the image plane), .w mover id (0 backdrop,
 * sphere index + 1).  Ground truth is the clean (firefly-free) radiance box-
 * filtered over the pixel with 8x8 stratified samples (64 spp).
 *
 * This renderer has no reference counterpart; it is the project's own input
 * generator.  All entry points here are test/benchmark infrastructure next
 * to the drop-in boundary in taa_gb300.h.
 */
#ifndef TAA_SYNTH_H
#define TAA_SYNTH_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct taa_synth_scene_t {
    uint32_t struct_size;      /* sizeof(taa_synth_scene_t) */
    int32_t  width, height;
    uint64_t seed;
    int32_t  num_spheres;      /* <= TAA_SYNTH_MAX_SPHERES */
    float    radius_min, radius_max;  /* px */
    float    sphere_speed_max; /* |v| components uniform in [-max, max] px/frame */
    float    spin_max;         /* spin uniform in [-max, max] rad/frame */
    float    cam_v0[2];        /* px/frame */
    float    cam_accel[2];     /* px/frame^2 */
    float    checker_period;   /* px */
    float    firefly_fraction;
    float    firefly_max;
    int32_t  jitter_phase;     /* Halton index offset */
    int32_t  jitter_enabled;   /* 0: no jitter */
} taa_synth_scene_t;

#define TAA_SYNTH_MAX_SPHERES 256
/* floats per sphere in the sphere table: cx, cy, r, zc, albedo rgb, vx, vy, spin, stripe period, pad */
#define TAA_SYNTH_SPHERE_FLOATS 12

/* Outputs of one frame; any pointer may be NULL.  Pitches in bytes. */
typedef struct taa_synth_frame_t {
    void* color;     size_t color_pitch;     /* RGBA16F */
    void* depth;     size_t depth_pitch;     /* D32F */
    void* motion;    size_t motion_pitch;    /* RG16F or RGBA16F per motion_channels */
    int32_t motion_channels;                 /* 2 or 4 */
    void* truth;     size_t truth_pitch;     /* RGBA32F, 64-spp clean radiance */
} taa_synth_frame_t;

/* Defaults of the 720p configuration (checker 7.3 px, 32 spheres r 20-120 px,
 * |v| <= 6 px/frame, pan 3 px/frame, 1 % fireflies up to 64). */
int taa_synth_default_scene(taa_synth_scene_t* out, int32_t width, int32_t height, uint64_t seed);

/* Sphere table derived from the seed (host only, deterministic). */
int taa_synth_spheres(const taa_synth_scene_t* scene, float* table, int32_t capacity);

/* Jitter of frame t in pixels (x, y) and in NDC (x, y). */
int taa_synth_jitter(const taa_synth_scene_t* scene, int32_t frame, float out_px[2], float out_ndc[2]);

/* Camera matrices of frame t (column-major, FP64): unjittered projection and
 * view, consistent with the backdrop's pan so that matrix reprojection
 * (taa.comp:426-430) lands the backdrop exactly. */
int taa_synth_camera(const taa_synth_scene_t* scene, int32_t frame, double proj[16], double view[16]);

/* Render frame t on the GPU into device buffers (asynchronous on stream). */
int taa_synth_render(const taa_synth_scene_t* scene, int32_t frame, void* stream, const taa_synth_frame_t* out);

#ifdef __cplusplus
}
#endif

#endif /* TAA_SYNTH_H */
