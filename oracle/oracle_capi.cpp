// oracle_capi.cpp - C entry points of the oracle for the test harness (ctypes).
//
// THIS IS THE ORACLE (test infrastructure): only tests, the smoke check and
// the benchmark's CPU-baseline leg load it, as the checker.
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "taa_oracle.hpp"
#include "../include/taa_synth.h"
#include "../taa-star_gb300/csrc/synth_scene.h"

using namespace taa_oracle;

extern "C" {

int oracle_resolve(int precision, const taa_uniforms_t* u, int in_w, int in_h, int out_w, int out_h,
                   const float* color, const float* depth, const float* history, const float* history_depth,
                   const float* velocity4, const uint32_t* material, const uint32_t* prev_material,
                   const uint32_t* prev_segmask, const float* uvnrm, double* out_history, double* out_screen,
                   double* out_debug, uint32_t* out_segmask, int nthreads) {
    if (!u) return -1;
    ResolveInputs in;
    in.color = {color, in_w, in_h, 4};
    in.depth = {depth, in_w, in_h, 1};
    in.history = {history, out_w, out_h, 4};
    in.history_depth = {history_depth, in_w, in_h, 1};
    in.velocity = {velocity4, in_w, in_h, 4};
    in.material = {material, in_w, in_h};
    in.prev_material = {prev_material, in_w, in_h};
    in.prev_segmask = {prev_segmask, out_w, out_h};
    in.uvnrm = {uvnrm, in_w, in_h, 4};
    in.out_w = out_w;
    in.out_h = out_h;
    ResolveOutputs out{out_history, out_screen, out_debug, out_segmask};
    return resolve(precision, *u, in, out, nthreads);
}

int oracle_cas(int precision, const float* in, int w, int h, uint32_t peak_bits, double* out, int nthreads) {
    return cas(precision, in, w, h, peak_bits, out, nthreads);
}

int oracle_sharpen(int precision, const float* in, int w, int h, float factor, double* out, int nthreads) {
    return sharpen(precision, in, w, h, factor, out, nthreads);
}

int oracle_fxaa(int precision, const float* in, const uint32_t* segmask, int w, int h, float rcp_x, float rcp_y,
                float subpix, float thr, float thr_min, double* out, int nthreads) {
    const float rcp[2] = {rcp_x, rcp_y};
    return fxaa(precision, in, segmask, w, h, rcp, subpix, thr, thr_min, out, nthreads);
}

int oracle_post_process(int precision, const float* in, const float* debug, int w, int h, const int* zoom_src,
                        const int* zoom_dst, const float* mask_l, const float* mask_r, int zoom, int show_zoom_box,
                        int split_x, int show_l, int show_r, double* out, int nthreads) {
    PostParams pp{};
    for (int i = 0; i < 4; ++i) {
        pp.zoom_src[i] = zoom_src[i];
        pp.zoom_dst[i] = zoom_dst[i];
        pp.mask_l[i] = mask_l[i];
        pp.mask_r[i] = mask_r[i];
    }
    pp.zoom = zoom;
    pp.show_zoom_box = show_zoom_box;
    pp.split_x = split_x;
    pp.show_l = show_l;
    pp.show_r = show_r;
    return post_process(precision, in, debug, w, h, pp, out, nthreads);
}

void oracle_cas_setup(float s, float iw, float ih, float ow, float oh, uint32_t* c0, uint32_t* c1) {
    cas_setup(s, iw, ih, ow, oh, c0, c1);
}

float oracle_halton(int i, int b) { return halton(i, b); }

void oracle_jitter_offset(int dist, uint64_t frame, int w, int h, int fixed_index, int slow_motion, float rot,
                          float scale, float* out, int* n) {
    jitter_offset(dist, frame, w, h, fixed_index, slow_motion, rot, scale, out, n);
}

void oracle_quantize_half(const float* in, float* out, size_t n) {
    for (size_t i = 0; i < n; ++i) out[i] = quantize_half(in[i]);
}

// Counts x in [lo, hi) (as float bit patterns of positive floats) for which
// the one-step residual correction of x * RN(1/d) differs from IEEE x / d.
// Used to check the constant-divisor division of the kernels.
long long oracle_check_div_const(float d, uint32_t lo_bits, uint32_t hi_bits, int nthreads) {
    const float rd = 1.0f / d;
    if (nthreads < 1) nthreads = 1;
    std::vector<long long> bad(nthreads, 0);
    std::vector<std::thread> pool;
    uint64_t span = (uint64_t)hi_bits - lo_bits;
    for (int t = 0; t < nthreads; ++t)
        pool.emplace_back([&, t] {
            uint64_t b0 = lo_bits + span * t / nthreads, b1 = lo_bits + span * (t + 1) / nthreads;
            long long n = 0;
            for (uint64_t b = b0; b < b1; ++b) {
                uint32_t u = (uint32_t)b;
                float x;
                std::memcpy(&x, &u, 4);
                float q = x * rd;
                float r = std::fma(-d, q, x);
                float q2 = std::fma(r, rd, q);
                float ref = x / d;
                if (q2 != ref) ++n;
            }
            bad[t] = n;
        });
    for (auto& th : pool) th.join();
    long long s = 0;
    for (long long v : bad) s += v;
    return s;
}

// The reference's initial parameter values (source/taa.hpp:31-76), for the
// benchmark's reference arm, which builds its inputs without the library.
void oracle_default_parameters(taa_parameters_t* p) {
    std::memset(p, 0, sizeof *p);
    p->mAlpha = 0.05f;
    p->mColorClampingOrClipping = 1;
    p->mUnjitterFactor = 1.0f;
    p->mVarClipGamma = 1.0f;
    p->mMinAlpha = 1.0f - 0.97f;
    p->mMaxAlpha = 1.0f - 0.88f;
    p->mRejectionAlpha = 1.0f;
    p->mUseVelocityVectors = 1;
    p->mNoiseFactor = 1.f / 510.f;
    p->mVelBasedAlphaMax = 0.2f;
    p->mVelBasedAlphaFactor = 1.f / 40.f;
    p->mRayTraceAugmentFlags = 0xffffffffu & ~(TAA_RTFLAG_ALL | TAA_RTFLAG_FXD);
    p->mRayTraceAugment_WNrm = 0.5f;
    p->mRayTraceAugment_WDpt = 0.015f;
    p->mRayTraceAugment_WMId = 0.25f;
    p->mRayTraceAugment_WLum = 0.5f;
    p->mRayTraceAugment_Thresh = 0.5f;
    p->mRayTraceHistoryCount = -1;
    p->mDebugMask[0] = p->mDebugMask[1] = p->mDebugMask[2] = 1.0f;
    p->mDebugScale = 1.0f;
}

// The analytic scene's defaults, its seeded sphere table and a frame's
// sub-pixel jitter (include/taa_synth.h), from the scene header the oracle
// shares with the renderer.
void oracle_synth_default_scene(taa_synth_scene_t* s, int w, int h, uint64_t seed) {
    taa_synth::default_scene(*s, w, h, seed);
}
void oracle_synth_spheres(const taa_synth_scene_t* s, float* table) { taa_synth::spheres(*s, table); }
void oracle_synth_jitter(const taa_synth_scene_t* s, int frame, float ndc[2]) {
    float jx, jy;
    taa_synth::jitter_px(*s, frame, jx, jy);
    ndc[0] = 2.0f * jx / (float)s->width;
    ndc[1] = 2.0f * jy / (float)s->height;
}

// FP64 evaluation of the analytic scene (the scene's truth; the GPU renders
// the same formulas in FP32).  Outputs: color RGBA (before the FP16 store),
// depth, motion (4 channels, UV units, .w mover id), truth (64 spp).  Any
// output pointer may be null.
int oracle_synth_frame(const taa_synth_scene_t* s, const float* spheres, int frame, double* color, double* depth,
                       double* motion, double* truth, int nthreads) {
    if (!s || !spheres) return -1;
    const int W = s->width, H = s->height;
    if (nthreads < 1) nthreads = 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t)
        pool.emplace_back([&, t] {
            for (int y = t; y < H; y += nthreads)
                for (int x = 0; x < W; ++x) {
                    float jx, jy;
                    taa_synth::jitter_px(*s, frame, jx, jy);
                    double sx = (double)x + 0.5 - (double)jx, sy = (double)y + 0.5 - (double)jy;
                    taa_synth::Hit<double> h = taa_synth::shade<double>(*s, spheres, frame, sx, sy);
                    size_t o = (size_t)y * W + x;
                    double r = h.r, g = h.g, b = h.b;
                    uint32_t u1, u2;
                    taa_synth::pixel_hash(s->seed, x, y, frame, u1, u2);
                    if ((float)u1 * (1.0f / 16777216.0f) < s->firefly_fraction) {
                        r = g = b = 4.0 + ((double)s->firefly_max - 4.0) * ((double)u2 / 16777216.0);
                    }
                    if (color) {
                        color[o * 4 + 0] = r;
                        color[o * 4 + 1] = g;
                        color[o * 4 + 2] = b;
                        color[o * 4 + 3] = 1.0;
                    }
                    if (depth) depth[o] = h.depth;
                    if (motion) {
                        motion[o * 4 + 0] = h.mx / W;
                        motion[o * 4 + 1] = h.my / H;
                        motion[o * 4 + 2] = 0.0;
                        motion[o * 4 + 3] = (double)h.id;
                    }
                    if (truth) {
                        double ar = 0, ag = 0, ab = 0;
                        for (int j = 0; j < 8; ++j)
                            for (int i = 0; i < 8; ++i) {
                                taa_synth::Hit<double> q = taa_synth::shade<double>(
                                    *s, spheres, frame, x + (i + 0.5) / 8.0, y + (j + 0.5) / 8.0);
                                ar += q.r;
                                ag += q.g;
                                ab += q.b;
                            }
                        truth[o * 4 + 0] = ar / 64.0;
                        truth[o * 4 + 1] = ag / 64.0;
                        truth[o * 4 + 2] = ab / 64.0;
                        truth[o * 4 + 3] = 1.0;
                    }
                }
        });
    for (auto& th : pool) th.join();
    return 0;
}

}  // extern "C"
