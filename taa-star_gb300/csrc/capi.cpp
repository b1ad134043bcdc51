// capi.cpp - the C ABI of libtaa_gb300 (include/taa_gb300.h, include/taa_synth.h).
//
// Host side of the drop-in: context lifetime, argument validation, kernel
// form selection, and the small host computations the reference does on the
// CPU around its dispatch (jitter table, matrix composition, CasSetup).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/taa_gb300.h"
#include "../../include/taa_synth.h"
#include "host_util.h"
#include "kernels.h"
#include "synth_scene.h"

using taa_dev::FrameArgs;
using taa_dev::Img;
using taa_dev::ImgW;

namespace taa_host {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}
int ok() { return TAA_OK; }

int cuda_fail(cudaError_t e, const char* what) {
    return fail(TAA_E_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

bool finite(float v) { return std::isfinite(v); }

int check_parameters(const taa_parameters_t& p, int idx) {
    const float fs[] = {p.mAlpha, p.mUnjitterFactor, p.mVarClipGamma, p.mMinAlpha, p.mMaxAlpha, p.mRejectionAlpha,
                        p.mNoiseFactor, p.mVelBasedAlphaMax, p.mVelBasedAlphaFactor, p.mRayTraceAugment_WNrm,
                        p.mRayTraceAugment_WDpt, p.mRayTraceAugment_WMId, p.mRayTraceAugment_WLum,
                        p.mRayTraceAugment_Thresh, p.mDebugScale, p.mDebugMask[0], p.mDebugMask[1], p.mDebugMask[2],
                        p.mDebugMask[3]};
    for (size_t i = 0; i < sizeof fs / sizeof fs[0]; ++i)
        if (!finite(fs[i])) return fail(TAA_E_INVAL, "param[%d]: float field %zu is not finite", idx, i);
    return ok();
}

size_t history_texel(uint32_t fmt) { return fmt == TAA_HISTORY_RGBA32F ? 16 : 8; }
size_t motion_texel(uint32_t fmt) { return fmt == TAA_MOTION_RGBA16F ? 8 : 4; }

// Validates one binding: alignment, pitch and the byte range it spans.
int check_image(const char* name, const void* p, size_t pitch, int w, int h, size_t texel, bool required,
                const char** lo, const char** hi) {
    if (!p) {
        if (required) return fail(TAA_E_INVAL, "%s: required binding is NULL", name);
        return ok();
    }
    if (pitch < (size_t)w * texel) return fail(TAA_E_INVAL, "%s: pitch %zu < width*texel %zu", name, pitch, (size_t)w * texel);
    if ((uintptr_t)p % texel != 0 || pitch % texel != 0)
        return fail(TAA_E_ALIGN, "%s: pointer/pitch not a multiple of the %zu-byte texel", name, texel);
    if (lo) *lo = (const char*)p;
    if (hi) *hi = (const char*)p + pitch * (size_t)(h - 1) + (size_t)w * texel;
    return ok();
}

bool any_param(const taa_uniforms_t& u, int out_w, uint32_t taa_parameters_t::*f) {
    bool right_used = u.splitScreen && u.splitX < out_w - 1;
    return u.param[0].*f || (right_used && u.param[1].*f);
}

// Validates a context description (sizes, enums).
int check_desc(const taa_desc_t& d, const char* who) {
    if (d.struct_size != sizeof(taa_desc_t)) return fail(TAA_E_INVAL, "%s: struct_size %u != %zu", who, d.struct_size, sizeof(taa_desc_t));
    if (d.in_width <= 0 || d.in_height <= 0 || d.out_width <= 0 || d.out_height <= 0 || d.in_width > 32768 ||
        d.in_height > 32768 || d.out_width > 32768 || d.out_height > 32768)
        return fail(TAA_E_INVAL, "%s: image sizes must be in 1..32768", who);
    if (d.history_format > TAA_HISTORY_RGBA16F) return fail(TAA_E_INVAL, "%s: history_format %u", who, d.history_format);
    if (d.motion_format > TAA_MOTION_RG16F) return fail(TAA_E_INVAL, "%s: motion_format %u", who, d.motion_format);
    if (d.form > TAA_FORM_FAST) return fail(TAA_E_INVAL, "%s: form %u", who, d.form);
    if (d.sharpener > TAA_SHARPEN_CAS) return fail(TAA_E_INVAL, "%s: sharpener %u", who, d.sharpener);
    if (!finite(d.sharpen_factor)) return fail(TAA_E_INVAL, "%s: sharpen_factor not finite", who);
    if (d.flags & ~(TAA_FLAG_LEARNED_TCGEN05 | TAA_FLAG_FXAA | TAA_FLAG_FP16_GUARD | TAA_FLAG_FUSED_SHARPEN))
        return fail(TAA_E_INVAL, "%s: unknown flags 0x%x", who, d.flags);
    if ((d.flags & TAA_FLAG_LEARNED_TCGEN05) && d.form != TAA_FORM_LEARNED)
        return fail(TAA_E_INVAL, "%s: TAA_FLAG_LEARNED_TCGEN05 needs TAA_FORM_LEARNED", who);
    if ((d.flags & TAA_FLAG_FP16_GUARD) && d.form != TAA_FORM_FP16)
        return fail(TAA_E_INVAL, "%s: TAA_FLAG_FP16_GUARD needs TAA_FORM_FP16", who);
    return ok();
}

// Validates a uniform block (finite floats).
int check_uniforms(const taa_uniforms_t& u, const char* who) {
    for (int i = 0; i < 2; ++i) {
        int rc = check_parameters(u.param[i], i);
        if (rc) return rc;
    }
    const float m[] = {u.mJitterNdc[0], u.mJitterNdc[1], u.mSinTime[0], u.mCamNearPlane, u.mCamFarPlane};
    for (float v : m)
        if (!finite(v)) return fail(TAA_E_INVAL, "%s: jitter/time/near/far must be finite", who);
    for (int i = 0; i < 16; ++i)
        if (!finite(u.mHistoryViewProjMatrix[i]) || !finite(u.mInverseViewProjMatrix[i]))
            return fail(TAA_E_INVAL, "%s: matrices must be finite", who);
    return ok();
}

// Validates one frame's bindings against a description (sizes, formats,
// alignment, aliasing) and fills the kernel arguments.
int frame_args(const taa_desc_t& d, const taa_uniforms_t& U, uint32_t cas_peak_bits, const taa_frame_io_t* io,
               const char* who, FrameArgs* out) {
    const int iw = d.in_width, ih = d.in_height, ow = d.out_width, oh = d.out_height;
    const size_t ht = history_texel(d.history_format), mt = motion_texel(d.motion_format);
    const char *hlo = nullptr, *hhi = nullptr, *olo = nullptr, *ohi = nullptr;
    int rc;
    if ((rc = check_image("color", io->color, io->color_pitch, iw, ih, 8, true))) return rc;
    if ((rc = check_image("depth", io->depth, io->depth_pitch, iw, ih, 4, true))) return rc;
    if ((rc = check_image("velocity", io->velocity, io->velocity_pitch, iw, ih, mt, true))) return rc;
    if ((rc = check_image("history", io->history, io->history_pitch, ow, oh, ht, false, &hlo, &hhi))) return rc;
    if ((rc = check_image("history_out", io->history_out, io->history_out_pitch, ow, oh, ht, true, &olo, &ohi))) return rc;
    bool depth_cull = any_param(U, ow, &taa_parameters_t::mDepthCulling);
    if ((rc = check_image("history_depth", io->history_depth, io->history_depth_pitch, iw, ih, 4, depth_cull))) return rc;
    const char *rlo = nullptr, *rhi = nullptr, *slo = nullptr, *shi = nullptr;
    if ((rc = check_image("result", io->result, io->result_pitch, ow, oh, 8, false, &rlo, &rhi))) return rc;
    if ((rc = check_image("debug", io->debug, io->debug_pitch, ow, oh, 8, false))) return rc;
    if ((rc = check_image("segmask", io->segmask, io->segmask_pitch, ow, oh, 4, false))) return rc;
    if ((rc = check_image("material", io->material, io->material_pitch, iw, ih, 4, false))) return rc;
    if ((rc = check_image("prev_material", io->prev_material, io->prev_material_pitch, iw, ih, 4, false))) return rc;
    if ((rc = check_image("prev_segmask", io->prev_segmask, io->prev_segmask_pitch, ow, oh, 4, false))) return rc;
    if ((rc = check_image("uvnrm", io->uvnrm, io->uvnrm_pitch, iw, ih, 16, false))) return rc;
    const bool sharpen = d.sharpener != TAA_SHARPEN_OFF;
    if ((rc = check_image("sharpened", io->sharpened, io->sharpened_pitch, ow, oh, 8, sharpen, &slo, &shi))) return rc;
    if (hlo && hlo < ohi && olo < hhi) return fail(TAA_E_INVAL, "%s: history and history_out overlap", who);
    // the sharpen pass reads the result image around each pixel it writes
    if (sharpen && rlo && slo && rlo < shi && slo < rhi)
        return fail(TAA_E_INVAL, "%s: result and sharpened overlap", who);

    FrameArgs& a = *out;
    a = FrameArgs{};
    a.color = Img{(const char*)io->color, io->color_pitch, iw, ih};
    a.depth = Img{(const char*)io->depth, io->depth_pitch, iw, ih};
    a.history = Img{(const char*)io->history, io->history_pitch, ow, oh};
    a.history_depth = Img{(const char*)io->history_depth, io->history_depth_pitch, iw, ih};
    a.velocity = Img{(const char*)io->velocity, io->velocity_pitch, iw, ih};
    a.material = Img{(const char*)io->material, io->material_pitch, iw, ih};
    a.prev_material = Img{(const char*)io->prev_material, io->prev_material_pitch, iw, ih};
    a.prev_segmask = Img{(const char*)io->prev_segmask, io->prev_segmask_pitch, ow, oh};
    a.uvnrm = Img{(const char*)io->uvnrm, io->uvnrm_pitch, iw, ih};
    a.result = ImgW{(char*)io->result, io->result_pitch};
    a.debug = ImgW{(char*)io->debug, io->debug_pitch};
    a.history_out = ImgW{(char*)io->history_out, io->history_out_pitch};
    a.segmask = ImgW{(char*)io->segmask, io->segmask_pitch};
    a.sharpened = ImgW{(char*)io->sharpened, io->sharpened_pitch};
    a.out_w = ow;
    a.out_h = oh;
    a.inv_out_w = 1.0f / (float)ow;
    a.inv_out_h = 1.0f / (float)oh;
    a.cas_peak_bits = cas_peak_bits;
    a.sharpen_factor = d.sharpen_factor;
    a.neg_zero2 = taa_dev::kNegZeroPair;
    cudaError_t se = taa_dev::device_status_word(&a.status);
    if (se != cudaSuccess) return cuda_fail(se, "device status word");
    return ok();

}

int learned_supported(const taa_desc_t& d, const taa_uniforms_t& U, const taa_frame_io_t* io, const char* who) {
    const taa_parameters_t& P = U.param[0];
    if (d.history_format != TAA_HISTORY_RGBA32F || d.sharpener != TAA_SHARPEN_OFF)
        return fail(TAA_E_UNSUPPORTED, "%s: the learned form keeps RGBA32F history and has no sharpener", who);
    if (!taa_dev::fast_path_supported(U, d.in_width, d.in_height, d.out_width, d.out_height))
        return fail(TAA_E_UNSUPPORTED, "%s: these parameters need the plain form", who);
    if (!P.mUseYCoCg || P.mToneMapLumaKaris || P.mInterpolationMode != 2)
        return fail(TAA_E_UNSUPPORTED, "%s: the learned form works in YCoCg without tonemapping, Catmull-Rom history", who);
    if (io && (io->debug || io->segmask))
        return fail(TAA_E_UNSUPPORTED, "%s: debug and segmask outputs run with the plain form", who);
    return TAA_OK;
}

}  // namespace taa_host

using namespace taa_host;

extern "C" {

const char* taa_version(int* abi_version) {
    if (abi_version) *abi_version = TAA_GB300_ABI_VERSION;
    return "taa_gb300 0.1.0 (sm_103a)";
}

const char* taa_last_error(void) { return g_last_error.c_str(); }

// source/taa.hpp:31-76
int taa_default_parameters(taa_parameters_t* o) {
    if (!o) return fail(TAA_E_INVAL, "taa_default_parameters: out is NULL");
    std::memset(o, 0, sizeof *o);
    o->mAlpha = 0.05f;
    o->mColorClampingOrClipping = 1;
    o->mUnjitterFactor = 1.0f;
    o->mVarClipGamma = 1.0f;
    o->mMinAlpha = 1.0f - 0.97f;
    o->mMaxAlpha = 1.0f - 0.88f;
    o->mRejectionAlpha = 1.0f;
    o->mUseVelocityVectors = 1;
    o->mNoiseFactor = 1.f / 510.f;
    o->mVelBasedAlphaMax = 0.2f;
    o->mVelBasedAlphaFactor = 1.f / 40.f;
    o->mRayTraceAugmentFlags = 0xffffffffu & ~(TAA_RTFLAG_ALL | TAA_RTFLAG_FXD);
    o->mRayTraceAugment_WNrm = 0.5f;
    o->mRayTraceAugment_WDpt = 0.015f;
    o->mRayTraceAugment_WMId = 0.25f;
    o->mRayTraceAugment_WLum = 0.5f;
    o->mRayTraceAugment_Thresh = 0.5f;
    o->mRayTraceHistoryCount = -1;
    o->mDebugMask[0] = o->mDebugMask[1] = o->mDebugMask[2] = 1.f;
    o->mDebugMask[3] = 0.f;
    o->mDebugScale = 1.0f;
    return ok();
}

// helpers::halton (source/helper_functions.hpp:9-17), in float as the reference.
static float halton_host(int i, int b) {
    float f = 1.0f, r = 0.0f;
    while (i > 0) {
        f = f / (float)b;
        r = r + f * (float)(i % b);
        i = i / b;
    }
    return r;
}

namespace {
// The frame's entry of a jitter table and the debugging knobs (source/taa.hpp:219-232).
void pick_jitter(const float* tx, const float* ty, int n, uint64_t frame_id, const taa_jitter_opts_t* opts,
                 float out[2]) {
    taa_jitter_opts_t o = {-1, 1, 0.f, 1.f};
    if (opts) o = *opts;
    if (o.slow_motion > 1) frame_id /= (uint64_t)o.slow_motion;
    if (o.fixed_index >= 0) frame_id = (uint64_t)o.fixed_index;
    float x = tx[frame_id % (uint64_t)n], y = ty[frame_id % (uint64_t)n];
    if (o.rotate_degrees != 0.f) {
        float r = o.rotate_degrees * (float)(3.14159265358979323846 / 180.0);
        float s = std::sin(r), c = std::cos(r);
        float nx = x * c - y * s, ny = x * s + y * c;
        x = nx;
        y = ny;
    }
    out[0] = x * o.extra_scale;
    out[1] = y * o.extra_scale;
}
}  // namespace

// source/taa.hpp:150-233.  The reference fills its tables once from the
// first resolution it sees (function-local statics); here every call uses
// the resolution it is given.
int taa_get_jitter_offset(int32_t dist, uint64_t frame_id, int32_t w, int32_t h, const taa_jitter_opts_t* opts,
                          float out[2], int32_t* out_n) {
    if (!out) return fail(TAA_E_INVAL, "taa_get_jitter_offset: out is NULL");
    if (w <= 0 || h <= 0) return fail(TAA_E_INVAL, "taa_get_jitter_offset: bad resolution %dx%d", w, h);
    if (dist < 0 || dist > 4) return fail(TAA_E_INVAL, "taa_get_jitter_offset: sample distribution %d not in 0..4", dist);
    const float sx = 2.0f / (float)w, sy = 2.0f / (float)h;
    float tx[16], ty[16];
    int n = 0;
    if (dist == 0 || dist == 1) {
        // circular quad / uniform-4 helix, in units of +-0.25 px
        static const float q[2][4][2] = {{{-.25f, -.25f}, {.25f, -.25f}, {.25f, .25f}, {-.25f, .25f}},
                                         {{-.25f, -.25f}, {.25f, .25f}, {.25f, -.25f}, {-.25f, .25f}}};
        for (n = 0; n < 4; ++n) {
            tx[n] = sx * q[dist][n][0];
            ty[n] = sy * q[dist][n][1];
        }
    } else if (dist == 2 || dist == 3) {
        int len = dist == 2 ? 8 : 16;
        for (n = 0; n < len; ++n) {
            tx[n] = sx * (halton_host(n + 1, 2) - 0.5f);
            ty[n] = sy * (halton_host(n + 1, 3) - 0.5f);
        }
    } else {
        const float e = 1.f / 8.f;
        for (int j = 0; j < 4; ++j)
            for (int i = 0; i < 4; ++i, ++n) {
                tx[n] = sx * ((float)(2 * i - 3) * e);
                ty[n] = sy * ((float)(2 * j - 3) * e);
            }
    }
    pick_jitter(tx, ty, n, frame_id, opts, out);
    if (out_n) *out_n = n;
    return ok();
}

// Sample distribution 5 of source/taa.hpp:207-211: the debug sample offsets,
// in pixels, scaled to NDC.
int taa_get_jitter_offset_custom(const float (*offsets_px)[2], int32_t count, uint64_t frame_id, int32_t w, int32_t h,
                                 const taa_jitter_opts_t* opts, float out[2]) {
    if (!out || !offsets_px) return fail(TAA_E_INVAL, "taa_get_jitter_offset_custom: NULL argument");
    if (w <= 0 || h <= 0) return fail(TAA_E_INVAL, "taa_get_jitter_offset_custom: bad resolution %dx%d", w, h);
    if (count < 1 || count > TAA_SETTINGS_MAX_SAMPLE_OFFSETS)
        return fail(TAA_E_INVAL, "taa_get_jitter_offset_custom: count %d not in 1..%d", count,
                    TAA_SETTINGS_MAX_SAMPLE_OFFSETS);
    const float sx = 2.0f / (float)w, sy = 2.0f / (float)h;
    float tx[TAA_SETTINGS_MAX_SAMPLE_OFFSETS], ty[TAA_SETTINGS_MAX_SAMPLE_OFFSETS];
    for (int i = 0; i < count; ++i) {
        if (!finite(offsets_px[i][0]) || !finite(offsets_px[i][1]))
            return fail(TAA_E_INVAL, "taa_get_jitter_offset_custom: offset %d not finite", i);
        tx[i] = offsets_px[i][0] * sx;
        ty[i] = offsets_px[i][1] * sy;
    }
    pick_jitter(tx, ty, count, frame_id, opts, out);
    return ok();
}

// glm::translate(vec3(j.x, j.y, 0)) * P (source/taa.hpp:248), column-major.
int taa_jittered_projection(const float p[16], const float j[2], float out[16]) {
    if (!p || !j || !out) return fail(TAA_E_INVAL, "taa_jittered_projection: NULL argument");
    float r[16];
    for (int c = 0; c < 4; ++c) {
        // T * column c: rows 0 and 1 gain j * row 3
        r[c * 4 + 0] = p[c * 4 + 0] + j[0] * p[c * 4 + 3];
        r[c * 4 + 1] = p[c * 4 + 1] + j[1] * p[c * 4 + 3];
        r[c * 4 + 2] = p[c * 4 + 2];
        r[c * 4 + 3] = p[c * 4 + 3];
    }
    std::memcpy(out, r, sizeof r);
    return ok();
}

static void mat_mul_d(const double* a, const double* b, double* o) {  // column-major o = a*b
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + r] * b[c * 4 + k];
            o[c * 4 + r] = s;
        }
}

// Gauss-Jordan inverse with partial pivoting; false if singular.
static bool mat_inv_d(const double* m, double* inv) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (!(std::fabs(a[piv][c]) > 1e-300)) return false;
        if (piv != c)
            for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
        double d = a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            double f = a[r][c];
            if (f != 0.0)
                for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[c * 4 + r] = a[r][c + 4];
    return true;
}

// source/taa.hpp:993-994 in FP64.
int taa_compose_matrices(const double pc[16], const double vc[16], const double pp[16], const double vp[16],
                         float inv_vp[16], float hist_vp[16]) {
    if (!pc || !vc || !pp || !vp || !inv_vp || !hist_vp) return fail(TAA_E_INVAL, "taa_compose_matrices: NULL argument");
    double cur[16], inv[16], prev[16];
    mat_mul_d(pc, vc, cur);
    if (!mat_inv_d(cur, inv)) return fail(TAA_E_INVAL, "taa_compose_matrices: proj_cur*view_cur is singular");
    mat_mul_d(pp, vp, prev);
    for (int i = 0; i < 16; ++i) {
        inv_vp[i] = (float)inv[i];
        hist_vp[i] = (float)prev[i];
    }
    return ok();
}

static uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// CasSetup (shaders/ffx_cas.h:375-394) with ffx_a.h's CPU helpers.
int taa_cas_setup(float sharpness, float in_w, float in_h, float out_w, float out_h, uint32_t c0[4], uint32_t c1[4]) {
    if (!c0 || !c1) return fail(TAA_E_INVAL, "taa_cas_setup: NULL argument");
    c0[0] = fbits(in_w * (1.0f / out_w));
    c0[1] = fbits(in_h * (1.0f / out_h));
    c0[2] = fbits(0.5f * in_w * (1.0f / out_w) - 0.5f);
    c0[3] = fbits(0.5f * in_h * (1.0f / out_h) - 0.5f);
    float s = sharpness < 0.f ? 0.f : (sharpness > 1.f ? 1.f : sharpness);
    float sharp = -(1.0f / (5.0f * s + (-8.0f * s + 8.0f)));
    c1[0] = fbits(sharp);
    // packed FP16 copy of the sharpness for the packed-math CAS variant:
    // ffx_a.h's CPU converter truncates the mantissa
    auto h = [](float f) -> uint32_t {
        uint32_t u = fbits(f), sg = (u >> 16) & 0x8000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
        if (e < 103u) return sg;
        if (e < 113u) return sg + (1u << (e - 103u)) + (m >> (126u - e));
        if (e < 143u) return sg + ((e - 112u) << 10) + (m >> 13);
        return sg + 0x7bffu;
    };
    c1[1] = h(sharp) | (h(0.0f) << 16);
    c1[2] = fbits(8.0f * in_w * (1.0f / out_w));
    c1[3] = 0;
    return ok();
}

// ---------------------------------------------------------------- context

static int ensure_scratch(taa_ctx* c) {
    if (c->desc.sharpener == TAA_SHARPEN_OFF || c->scratch_screen) return ok();
    cudaError_t e = cudaMallocPitch(&c->scratch_screen, &c->scratch_pitch, (size_t)c->desc.out_width * 8,
                                    (size_t)c->desc.out_height);
    if (e != cudaSuccess) {
        c->scratch_screen = nullptr;
        return e == cudaErrorMemoryAllocation ? fail(TAA_E_NOMEM, "scratch screen image: out of device memory")
                                              : cuda_fail(e, "cudaMallocPitch");
    }
    return ok();
}

int taa_create(const taa_desc_t* d, taa_ctx** out) {
    if (!d || !out) return fail(TAA_E_INVAL, "taa_create: NULL argument");
    *out = nullptr;
    int rc0 = check_desc(*d, "taa_create");
    if (rc0) return rc0;
    taa_ctx* c = new (std::nothrow) taa_ctx();
    if (!c) return fail(TAA_E_NOMEM, "taa_create: host allocation failed");
    c->desc = *d;
    cudaError_t e = cudaGetDevice(&c->device);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaGetDevice");
    }
    taa_cas_setup(d->sharpen_factor, (float)d->out_width, (float)d->out_height, (float)d->out_width,
                  (float)d->out_height, c->cas_const0, c->cas_const1);
    int rc = ensure_scratch(c);
    if (rc == TAA_OK && d->form == TAA_FORM_LEARNED) {
        e = cudaMalloc(&c->mlp_weights, sizeof(float) * (size_t)taa_dev::learned_param_count());
        if (e == cudaSuccess) e = cudaMalloc(&c->mlp_blob, (size_t)taa_dev::learned_blob_bytes());
        if (e != cudaSuccess) rc = e == cudaErrorMemoryAllocation ? fail(TAA_E_NOMEM, "taa_create: out of device memory")
                                                                  : cuda_fail(e, "taa_create: network buffers");
    }
    if (rc == TAA_OK && (d->flags & TAA_FLAG_FXAA)) {
        c->fxaa_cap = (size_t)d->out_width * (size_t)d->out_height;
        e = cudaMalloc(&c->fxaa_list, (c->fxaa_cap + 4) * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMemset(c->fxaa_list, 0, 4 * sizeof(uint32_t));  // the list head
        if (e != cudaSuccess) rc = e == cudaErrorMemoryAllocation ? fail(TAA_E_NOMEM, "taa_create: out of device memory")
                                                                  : cuda_fail(e, "taa_create: FXAA work list");
    }
    if (rc != TAA_OK) {
        taa_destroy(c);
        return rc;
    }
    *out = c;
    return ok();
}

int taa_destroy(taa_ctx* c) {
    if (!c) return ok();
    if (c->scratch_screen) cudaFree(c->scratch_screen);
    if (c->mlp_weights) cudaFree(c->mlp_weights);
    if (c->mlp_blob) cudaFree(c->mlp_blob);
    if (c->fxaa_list) cudaFree(c->fxaa_list);
    delete c;
    return ok();
}

int taa_set_uniforms(taa_ctx* c, const taa_uniforms_t* u) {
    if (!c || !u) return fail(TAA_E_INVAL, "taa_set_uniforms: NULL argument");
    int rc0 = check_uniforms(*u, "taa_set_uniforms");
    if (rc0) return rc0;
    c->uniforms = *u;
    c->have_uniforms = true;
    return ok();
}

int taa_set_sharpener(taa_ctx* c, uint32_t sharpener, float factor) {
    if (!c) return fail(TAA_E_INVAL, "taa_set_sharpener: NULL context");
    if (sharpener > TAA_SHARPEN_CAS) return fail(TAA_E_INVAL, "taa_set_sharpener: sharpener %u", sharpener);
    if (!finite(factor)) return fail(TAA_E_INVAL, "taa_set_sharpener: factor not finite");
    c->desc.sharpener = sharpener;
    c->desc.sharpen_factor = factor;
    taa_cas_setup(factor, (float)c->desc.out_width, (float)c->desc.out_height, (float)c->desc.out_width,
                  (float)c->desc.out_height, c->cas_const0, c->cas_const1);
    return ensure_scratch(c);
}

// True when a sharpener runs in the same launch as the tiled FP32 resolve
// (TAA_FLAG_FUSED_SHARPEN); otherwise a sharpener is a pass of its own after
// the resolve, in every form.
static bool fused_sharpen(const taa_desc_t& d) {
    return d.sharpener != TAA_SHARPEN_OFF && (d.flags & TAA_FLAG_FUSED_SHARPEN) &&
           d.form != TAA_FORM_PLAIN && d.form != TAA_FORM_LEARNED;
}

// AUTO picks the reassociating FP32 form where it runs the parameters, else
// the tiled FP32 form (bit-identical to the plain form); the FP16 form is used
// only when asked for, since its error contract is looser.  Parameters the
// tiled forms do not implement fall back to the plain form; the FP16 and fast
// forms with a fused sharpener run as the tiled FP32 form.
static int select_form(const taa_ctx* c, const taa_frame_io_t* io) {
    if (c->desc.form == TAA_FORM_PLAIN) return TAA_FORM_PLAIN;
    if (c->desc.form == TAA_FORM_LEARNED) return TAA_FORM_LEARNED;
    const taa_desc_t& d = c->desc;
    const bool fused = fused_sharpen(d);
    if (!taa_dev::fast_path_supported(c->uniforms, d.in_width, d.in_height, d.out_width, d.out_height, !fused,
                                      !fused)) {
        // upsampling: the fast form's path for it in the benchmark mode, else the tiled FP32 form's
        if (!fused && !(io && io->debug) && (d.form == TAA_FORM_AUTO || d.form == TAA_FORM_FAST) &&
            taa_dev::fast32_up_supported(c->uniforms, (int)d.history_format, d.in_width, d.in_height, d.out_width,
                                         d.out_height))
            return TAA_FORM_FAST;
        if (!fused && !(io && io->debug) &&
            taa_dev::up_path_supported(c->uniforms, d.in_width, d.in_height, d.out_width, d.out_height))
            return TAA_FORM_TILED;
        return TAA_FORM_PLAIN;
    }
    // a debug binding: the tiled FP32 form writes it (the fused sharpener does not)
    if (io && io->debug) return fused ? TAA_FORM_PLAIN : TAA_FORM_TILED;
    if (d.form == TAA_FORM_FP16 && !fused) return TAA_FORM_FP16;
    // the one-launch sharpener exists for the fast and the exact FP32 forms; an FP16
    // context asking for it gets the fast form's (faster than FP16 here, and within 1e-4)
    if ((d.form == TAA_FORM_AUTO || d.form == TAA_FORM_FAST || (d.form == TAA_FORM_FP16 && fused)) &&
        taa_dev::fast32_supported(c->uniforms, (int)d.history_format, d.in_width, d.in_height, d.out_width,
                                  d.out_height))
        return TAA_FORM_FAST;
    // one view without the one-launch sharpener: also the reference's default mode (clamp to
    // the RGB min/max box) and RGBA16F history on the strip body
    if ((d.form == TAA_FORM_AUTO || d.form == TAA_FORM_FAST) && !fused &&
        (taa_dev::fast32_single_supported(c->uniforms, (int)d.history_format, d.in_width, d.in_height, d.out_width,
                                          d.out_height) ||
         taa_dev::fast32_gen_supported(c->uniforms, (int)d.history_format, d.in_width, d.in_height, d.out_width,
                                       d.out_height)))
        return TAA_FORM_FAST;
    return TAA_FORM_TILED;
}

int taa_selected_form(const taa_ctx* c) {
    if (!c) return fail(TAA_E_INVAL, "taa_selected_form: NULL context");
    if (!c->have_uniforms) return fail(TAA_E_INVAL, "taa_selected_form: no uniforms set");
    return select_form(c, nullptr);
}

int taa_resolve(taa_ctx* c, void* stream, const taa_frame_io_t* io) {
    if (!c || !io) return fail(TAA_E_INVAL, "taa_resolve: NULL argument");
    if (!c->have_uniforms) return fail(TAA_E_INVAL, "taa_resolve: taa_set_uniforms was not called");
    const taa_desc_t& d = c->desc;
    const taa_uniforms_t& U = c->uniforms;
    const bool sharpen = d.sharpener != TAA_SHARPEN_OFF;
    FrameArgs a{};
    int rc = frame_args(d, U, c->cas_const1[0], io, "taa_resolve", &a);
    if (rc) return rc;

    cudaStream_t s = (cudaStream_t)stream;
    int form = select_form(c, io);
    cudaError_t e;
    if (form == TAA_FORM_LEARNED) {
        if (!c->have_mlp) return fail(TAA_E_INVAL, "taa_resolve: the learned form has no weights (taa_set_mlp)");
        if ((rc = learned_supported(d, U, io, "taa_resolve"))) return rc;
        const int mc = d.motion_format == TAA_MOTION_RGBA16F ? 4 : 2;
        if (taa_dev::fast32_supported(U, (int)d.history_format, d.in_width, d.in_height, d.out_width, d.out_height))
            // the benchmark mode: the strip body, the network per warp or on tcgen05
            e = (d.flags & TAA_FLAG_LEARNED_TCGEN05) ? taa_dev::launch_resolve_learned_strips_tc(mc, U, a, c->mlp_blob, s)
                                                     : taa_dev::launch_resolve_learned_strips(mc, U, a, c->mlp_blob, s);
        else
            e = taa_dev::launch_resolve_learned((int)d.history_format, d.motion_format == TAA_MOTION_RGBA16F ? 4 : 2,
                                                false, (d.flags & TAA_FLAG_LEARNED_TCGEN05) != 0, U, a, c->mlp_blob,
                                                nullptr, nullptr, 0, 0, 0, 0.f, Img{}, s);
    } else if (form == TAA_FORM_PLAIN) {
        if (sharpen && !a.result.p) a.result = ImgW{(char*)c->scratch_screen, c->scratch_pitch};
        e = taa_dev::launch_resolve_plain(U, a, (int)d.history_format, d.motion_format == TAA_MOTION_RGBA16F ? 4 : 2, s);
        if (e == cudaSuccess && sharpen) e = taa_dev::launch_sharpen((int)d.sharpener, a, s);
    } else {
        const int mc = d.motion_format == TAA_MOTION_RGBA16F ? 4 : 2;
        // without TAA_FLAG_FUSED_SHARPEN a sharpener reads the RGBA16F result
        // image the resolve writes (the caller's, or the context's)
        if (sharpen && !fused_sharpen(d) && !a.result.p) a.result = ImgW{(char*)c->scratch_screen, c->scratch_pitch};
        if (form == TAA_FORM_FAST && fused_sharpen(d)) {
            e = taa_dev::launch_resolve_fast32_sharpen(mc, (int)d.sharpener, U, a, s);
        } else if (form == TAA_FORM_FAST && (d.in_width != d.out_width || d.in_height != d.out_height)) {
            e = taa_dev::launch_resolve_fast32_up(mc, U, a, s);
            if (e == cudaSuccess && sharpen) e = taa_dev::launch_sharpen((int)d.sharpener, a, s);
        } else if (form == TAA_FORM_FAST) {
            e = taa_dev::fast32_single_supported(U, (int)d.history_format, d.in_width, d.in_height, d.out_width,
                                                 d.out_height)
                    ? taa_dev::launch_resolve_fast32(mc, (int)d.history_format, U, a, s)
                    : taa_dev::launch_resolve_fast32_gen(mc, U, a, s);
            if (e == cudaSuccess && sharpen) e = taa_dev::launch_sharpen((int)d.sharpener, a, s);
        } else if (form == TAA_FORM_FP16) {
            e = (d.flags & TAA_FLAG_FP16_GUARD)
                    ? taa_dev::launch_resolve_half_guarded((int)d.history_format, mc, U.param[0].mInterpolationMode, U, a, s)
                    : taa_dev::launch_resolve_half((int)d.history_format, mc, U.param[0].mInterpolationMode, U, a, s);
            if (e == cudaSuccess && sharpen) e = taa_dev::launch_sharpen((int)d.sharpener, a, s);
        } else if (!fused_sharpen(d)) {
            e = taa_dev::launch_resolve_tiled((int)d.history_format, mc, U.param[0].mInterpolationMode, U, a, s);
            if (e == cudaSuccess && sharpen) e = taa_dev::launch_sharpen((int)d.sharpener, a, s);
        } else {
            taa_dev::FastKey k;
            k.form = form;
            k.history_fmt = (int)d.history_format;
            k.motion_ch = mc;
            k.interp = U.param[0].mInterpolationMode;
            k.sharpen = (int)d.sharpener;
            e = taa_dev::launch_resolve_fast(k, U, a, s);
        }
    }
    if (e != cudaSuccess) return cuda_fail(e, "taa_resolve launch");
    return ok();
}

// taa_resolve on a copy of the context that carries the given sharpener and,
// where a resolve hands a screen image to the sharpen pass after it, the
// library's fixed buffer (static_scratch.cu) instead of an allocated one.
int taa_resolve_static_scratch(taa_ctx* c, void* stream, const taa_frame_io_t* io, uint32_t sharpener, float factor) {
    if (!c || !io) return fail(TAA_E_INVAL, "taa_resolve_static_scratch: NULL argument");
    if (!c->have_uniforms) return fail(TAA_E_INVAL, "taa_resolve_static_scratch: taa_set_uniforms was not called");
    if (sharpener > TAA_SHARPEN_CAS) return fail(TAA_E_INVAL, "taa_resolve_static_scratch: sharpener %u", sharpener);
    if (!finite(factor)) return fail(TAA_E_INVAL, "taa_resolve_static_scratch: factor not finite");
    taa_ctx v = *c;
    const int ow = v.desc.out_width, oh = v.desc.out_height;
    v.desc.sharpener = sharpener;
    v.desc.sharpen_factor = factor;
    taa_cas_setup(factor, (float)ow, (float)oh, (float)ow, (float)oh, v.cas_const0, v.cas_const1);
    v.scratch_screen = nullptr;
    v.scratch_pitch = 0;
    const int vform = select_form(&v, io);
    const bool two_pass = vform == TAA_FORM_PLAIN || (vform != TAA_FORM_LEARNED && !fused_sharpen(v.desc));
    if (sharpener != TAA_SHARPEN_OFF && !io->result && two_pass) {
        const size_t texels = (size_t)ow * (size_t)oh;
        if (texels > (size_t)TAA_STATIC_SCRATCH_MAX_TEXELS)
            return fail(TAA_E_INVAL,
                        "taa_resolve_static_scratch: a %dx%d screen image (%zu texels) exceeds the static buffer "
                        "of %d texels; bind io->result or use taa_resolve",
                        ow, oh, texels, TAA_STATIC_SCRATCH_MAX_TEXELS);
        void* p = nullptr;
        size_t bytes = 0;
        cudaError_t e = taa_dev::static_screen_scratch(&p, &bytes);
        if (e != cudaSuccess) return cuda_fail(e, "taa_resolve_static_scratch: cudaGetSymbolAddress");
        if (bytes < texels * 8) return fail(TAA_E_INVAL, "taa_resolve_static_scratch: static buffer too small");
        v.scratch_screen = p;
        v.scratch_pitch = (size_t)ow * 8;
    }
    return taa_resolve(&v, stream, io);
}

int taa_set_mlp(taa_ctx* c, const taa_mlp_weights_t* w) {
    if (!c || !w) return fail(TAA_E_INVAL, "taa_set_mlp: NULL argument");
    if (c->desc.form != TAA_FORM_LEARNED || !c->mlp_blob)
        return fail(TAA_E_INVAL, "taa_set_mlp: the context was not created with TAA_FORM_LEARNED");
    const float* p = reinterpret_cast<const float*>(w);
    for (int i = 0; i < taa_dev::learned_param_count(); ++i)
        if (!finite(p[i])) return fail(TAA_E_INVAL, "taa_set_mlp: weight %d is not finite", i);
    cudaError_t e = cudaMemcpy(c->mlp_weights, w, sizeof(taa_mlp_weights_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = taa_dev::launch_mlp_build_blob(c->mlp_weights, c->mlp_blob, nullptr);
    if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
    if (e != cudaSuccess) return cuda_fail(e, "taa_set_mlp");
    c->have_mlp = true;
    return ok();
}

int taa_device_status(uint32_t* bits, int clear) {
    if (!bits) return fail(TAA_E_INVAL, "taa_device_status: NULL argument");
    unsigned int* w = nullptr;
    cudaError_t e = taa_dev::device_status_word(&w);
    if (e != cudaSuccess) return cuda_fail(e, "taa_device_status: device status word");
    unsigned int v = 0;
    e = cudaMemcpy(&v, w, sizeof v, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "taa_device_status: read");
    if (clear && v) {
        e = cudaMemset(w, 0, sizeof v);
        if (e != cudaSuccess) return cuda_fail(e, "taa_device_status: clear");
    }
    *bits = v;
    return ok();
}

int taa_debug_set_window_wait(uint32_t first_wait_polls) {
    unsigned int* w = nullptr;
    cudaError_t e = taa_dev::device_status_word(&w);
    if (e != cudaSuccess) return cuda_fail(e, "taa_debug_set_window_wait: device status word");
    const unsigned int v = first_wait_polls;
    e = cudaMemcpy(w + 1, &v, sizeof v, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "taa_debug_set_window_wait");
    return ok();
}

// ---------------------------------------------------------------- synthetic scene

int taa_synth_default_scene(taa_synth_scene_t* o, int32_t w, int32_t h, uint64_t seed) {
    if (!o) return fail(TAA_E_INVAL, "taa_synth_default_scene: NULL");
    if (w <= 0 || h <= 0) return fail(TAA_E_INVAL, "taa_synth_default_scene: bad size");
    taa_synth::default_scene(*o, w, h, seed);
    return ok();
}

static int check_scene(const taa_synth_scene_t* s) {
    if (!s) return fail(TAA_E_INVAL, "synth: NULL scene");
    if (s->struct_size != sizeof(taa_synth_scene_t)) return fail(TAA_E_INVAL, "synth: struct_size mismatch");
    if (s->width <= 0 || s->height <= 0) return fail(TAA_E_INVAL, "synth: bad size");
    if (s->num_spheres < 0 || s->num_spheres > TAA_SYNTH_MAX_SPHERES) return fail(TAA_E_INVAL, "synth: num_spheres");
    if (!(s->checker_period > 0.f)) return fail(TAA_E_INVAL, "synth: checker_period");
    return ok();
}

int taa_synth_spheres(const taa_synth_scene_t* s, float* t, int32_t cap) {
    int rc = check_scene(s);
    if (rc) return rc;
    if (!t || cap < s->num_spheres) return fail(TAA_E_INVAL, "synth: sphere table too small");
    taa_synth::spheres(*s, t);
    return ok();
}

int taa_synth_jitter(const taa_synth_scene_t* s, int32_t frame, float px[2], float ndc[2]) {
    int rc = check_scene(s);
    if (rc) return rc;
    float jx, jy;
    taa_synth::jitter_px(*s, frame, jx, jy);
    if (px) {
        px[0] = jx;
        px[1] = jy;
    }
    if (ndc) {
        ndc[0] = 2.0f * jx / (float)s->width;
        ndc[1] = 2.0f * jy / (float)s->height;
    }
    return ok();
}

int taa_synth_camera(const taa_synth_scene_t* s, int32_t frame, double proj[16], double view[16]) {
    int rc = check_scene(s);
    if (rc) return rc;
    if (!proj || !view) return fail(TAA_E_INVAL, "synth: NULL matrix");
    using namespace taa_synth;
    std::memset(proj, 0, 16 * sizeof(double));
    std::memset(view, 0, 16 * sizeof(double));
    // clip = (2f/W X, 2f/H Y, A Z + B, Z); ndc.z = A + B/Z is the depth the renderer writes
    proj[0] = 2.0 * kFocal / s->width;
    proj[5] = 2.0 * kFocal / s->height;
    proj[10] = kFar / (kFar - kNear);
    proj[11] = 1.0;
    proj[14] = -kFar * kNear / (kFar - kNear);
    // the backdrop moves by -cam(t) px at depth kBackdropZ: camera at cam(t)*Z/f
    double t = frame;
    double cx = (double)s->cam_v0[0] * t + 0.5 * (double)s->cam_accel[0] * t * t;
    double cy = (double)s->cam_v0[1] * t + 0.5 * (double)s->cam_accel[1] * t * t;
    view[0] = view[5] = view[10] = view[15] = 1.0;
    view[12] = -cx * kBackdropZ / kFocal;
    view[13] = -cy * kBackdropZ / kFocal;
    return ok();
}

int taa_synth_render(const taa_synth_scene_t* s, int32_t frame, void* stream, const taa_synth_frame_t* out) {
    int rc = check_scene(s);
    if (rc) return rc;
    if (!out) return fail(TAA_E_INVAL, "synth: NULL output");
    if (out->motion && out->motion_channels != 2 && out->motion_channels != 4)
        return fail(TAA_E_INVAL, "synth: motion_channels must be 2 or 4");
    static thread_local float table[TAA_SYNTH_MAX_SPHERES * TAA_SYNTH_SPHERE_FLOATS];
    taa_synth_spheres(s, table, TAA_SYNTH_MAX_SPHERES);
    cudaError_t e = taa_dev::launch_synth(*s, table, frame, *out, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "taa_synth_render launch");
    return ok();
}

}  // extern "C"
