// synth_scene.h - evaluation of the analytic scene described in taa_synth.h.
//
// Written once for host and device and templated on the arithmetic type: the
// CUDA renderer instantiates it in FP32, the test-side renderer in FP64 (the
// scene's truth).  Integer hashing decides fireflies so both agree exactly.
#pragma once
#include <stdint.h>
#include <math.h>
#include "../../include/taa_synth.h"

#if defined(__CUDACC__)
#define SYN_HD __host__ __device__ __forceinline__
#else
#define SYN_HD inline
#endif

namespace taa_synth {

constexpr double kNear = 0.1;
constexpr double kFar = 1000.0;
constexpr double kFocal = 1000.0;     // px
constexpr double kBackdropZ = 500.0;  // view-space depth of the backdrop
constexpr double kPi = 3.14159265358979323846;

SYN_HD uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Per-pixel-per-frame hash -> two 24-bit uniforms in [0,1).
SYN_HD void pixel_hash(uint64_t seed, int x, int y, int t, uint32_t& u1, uint32_t& u2) {
    uint64_t key = (uint64_t)(uint32_t)x | ((uint64_t)(uint32_t)y << 21) | ((uint64_t)(uint32_t)t << 42);
    uint64_t z = mix64(seed * 0x9E3779B97F4A7C15ull + key + 0x632BE59BD9B4E019ull);
    u1 = (uint32_t)(z >> 40);
    u2 = (uint32_t)((z >> 16) & 0xFFFFFFu);
}

// Halton radical inverse in float, as helpers::halton (helper_functions.hpp:9-17).
SYN_HD float halton_f(int i, int b) {
    float f = 1.0f, r = 0.0f;
    while (i > 0) {
        f = f / (float)b;
        r = r + f * (float)(i % b);
        i = i / b;
    }
    return r;
}

// The scene's defaults for a w x h frame (the configurations' shared values).
inline void default_scene(taa_synth_scene_t& o, int32_t w, int32_t h, uint64_t seed) {
    o = taa_synth_scene_t{};
    o.struct_size = sizeof o;
    o.width = w;
    o.height = h;
    o.seed = seed;
    o.num_spheres = 32;
    o.radius_min = 20.f;
    o.radius_max = 120.f;
    o.sphere_speed_max = 6.f;
    o.spin_max = 0.f;
    o.cam_v0[0] = 3.f;
    o.checker_period = 7.3f;
    o.firefly_fraction = 0.01f;
    o.firefly_max = 64.f;
    o.jitter_phase = 0;
    o.jitter_enabled = 1;
}

// The seeded sphere table: num_spheres rows of TAA_SYNTH_SPHERE_FLOATS.
inline void spheres(const taa_synth_scene_t& s, float* t) {
    uint64_t st = s.seed ^ 0xA0761D6478BD642Full;
    auto uni = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        return (double)(mix64(st) >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int i = 0; i < s.num_spheres; ++i) {
        float* p = t + i * TAA_SYNTH_SPHERE_FLOATS;
        p[0] = (float)(uni() * s.width);
        p[1] = (float)(uni() * s.height);
        p[2] = (float)(s.radius_min + uni() * (s.radius_max - s.radius_min));
        p[3] = (float)(50.0 + uni() * 350.0);
        p[4] = (float)uni();
        p[5] = (float)uni();
        p[6] = (float)uni();
        p[7] = (float)((2.0 * uni() - 1.0) * s.sphere_speed_max);
        p[8] = (float)((2.0 * uni() - 1.0) * s.sphere_speed_max);
        p[9] = (float)((2.0 * uni() - 1.0) * s.spin_max);
        p[10] = p[2] / 3.0f;
        p[11] = 0.f;
    }
}

SYN_HD void jitter_px(const taa_synth_scene_t& s, int t, float& jx, float& jy) {
    if (!s.jitter_enabled) { jx = 0.f; jy = 0.f; return; }
    int idx = ((t + s.jitter_phase) % 8 + 8) % 8;
    jx = halton_f(idx + 1, 2) - 0.5f;
    jy = halton_f(idx + 1, 3) - 0.5f;
}

template <class R> SYN_HD R cam_x(const taa_synth_scene_t& s, R t) {
    return R(s.cam_v0[0]) * t + R(0.5) * R(s.cam_accel[0]) * t * t;
}
template <class R> SYN_HD R cam_y(const taa_synth_scene_t& s, R t) {
    return R(s.cam_v0[1]) * t + R(0.5) * R(s.cam_accel[1]) * t * t;
}

template <class R> SYN_HD R depth_ndc(R z) {
    return R(kFar / (kFar - kNear)) * (R(1) - R(kNear) / z);
}

template <class R> struct Hit {
    R r, g, b;      // clean radiance
    R depth;        // Vulkan [0,1]
    R mx, my;       // motion in px (current - previous position of the surface point)
    int id;         // 0 backdrop, sphere index + 1
};

// Radiance, depth and motion of the surface visible at screen position (sx, sy)
// at frame t.  `sph` is the sphere table (TAA_SYNTH_SPHERE_FLOATS floats each).
template <class R>
SYN_HD Hit<R> shade(const taa_synth_scene_t& s, const float* sph, int t, R sx, R sy) {
    Hit<R> h;
    const R tt = R(t);
    // backdrop
    R cx = cam_x<R>(s, tt), cy = cam_y<R>(s, tt);
    // the fixed sub-pixel offset keeps checker edges (every 3.65 px) off the
    // exact decimal pixel centres they would otherwise hit (10 * 3.65 = 36.5)
    R ux = sx + cx + R(0.31830988618), uy = sy + cy + R(0.21132486541);
    R half = R(s.checker_period) * R(0.5);
    long long qx = (long long)floor(ux / half), qy = (long long)floor(uy / half);
    R checker = ((qx + qy) & 1) ? R(1) : R(0);
    R zx = ux - R(0.5) * R(s.width), zy = uy - R(0.5) * R(s.height);
    R maxdim = R(s.width > s.height ? s.width : s.height);
    R zp = R(0.5) + R(0.5) * cos(R(kPi) / (R(2) * maxdim) * (zx * zx + zy * zy));
    R base = R(4) * (R(0.15) + R(0.85) * checker) * (R(0.25) + R(0.75) * zp);
    // a warm tint off the Cg = 0 plane (an RGB ramp such as 0.9/0.8/0.7 has
    // Cg exactly 0, which makes the variance box degenerate in Cg)
    h.r = base * R(0.95);
    h.g = base * R(0.8);
    h.b = base * R(0.6);
    R zbest = R(kBackdropZ);
    h.mx = -(cx - cam_x<R>(s, tt - R(1)));
    h.my = -(cy - cam_y<R>(s, tt - R(1)));
    h.id = 0;
    // spheres: nearest hit wins
    const R Lx = R(-0.4), Ly = R(-0.6), Lz = R(-0.7);
    const R Ln = R(1) / sqrt(Lx * Lx + Ly * Ly + Lz * Lz);
    for (int i = 0; i < s.num_spheres; ++i) {
        const float* p = sph + i * TAA_SYNTH_SPHERE_FLOATS;
        R rad = R(p[2]);
        R ccx = R(p[0]) + R(p[7]) * tt, ccy = R(p[1]) + R(p[8]) * tt;
        R dx = sx - ccx, dy = sy - ccy;
        R rho2 = (dx * dx + dy * dy) / (rad * rad);
        if (!(rho2 < R(1))) continue;
        R nz = sqrt(R(1) - rho2);
        R zc = R(p[3]);
        R z = zc - rad * zc / R(kFocal) * nz;
        if (!(z < zbest)) continue;
        zbest = z;
        R nx = dx / rad, ny = dy / rad;
        R lam = nx * Lx + ny * Ly + (-nz) * Lz;
        lam = lam * Ln;
        R shadef = R(0.2) + R(0.8) * (lam > R(0) ? lam : R(0));
        R spin = R(p[9]);
        R th = spin * tt;
        R cth = cos(th), sth = sin(th);
        R qxr = cth * dx + sth * dy;  // rotate by -theta into the texture frame
        R stripe = sin(R(2 * kPi) * qxr / R(p[10])) >= R(0) ? R(1) : R(0.1);
        R k = R(4) * shadef * stripe;
        h.r = k * R(p[4]);
        h.g = k * R(p[5]);
        h.b = k * R(p[6]);
        // previous position of this surface point: centre(t-1) + R(-spin) * d
        R cw = cos(spin), sw = sin(spin);
        R pdx = cw * dx + sw * dy, pdy = -sw * dx + cw * dy;
        R px = R(p[0]) + R(p[7]) * (tt - R(1)) + pdx;
        R py = R(p[1]) + R(p[8]) * (tt - R(1)) + pdy;
        h.mx = sx - px;
        h.my = sy - py;
        h.id = i + 1;
    }
    h.depth = depth_ndc<R>(zbest);
    return h;
}

}  // namespace taa_synth
