"""Known-answer tests of the oracle (CPU, no GPU).

The reference ships no tests or golden data for its resolve; these pin the
oracle's restatement of shaders/taa.comp on identities the shader's algebra
implies, in FP64 (exact where the algebra is exact) and FP32.
"""
import numpy as np
import pytest

import oracle as O
import taa_abi as T
import workloads as WL
from helpers import cpu_frames, max_rel


def rng_img(seed, h, w, ch=4, lo=0.0, hi=4.0, dtype=np.float16):
    r = np.random.default_rng(seed)
    return r.uniform(lo, hi, (h, w, ch)).astype(dtype).astype(np.float32)


def params(**kw):
    return WL.base_parameters(**kw)


def run(p, color, depth=None, vel=None, hist=None, hdepth=None, precision=64, **ukw):
    h, w = color.shape[:2]
    depth = np.full((h, w), 0.5, np.float32) if depth is None else depth
    vel = np.zeros((h, w, 2), np.float32) if vel is None else vel
    u = T.make_uniforms(p, **ukw)
    return O.resolve(u, color, depth, vel, history=hist, history_depth=hdepth, precision=precision)


def test_alpha_one_returns_current_colour_exactly():
    c = rng_img(1, 13, 17)
    hist = rng_img(2, 13, 17, dtype=np.float32)
    for prec in (64, 32):
        r = run(params(mAlpha=1.0), c, hist=hist, precision=prec)
        if prec == 64:
            np.testing.assert_array_equal(r["history"][..., :3], c[..., :3])
        else:
            assert max_rel(r["history"][..., :3], c[..., :3]) < 3e-7


def test_reset_history_returns_current(built):
    c = rng_img(3, 9, 11)
    hist = rng_img(4, 9, 11, dtype=np.float32)
    r = run(params(), c, hist=hist, mResetHistory=1)
    np.testing.assert_array_equal(r["history"][..., :3], c[..., :3])
    assert np.all(r["screen"][..., 3] == 1.0) and np.all(r["history"][..., 3] == 0.0)


def test_pass_through_and_bypass():
    c = rng_img(5, 7, 8)
    hist = rng_img(6, 7, 8, dtype=np.float32)
    r = run(params(mPassThrough=1), c, hist=hist)
    np.testing.assert_array_equal(r["screen"][..., :3], c[..., :3])
    np.testing.assert_array_equal(r["history"][..., :3], hist[..., :3])
    assert np.all(r["history"][..., 3] == 1) and np.all(r["screen"][..., 3] == 1)
    r = run(params(), c, hist=hist, mBypassHistoryUpdate=1)
    np.testing.assert_array_equal(r["screen"][..., :3], hist[..., :3])
    np.testing.assert_array_equal(r["history"][..., :3], hist[..., :3])


def test_constant_image_is_a_fixed_point():
    for prec in (32, 64):
        for clip in (0, 1, 2, 3):
            for var in (0, 1):
                c = np.full((12, 10, 4), 0.75, np.float32)
                hist = np.full((12, 10, 4), 0.75, np.float32)
                r = run(params(mColorClampingOrClipping=clip, mVarianceClipping=var), c, hist=hist, precision=prec)
                # FP64 is exact; FP32 mix(h, c, 0.1) = h*0.9f + c*0.1f is within an ulp
                np.testing.assert_allclose(r["history"][..., :3], 0.75, rtol=0 if prec == 64 else 2e-7)


def test_catmullrom_reproduces_history_at_texel_centres_and_linear_ramps():
    h, w = 16, 32  # powers of two: uv and the motion below are exact binary fractions
    hist = np.zeros((h, w, 4), np.float32)
    xs = np.arange(w, dtype=np.float32)
    hist[..., 0] = 0.5 + 0.125 * xs[None, :]
    hist[..., 1] = 1.0 + 0.0625 * np.arange(h, dtype=np.float32)[:, None]
    hist[..., 2] = 2.0
    c = np.ones((h, w, 4), np.float32)
    p = params(mAlpha=0.0, mColorClampingOrClipping=0, mUseYCoCg=0)
    # zero motion: f = 0, Catmull-Rom weights (0, 1, 0, 0) return the texel
    r = run(p, c, hist=hist)
    np.testing.assert_array_equal(r["history"][..., :3], hist[..., :3])
    # a constant fractional shift: a linear ramp is reproduced exactly away from the borders
    vel = np.zeros((h, w, 2), np.float32)
    vel[..., 0] = 0.25 / w
    vel[..., 1] = -0.5 / h
    r = run(p, c, vel=vel, hist=hist)
    inner = (slice(3, h - 3), slice(3, w - 3))
    want_r = 0.5 + 0.125 * (xs[None, :] - 0.25)
    want_g = 1.0 + 0.0625 * (np.arange(h)[:, None] + 0.5)
    np.testing.assert_allclose(r["history"][..., 0][inner], np.broadcast_to(want_r, (h, w))[inner], rtol=1e-12)
    np.testing.assert_allclose(r["history"][..., 1][inner], np.broadcast_to(want_g, (h, w))[inner], rtol=1e-12)


def test_bilinear_and_bspline_modes_on_a_ramp():
    h, w = 8, 32
    hist = np.zeros((h, w, 4), np.float32)
    hist[..., 0] = np.arange(w, dtype=np.float32)[None, :]
    c = np.ones((h, w, 4), np.float32)
    vel = np.zeros((h, w, 2), np.float32)
    vel[..., 0] = 0.375 / w
    p = params(mAlpha=0.0, mColorClampingOrClipping=0, mUseYCoCg=0, mInterpolationMode=0)
    r = run(p, c, vel=vel, hist=hist)
    inner = (slice(None), slice(2, w - 2))
    want = np.arange(w)[None, :] - 0.375
    np.testing.assert_allclose(r["history"][..., 0][inner], np.broadcast_to(want, (h, w))[inner], atol=1e-12)
    # the reference's mode 1 uses Catmull-Rom weights with four bilinear taps
    # (taa.comp:527-542); on a ramp it is not exact but stays within a texel
    p.mInterpolationMode = 1
    r = run(p, c, vel=vel, hist=hist)
    assert np.all(np.abs(r["history"][..., 0][inner] - np.broadcast_to(want, (h, w))[inner]) < 1.0)


def test_clip_is_identity_inside_the_box():
    c = rng_img(7, 9, 9, lo=1.0, hi=2.0)
    # history = current colour: inside every box that contains the centre
    hist = c.copy()
    for clip in (1, 2):
        r = run(params(mColorClampingOrClipping=clip, mVarianceClipping=0, mAlpha=0.0), c, hist=hist)
        np.testing.assert_allclose(r["history"][..., :3], c[..., :3], rtol=1e-15)


def test_clamp_limits_to_the_neighbourhood_box():
    c = rng_img(8, 9, 9, lo=1.0, hi=2.0)
    hist = np.full((9, 9, 4), 10.0, np.float32)
    r = run(params(mColorClampingOrClipping=1, mVarianceClipping=0, mUseYCoCg=0, mAlpha=0.0), c, hist=hist)
    pad = np.pad(c[..., :3], ((1, 1), (1, 1), (0, 0)), mode="edge")
    mx = np.max(np.stack([pad[dy:dy + 9, dx:dx + 9] for dy in range(3) for dx in range(3)]), axis=0)
    np.testing.assert_array_equal(r["history"][..., :3], mx)


def test_reject_outside_and_depth_culling():
    h, w = 8, 8
    c = np.ones((h, w, 4), np.float32)
    hist = np.full((h, w, 4), 3.0, np.float32)
    vel = np.zeros((h, w, 2), np.float32)
    vel[..., 0] = 2.5 / w  # columns 0 and 1 look outside the image (column 2 lands on uv.x = 0)
    p = params(mRejectOutside=1, mColorClampingOrClipping=0, mRejectionAlpha=1.0, mAlpha=0.0)
    r = run(p, c, vel=vel, hist=hist)
    assert np.all(r["history"][:, :2, 0] == 1.0)  # rejected -> alpha 1 -> current
    assert np.all(r["history"][:, 2:, 0] == 3.0)  # kept -> alpha 0 -> history
    # depth culling: previous depth far from the expected depth rejects
    depth = np.full((h, w), 0.5, np.float32)
    hdepth = np.full((h, w), 0.5, np.float32)
    hdepth[:, w // 2:] = 0.9
    p = params(mDepthCulling=1, mColorClampingOrClipping=0, mAlpha=0.0)
    r = run(p, c, depth=depth, hist=hist, hdepth=hdepth)
    assert np.all(r["history"][:, : w // 2, 0] == 3.0)
    assert np.all(r["history"][:, w // 2:, 0] == 1.0)


def test_velocity_mode_1_keeps_the_last_tap():
    # taa.comp:404-412: the 3x3 "longest" search ends with velocitySample.xy = sam,
    # the (1,1) tap, not the longest vector
    h, w = 9, 9
    c = np.ones((h, w, 4), np.float32)
    hist = np.zeros((h, w, 4), np.float32)
    hist[..., 0] = np.arange(w, dtype=np.float32)[None, :]
    vel = np.zeros((h, w, 2), np.float32)
    vel[5, 5, 0] = -1.0 / w  # the (1,1) neighbour of (4,4)
    vel[3, 3, 0] = 3.0 / w   # longer, but not the last tap
    p = params(mVelocitySampleMode=1, mColorClampingOrClipping=0, mUseYCoCg=0, mAlpha=0.0)
    r = run(p, c, vel=vel, hist=hist)
    assert r["history"][4, 4, 0] == pytest.approx(5.0)  # x - (-1)


def test_split_screen_uses_the_second_parameter_set():
    c = np.ones((6, 10, 4), np.float32)
    hist = np.full((6, 10, 4), 2.0, np.float32)
    p0 = params(mAlpha=0.0, mColorClampingOrClipping=0)
    p1 = params(mAlpha=1.0, mColorClampingOrClipping=0)
    u = T.make_uniforms(p0, p1, splitScreen=1, splitX=4)
    r = O.resolve(u, c, np.full((6, 10), 0.5, np.float32), np.zeros((6, 10, 2), np.float32), history=hist,
                  precision=64)
    assert np.all(r["history"][:, :5, 0] == 2.0) and np.all(r["history"][:, 5:, 0] == 1.0)


def test_exponential_blend_converges():
    # static pixels, no rectification: y_n = (1-a) y_{n-1} + a x_n
    p = params(mAlpha=0.1, mColorClampingOrClipping=0, mUseYCoCg=0)
    a = float(np.float32(0.1))  # the parameter block holds 0.1f
    hist = np.zeros((4, 4, 4), np.float32)
    y = 0.0
    for n in range(40):
        x = 1.0 if n % 2 else 3.0
        c = np.full((4, 4, 4), x, np.float32)
        r = run(p, c, hist=hist)
        y = (1 - a) * float(np.float32(y)) + a * x  # the history is stored as FP32 between frames
        np.testing.assert_allclose(r["history"][..., 0], y, rtol=1e-12)
        hist = r["history"].astype(np.float32)



def test_fp32_tracks_fp64_on_the_synthetic_scene(built):
    wl = WL.small(96, 54, frames=2)
    fr = cpu_frames(wl, range(2))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    args = (u, fr[1]["color"].astype(np.float32), fr[1]["depth"], fr[1]["motion"].astype(np.float32))
    kw = dict(history=fr[0]["color"].astype(np.float32), history_depth=fr[0]["depth"])
    r32 = O.resolve(*args, precision=32, **kw)
    r64 = O.resolve(*args, precision=64, **kw)
    rel = np.abs(r32["history"][..., :3] - r64["history"][..., :3]) / np.maximum(np.abs(r64["history"][..., :3]), 1e-3)
    assert rel.mean() < 1e-5
    # FP32 moments cancel in flat neighbourhoods (taa.comp:270 "Here be dragons")
    assert rel.max() < 2e-3


def test_quantize_half_matches_numpy():
    r = np.random.default_rng(9)
    x = np.concatenate([r.standard_normal(10000) * 10.0 ** r.integers(-8, 6, 10000),
                        [0.0, -0.0, 65504.0, 65519.9, 65520.0, 1e-8, 6e-8, 3e-8, -1e10]]).astype(np.float32)
    np.testing.assert_array_equal(O.quantize_half(x), x.astype(np.float16).astype(np.float32))


def test_constant_divisor_division_is_correctly_rounded():
    # x * RN(1/d) plus one residual correction equals IEEE x / d; scaling by a
    # power of two is exact, so one binade of x covers every binade
    one, two = 0x3F800000, 0x40000000
    assert O.check_div_const(9.0, one, two) == 0
    for d in list(range(1, 300)) + [720, 1080, 1280, 1440, 1920, 2160, 2560, 3840, 4096, 7680]:
        assert O.check_div_const(float(d), one, two) == 0, d


def test_cas_and_sharpen_on_flat_images():
    img = np.full((8, 8, 4), 0.5, np.float32)
    s = O.sharpen(img, 0.7)
    np.testing.assert_array_equal(s[..., :3], 0.5)
    c0, c1 = O.cas_setup(0.5, 8, 8, 8, 8)
    out = O.cas(img, c1[0])
    # APrxMedRcpF1 is an approximation: flat input comes back within its error
    np.testing.assert_allclose(out[..., :3], 0.5, rtol=2e-3)
    # HDR input is clipped to [0, 1] (ASatF1)
    out = O.cas(np.full((4, 4, 4), 3.0, np.float32), c1[0])
    np.testing.assert_array_equal(out[..., :3], 1.0)
