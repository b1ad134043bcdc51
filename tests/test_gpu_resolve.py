"""GPU parity of the resolve forms against the oracle (run with -m gpu).

* plain and tiled forms: both round like the FP32 oracle operation for
                operation (no FMA contraction; explicit FMAs where the oracle
                has them), so the FP32 history accumulator has the oracle's
                bits; the contract they are held to is 1e-4 relative (floor
                1e-3), and the screen is within one FP16 ulp of the oracle's
                value rounded to FP16.
* fused sharpen: the tiled form with CAS / simple sharpen in its epilogue matches
                the oracle's two separate passes (TAA -> FP16 store -> sharpen).
"""
import itertools

import numpy as np
import pytest
import torch

import oracle as O
import taa_abi as T
import workloads as WL
from helpers import cpu_frames, gpu_resolve, half_ulp, max_rel, psnr, rel_l2, to_dev

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4  # FP32 forms vs the FP32 oracle, relative with a 1e-3 floor


def oracle_for(u, fr_cur, fr_prev, history, out_size=None, precision=32, want_debug=False):
    return O.resolve(u, fr_cur["color"].astype(np.float32), fr_cur["depth"], fr_cur["motion"].astype(np.float32),
                     history=history, history_depth=fr_prev["depth"], out_size=out_size, precision=precision,
                     want_debug=want_debug)


def screen_ok(gpu16, ref):
    """GPU screen (FP16-stored) vs oracle value: within one FP16 ulp of the reference."""
    ref = np.asarray(ref, np.float64)
    q = ref.astype(np.float32).astype(np.float16).astype(np.float64)
    return np.all(np.abs(np.asarray(gpu16, np.float64) - q) <= half_ulp(ref) + 1e-12)


MODES = {
    "base": {},
    "c2": dict(mDepthCulling=1, mRejectOutside=1),
    "bilinear": dict(mInterpolationMode=0),
    "bspline": dict(mInterpolationMode=1),
    "clamp_rgb": dict(mColorClampingOrClipping=1, mUseYCoCg=0, mVarianceClipping=0),
    "clip_slow_shaped": dict(mColorClampingOrClipping=3, mShapedNeighbourhood=1, mVarianceClipping=0),
    "shrink_chroma": dict(mShrinkChromaAxis=1),
    "tonemap_lottes": dict(mToneMapLumaKaris=1, mLumaWeightingLottes=1),
    "reduce_blend_velalpha": dict(mReduceBlendNearClamp=1, mVelBasedAlpha=1),
    "closest_velocity": dict(mVelocitySampleMode=2),
    "matrix_reprojection": dict(mUseVelocityVectors=0),
}


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("size", [(33, 31), (17, 9), (64, 36)])
def test_tiled_and_plain_match_oracle(cuda, mode, size):
    w, h = size
    wl = WL.small(w, h, frames=2, params=MODES[mode])
    fr = cpu_frames(wl, range(2), motion_channels=2)
    hist = np.ascontiguousarray(fr[0]["color"].astype(np.float32))
    kw = {}
    if mode == "matrix_reprojection":
        sc = wl.scene()
        p0, v0 = T.synth_camera(sc, 0)
        p1, v1 = T.synth_camera(sc, 1)
        inv, hvp = T.compose_matrices(p1, v1, p0, v0)
        kw = dict(mInverseViewProjMatrix=inv, mHistoryViewProjMatrix=hvp)
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"], **kw)
    ref = oracle_for(u, fr[1], fr[0], hist)
    for form in (T.TAA_FORM_PLAIN, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, form=form)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == form
        out = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"])
        err = max_rel(out["history_out"][..., :3], ref["history"][..., :3])
        assert err <= REL_TOL, (form, err)
        np.testing.assert_array_equal(out["history_out"], ref["history"].astype(np.float32), err_msg=str(form))
        assert screen_ok(out["result"][..., :3], ref["screen"][..., :3]), form
        ctx.close()


def test_plain_form_rounds_like_the_fp32_oracle(cuda):
    wl = WL.small(80, 45, frames=3, params=dict(mDepthCulling=1, mRejectOutside=1))
    fr = cpu_frames(wl, range(3), motion_channels=4)
    hist = np.ascontiguousarray(fr[0]["color"].astype(np.float32))
    ctx = T.Taa(80, 45, motion_format=T.TAA_MOTION_RGBA16F, form=T.TAA_FORM_PLAIN)
    for f in (1, 2):
        u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[f]["jitter"])
        ctx.set_uniforms(u)
        ref = oracle_for(u, fr[f], fr[f - 1], hist)
        out = gpu_resolve(ctx, cuda, fr[f]["color"], fr[f]["depth"], fr[f]["motion"], hist, fr[f - 1]["depth"])
        np.testing.assert_array_equal(out["history_out"], ref["history"].astype(np.float32))
        hist = out["history_out"]


@pytest.mark.parametrize("hist_fp16,motion4", [(False, False), (True, True), (True, False)])
def test_formats(cuda, hist_fp16, motion4):
    w, h = 48, 40
    wl = WL.small(w, h, frames=2)
    fr = cpu_frames(wl, range(2), motion_channels=4 if motion4 else 2)
    hist = fr[0]["color"].astype(np.float32)
    if hist_fp16:
        hist = hist.astype(np.float16).astype(np.float32)
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    ref = oracle_for(u, fr[1], fr[0], hist)
    for form in (T.TAA_FORM_PLAIN, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, form=form, history_format=T.TAA_HISTORY_RGBA16F if hist_fp16 else T.TAA_HISTORY_RGBA32F,
                    motion_format=T.TAA_MOTION_RGBA16F if motion4 else T.TAA_MOTION_RG16F)
        ctx.set_uniforms(u)
        out = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"],
                          history_fp16=hist_fp16)
        if hist_fp16:
            assert screen_ok(out["history_out"][..., :3], ref["history"][..., :3])
        else:
            assert max_rel(out["history_out"][..., :3], ref["history"][..., :3]) <= REL_TOL


@pytest.mark.parametrize("sharpener,interp", [(T.TAA_SHARPEN_CAS, 2), (T.TAA_SHARPEN_CAS, 0), (T.TAA_SHARPEN_SIMPLE, 2)])
@pytest.mark.parametrize("form,flags", [(T.TAA_FORM_TILED, 0), (T.TAA_FORM_TILED, T.TAA_FLAG_FUSED_SHARPEN),
                                        (T.TAA_FORM_PLAIN, 0)])
def test_sharpened_resolve_matches_two_pass_oracle(cuda, sharpener, interp, form, flags):
    """The sharpened image of a resolve with a sharpener - the resolve then the
    sharpen pass, or the tiled form's single launch (TAA_FLAG_FUSED_SHARPEN) -
    is the oracle's sharpener applied to its RGBA16F result image."""
    w, h = 70, 41
    wl = WL.small(w, h, frames=2, params=dict(mInterpolationMode=interp))
    fr = cpu_frames(wl, range(2))
    hist = fr[0]["color"].astype(np.float32)
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    ref = oracle_for(u, fr[1], fr[0], hist)
    screen16 = ref["screen"].astype(np.float32).astype(np.float16).astype(np.float32)  # the RGBA16F result image
    if sharpener == T.TAA_SHARPEN_CAS:
        _, c1 = O.cas_setup(0.5, w, h, w, h)
        sref = O.cas(screen16, c1[0])
    else:
        sref = O.sharpen(screen16, 0.5)
    ctx = T.Taa(w, h, form=form, sharpener=sharpener, sharpen_factor=0.5, flags=flags)
    ctx.set_uniforms(u)
    out = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"],
                      want_result=False, want_sharpened=True)
    assert max_rel(out["history_out"][..., :3], ref["history"][..., :3]) <= REL_TOL
    assert screen_ok(out["sharpened"][..., :3], sref[..., :3])
    assert np.all(out["sharpened"][..., 3] == 1.0)


@pytest.mark.parametrize("size", [(1, 1), (2, 3), (31, 1), (1, 17)])
def test_degenerate_sizes(cuda, size):
    w, h = size
    wl = WL.small(max(w, 4), max(h, 4), frames=2)
    fr = cpu_frames(wl, range(2))
    fr = [{k: (v[:h, :w] if isinstance(v, np.ndarray) else v) for k, v in f.items()} for f in fr]
    hist = np.ascontiguousarray(fr[0]["color"].astype(np.float32))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    ref = oracle_for(u, fr[1], fr[0], hist)
    for form in (T.TAA_FORM_PLAIN, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, form=form, sharpener=T.TAA_SHARPEN_CAS)
        ctx.set_uniforms(u)
        out = gpu_resolve(ctx, cuda, np.ascontiguousarray(fr[1]["color"]), np.ascontiguousarray(fr[1]["depth"]),
                          np.ascontiguousarray(fr[1]["motion"]), hist, np.ascontiguousarray(fr[0]["depth"]),
                          want_sharpened=True)
        assert max_rel(out["history_out"][..., :3], ref["history"][..., :3]) <= REL_TOL


def test_null_history_reads_zeros(cuda):
    w, h = 24, 16
    wl = WL.small(w, h, frames=2)
    fr = cpu_frames(wl, range(2))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"], mResetHistory=1)
    ref = oracle_for(u, fr[1], fr[0], None)
    for form in (T.TAA_FORM_PLAIN, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, form=form)
        ctx.set_uniforms(u)
        out = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], None, fr[0]["depth"])
        assert max_rel(out["history_out"][..., :3], ref["history"][..., :3]) <= REL_TOL


def test_split_screen_debug_passthrough_use_the_plain_form(cuda):
    w, h = 40, 24
    wl = WL.small(w, h, frames=2)
    fr = cpu_frames(wl, range(2), motion_channels=4)
    hist = fr[0]["color"].astype(np.float32)
    p0 = wl.parameters()
    p1 = WL.base_parameters(mPassThrough=1)
    for dbg in range(10):
        p0.mDebugMode = dbg
        u = T.make_uniforms(p0, p1, jitter_ndc=fr[1]["jitter"], splitScreen=1, splitX=19)
        ref = oracle_for(u, fr[1], fr[0], hist, want_debug=True)
        ctx = T.Taa(w, h, motion_format=T.TAA_MOTION_RGBA16F)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == T.TAA_FORM_PLAIN
        out = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"],
                          want_debug=True)
        assert max_rel(out["history_out"][..., :3], ref["history"][..., :3]) <= REL_TOL
        assert screen_ok(out["debug"], ref["debug"]), dbg


def test_validation_errors(cuda):
    import torch
    w, h = 16, 16
    ctx = T.Taa(w, h)
    with pytest.raises(T.TaaError):  # no uniforms yet
        ctx.resolve(color=torch.zeros(h, w, 4, dtype=torch.float16, device=cuda))
    ctx.set_uniforms(T.make_uniforms(WL.base_parameters()))
    col = torch.zeros(h, w, 4, dtype=torch.float16, device=cuda)
    dep = torch.zeros(h, w, dtype=torch.float32, device=cuda)
    vel = torch.zeros(h, w, 2, dtype=torch.float16, device=cuda)
    hist = torch.zeros(h, w, 4, dtype=torch.float32, device=cuda)
    out = torch.zeros(h, w, 4, dtype=torch.float32, device=cuda)
    ctx.resolve(color=col, depth=dep, velocity=vel, history=hist, history_out=out)
    with pytest.raises(T.TaaError) as e:  # aliasing history and history_out
        ctx.resolve(color=col, depth=dep, velocity=vel, history=hist, history_out=hist)
    assert e.value.code == T.TAA_E_INVAL
    with pytest.raises(T.TaaError) as e:  # misaligned colour pointer
        big = torch.zeros(h * w * 4 + 1, dtype=torch.float16, device=cuda)
        ctx.resolve(color=big[1:].view(h, w, 4), depth=dep, velocity=vel, history=hist, history_out=out)
    assert e.value.code == T.TAA_E_ALIGN
    with pytest.raises(T.TaaError):  # missing velocity
        ctx.resolve(color=col, depth=dep, history=hist, history_out=out)
    bad = T.make_uniforms(WL.base_parameters(mAlpha=float("nan")))
    with pytest.raises(T.TaaError):
        ctx.set_uniforms(bad)
    p = WL.base_parameters(mDepthCulling=1)
    ctx.set_uniforms(T.make_uniforms(p))
    with pytest.raises(T.TaaError):  # depth culling needs the previous depth
        ctx.resolve(color=col, depth=dep, velocity=vel, history=hist, history_out=out)
    sctx = T.Taa(w, h, sharpener=T.TAA_SHARPEN_CAS)
    sctx.set_uniforms(T.make_uniforms(WL.base_parameters()))
    img = torch.zeros(h, w, 4, dtype=torch.float16, device=cuda)
    with pytest.raises(T.TaaError) as e:  # the sharpen pass reads the result around each pixel it writes
        sctx.resolve(color=col, depth=dep, velocity=vel, history=hist, history_out=out, result=img, sharpened=img)
    assert e.value.code == T.TAA_E_INVAL
    sctx.close()


def test_gpu_renderer_matches_fp64_scene(cuda):
    import torch
    wl = WL.small(160, 90, frames=3, spin_max=0.05)
    sc = wl.scene()
    sph = T.synth_spheres(sc)
    for f in (0, 2):
        col = torch.zeros(90, 160, 4, dtype=torch.float16, device=cuda)
        dep = torch.zeros(90, 160, dtype=torch.float32, device=cuda)
        mot = torch.zeros(90, 160, 4, dtype=torch.float16, device=cuda)
        tru = torch.zeros(90, 160, 4, dtype=torch.float32, device=cuda)
        T.synth_render(sc, f, color=col, depth=dep, motion=mot, truth=tru)
        torch.cuda.synchronize()
        ref = O.synth_frame(sc, sph, f, truth=True)
        c = col.float().cpu().numpy()
        qc = ref["color"].astype(np.float16).astype(np.float32)
        # FP32 evaluation flips the FP16 rounding of values near a rounding
        # boundary, and discontinuities (checker edges, silhouettes) of
        # samples within FP32 error of an edge
        exact = np.mean(np.all(c == qc, axis=-1))
        near = np.mean(np.all(np.abs(c - ref["color"]) <= 1.01 * half_ulp(ref["color"]), axis=-1))
        assert exact > 0.95 and near > 0.995, (exact, near)
        d = dep.cpu().numpy()
        assert np.mean(np.abs(d - ref["depth"]) < 1e-6) > 0.99
        m = mot.float().cpu().numpy()
        assert np.mean(np.all(np.abs(m - ref["motion"].astype(np.float16)) <= 2 * half_ulp(ref["motion"]), -1)) > 0.99
        t = tru.cpu().numpy()
        assert np.mean(np.abs(t - ref["truth"]) <= 1e-3 * np.maximum(1, np.abs(ref["truth"]))) > 0.99


FP16_MODES = ["base", "c2", "bilinear", "bspline", "clamp_rgb", "clip_slow_shaped", "shrink_chroma",
              "tonemap_lottes", "reduce_blend_velalpha", "closest_velocity"]


@pytest.mark.parametrize("guard", [0, 1], ids=["fast", "guarded"])
@pytest.mark.parametrize("mode", FP16_MODES)
def test_fp16_form_frame_error_vs_fp64(cuda, mode, guard):
    """The FP16 form's contract: per frame, PSNR >= 50 dB against the FP64
    oracle fed the same history, relative L2 <= 1e-2 (see test_gpu_sequences
    for why FP16 chroma cannot hold 1e-3 next to fireflies)."""
    w, h = 96, 64
    wl = WL.small(w, h, frames=2, params=MODES[mode])
    fr = cpu_frames(wl, range(2))
    hist = np.ascontiguousarray(fr[0]["color"].astype(np.float32))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    ref = oracle_for(u, fr[1], fr[0], hist, precision=64)
    ctx = T.Taa(w, h, form=T.TAA_FORM_FP16, flags=T.TAA_FLAG_FP16_GUARD if guard else 0)
    ctx.set_uniforms(u)
    assert ctx.selected_form() == T.TAA_FORM_FP16
    out = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"])
    got, want = out["history_out"][..., :3], ref["history"][..., :3]
    print(mode, "guarded" if guard else "fast", "relL2", rel_l2(got, want), "PSNR", psnr(got, want))
    assert rel_l2(got, want) <= 1e-2, rel_l2(got, want)
    assert psnr(got, want) >= 50.0

def test_device_status_stays_clear(cuda):
    # the tiled forms wait on their history-window copy with a bounded poll;
    # in a normal run no wait gives up, so no status bit is set
    T.device_status(clear=True)
    w, h = 256, 96
    wl = WL.small(w, h, frames=2)
    fr = cpu_frames(wl, range(2))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    hist = fr[0]["color"].astype(np.float32)
    for form in (T.TAA_FORM_TILED, T.TAA_FORM_FP16):
        ctx = T.Taa(w, h, form=form)
        ctx.set_uniforms(u)
        gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"])
        ctx.close()
    assert T.device_status(clear=True) == 0


@pytest.mark.parametrize("mode", ["anti_ghosting", "velocity_longest", "noise", "all_three"])
def test_tiled_and_batch_run_the_extra_modes(cuda, mode):
    """Dynamic anti-ghosting (5-tap mover test, the mask in the history alpha),
    the 3x3-longest velocity (the reference keeps the last tap) and noise run in
    the tiled forms and the batch: on a frame with moving blocks (motion .w set)
    and a history whose alpha marks earlier movers, the tiled form gives the FP32
    oracle's bits (the plain form's for noise, which hashes CUDA's sinf) and the
    batch gives each view the tiled form's bits."""
    w, h = 97, 61
    over = {"anti_ghosting": dict(mDynamicAntiGhosting=1), "velocity_longest": dict(mVelocitySampleMode=1),
            "noise": dict(mAddNoise=1, mNoiseFactor=1.0 / 64.0),
            "all_three": dict(mDynamicAntiGhosting=1, mVelocitySampleMode=1, mAddNoise=1)}[mode]
    wl = WL.small(w, h, frames=2, seed=29, params=dict(mUseVelocityVectors=1, **over))
    fr = cpu_frames(wl, range(2), motion_channels=4)
    rng = np.random.default_rng(3)
    mot = fr[1]["motion"].astype(np.float32)
    yy, xx = np.mgrid[0:h, 0:w]
    movers = ((yy // 8 + xx // 8) % 3) == 0
    mot[..., 3] = np.where(movers, 1.0, 0.0)
    mot[movers, 0] += np.float32(2.0 / w)  # movers move by two texels
    fr[1]["motion"] = mot.astype(np.float16)
    hist = fr[0]["color"].astype(np.float32)
    hist[..., 3] = (rng.uniform(size=(h, w)) < 0.4).astype(np.float32)  # earlier movers
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"], mSinTime=(0.37, 0.0, 0.0, 0.0))
    outs = {}
    for form in (T.TAA_FORM_PLAIN, T.TAA_FORM_TILED, T.TAA_FORM_FP16):
        ctx = T.Taa(w, h, motion_format=T.TAA_MOTION_RGBA16F, form=form)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == form
        outs[form] = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist,
                                 fr[0]["depth"])["history_out"]
        ctx.close()
    tiled, plain = outs[T.TAA_FORM_TILED], outs[T.TAA_FORM_PLAIN]
    if mode in ("noise", "all_three"):
        np.testing.assert_array_equal(tiled, plain)
    else:
        ref = oracle_for(u, fr[1], fr[0], hist)["history"].astype(np.float32)
        np.testing.assert_array_equal(tiled, ref)
        np.testing.assert_array_equal(plain, ref)
    if "anti" in mode or mode == "all_three":
        assert 0.0 < tiled[..., 3].mean() < 1.0  # the mask marks the movers and only them
    np.testing.assert_array_equal(outs[T.TAA_FORM_FP16][..., 3], tiled[..., 3])
    # the batch: two views of the same frame
    b = T.Batch([(w, h), (w, h)], motion_format=T.TAA_MOTION_RGBA16F)
    views = []
    for v in range(2):
        b.set_uniforms(v, u)
        views.append(dict(color=to_dev(fr[1]["color"], torch.float16, cuda),
                          depth=to_dev(fr[1]["depth"], torch.float32, cuda),
                          velocity=to_dev(fr[1]["motion"], torch.float16, cuda),
                          history=to_dev(hist, torch.float32, cuda),
                          history_depth=to_dev(fr[0]["depth"], torch.float32, cuda),
                          history_out=torch.full((h, w, 4), float("nan"), device=cuda),
                          result=torch.empty(h, w, 4, dtype=torch.float16, device=cuda)))
    b.prepare(0, views)
    for shape in ((16, 16), (16, 8)):  # the two-pixel and the one-pixel tile bodies
        b.set_tuning(shape[0], shape[1], T.TAA_SCHEDULE_INTERLEAVED)
        for v in range(2):
            views[v]["history_out"].fill_(float("nan"))
        b.launch(0)
        torch.cuda.synchronize()
        for v in range(2):
            np.testing.assert_array_equal(views[v]["history_out"].cpu().numpy(), tiled)
    b.close()


UP_MODES = {
    "base": {}, "c2": dict(mDepthCulling=1, mRejectOutside=1), "bilinear": dict(mInterpolationMode=0),
    "bspline": dict(mInterpolationMode=1), "clamp_rgb": dict(mColorClampingOrClipping=1, mUseYCoCg=0,
                                                            mVarianceClipping=0),
    "clip_slow_shaped": dict(mColorClampingOrClipping=3, mShapedNeighbourhood=1, mVarianceClipping=0),
    "tonemap_lottes": dict(mToneMapLumaKaris=1, mLumaWeightingLottes=1),
    "reprojection": dict(mUseVelocityVectors=0), "noise": dict(mAddNoise=1),
}


@pytest.mark.parametrize("sizes", [((48, 32), (96, 64)), ((64, 40), (96, 60)), ((80, 45), (97, 61)),
                                   ((40, 40), (40, 72))], ids=["2x", "1.5x", "odd", "one_axis"])
@pytest.mark.parametrize("mode", list(UP_MODES))
def test_upsampling_runs_in_the_tiled_form(cuda, mode, sizes):
    """TAAU (taa.comp:222-257): the tiled form's upsampling path gives the FP32
    oracle's bits (the plain form's for noise, which hashes CUDA's sinf) at
    integer, fractional and one-axis ratios and odd sizes."""
    (w, h), (ow, oh) = sizes
    wl = WL.small(w, h, frames=2, seed=ow + oh, params=UP_MODES[mode])
    fr = cpu_frames(wl, range(2), motion_channels=2)
    rng = np.random.default_rng(ow)
    hist = np.ascontiguousarray(rng.uniform(0.0, 2.0, (oh, ow, 4)).astype(np.float32))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"], mUpsampling=1)
    outs = {}
    for form in (T.TAA_FORM_PLAIN, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, ow, oh, form=form)
        ctx.set_uniforms(u)
        outs[ctx.selected_form()] = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist,
                                                fr[0]["depth"])
        ctx.close()
    assert set(outs) == {T.TAA_FORM_PLAIN, T.TAA_FORM_TILED}
    tiled, plain = outs[T.TAA_FORM_TILED], outs[T.TAA_FORM_PLAIN]
    np.testing.assert_array_equal(tiled["history_out"], plain["history_out"])
    np.testing.assert_array_equal(tiled["result"], plain["result"])
    if mode != "noise":
        ref = oracle_for(u, fr[1], fr[0], hist, out_size=(ow, oh))
        np.testing.assert_array_equal(tiled["history_out"], ref["history"].astype(np.float32))


def test_overlapping_result_and_sharpened_are_rejected(cuda):
    """With a sharpener the sharpen pass reads the result image around every
    pixel it writes, so taa_resolve refuses a sharpened binding inside the
    result image (TAA_E_INVAL before any launch); without a sharpener the same
    bindings are accepted."""
    import ctypes as C
    w, h = 40, 24
    lib = T.load()
    u = T.make_uniforms(T.default_parameters())
    big = torch.zeros((h + 4, w, 4), dtype=torch.float16, device=cuda)  # result; sharpened starts 2 rows in
    bind = dict(color=torch.zeros((h, w, 4), dtype=torch.float16, device=cuda),
                depth=torch.zeros((h, w), dtype=torch.float32, device=cuda),
                velocity=torch.zeros((h, w, 2), dtype=torch.float16, device=cuda),
                history_out=torch.zeros((h, w, 4), dtype=torch.float32, device=cuda))
    io = T.FrameIO()
    for name, t in bind.items():
        p, pitch = T.tensor_ptr_pitch(t)
        setattr(io, name, p)
        setattr(io, name + "_pitch", pitch)
    io.result, io.result_pitch = big.data_ptr(), w * 8
    io.sharpened, io.sharpened_pitch = big.data_ptr() + 2 * w * 8, w * 8
    for sharpener, want in ((T.TAA_SHARPEN_CAS, T.TAA_E_INVAL), (T.TAA_SHARPEN_SIMPLE, T.TAA_E_INVAL),
                            (T.TAA_SHARPEN_OFF, T.TAA_OK)):
        ctx = T.Taa(w, h, form=T.TAA_FORM_TILED, sharpener=sharpener)
        ctx.set_uniforms(u)
        rc = lib.taa_resolve(ctx.handle, None, C.byref(io))
        assert rc == want, (sharpener, rc)
        if want != T.TAA_OK:
            assert b"result and sharpened overlap" in lib.taa_last_error()
        ctx.close()
    torch.cuda.synchronize()
