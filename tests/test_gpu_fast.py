"""TAA_FORM_FAST, the reassociating FP32 resolve (run with -m gpu).

The form computes what the tiled FP32 form computes with the arithmetic
reassociated (shared row sums for the 3x3 moments, contracted FMAs,
hardware square-root and reciprocal approximations), so its contract is a
distance, not bits: frame relative L2 within 1e-5 of the reference shader's
own FP32 output on the golden fixtures (tests/golden) and of the exact tiled
form there, and within 1e-4 relative L2 / 50 dB PSNR of the FP64 oracle on
the benchmark sequences (the benchmark's "within 1e-4 relative").  On those
full frames the form is 2e-5 to 6e-5 from both the FP64 oracle and the FP32
oracle: the algorithm amplifies FP32 rounding (the variance of a flat
neighbourhood, taa.comp:270; the clip toward a near-degenerate box,
taa.comp:335-340), which puts the exact FP32 form itself 1e-5 to 5e-5 from
FP64, so any reassociation lands at that distance from the exact bits.
Parameters outside the benchmark mode run in the exact forms with their bits.
"""
import numpy as np
import pytest
import torch

import oracle as O
import taa_abi as T
import workloads as WL
from helpers import cpu_frames, gpu_resolve, psnr, rel_l2, to_dev
from test_gpu_golden import CASES, FIX, gpu

pytestmark = pytest.mark.gpu

FAST_RELL2 = 1e-5
# fixture cases in the benchmark mode: the fast form runs them
FAST_CASES = ("s:base", "s:c2_depth_reject", "s:bilinear", "s:gamma_1_5", "s:reset")


@pytest.mark.parametrize("key", CASES)
def test_fast_form_on_reference_fixtures(cuda, key):
    used, hist, _ = gpu(key, T.TAA_FORM_FAST, cuda)
    tused, thist, _ = gpu(key, T.TAA_FORM_TILED, cuda)
    if key in FAST_CASES:
        assert used == T.TAA_FORM_FAST
    if used == T.TAA_FORM_FAST:
        ref32 = FIX[f"{key}/ref32_history"].astype(np.float64)
        assert rel_l2(hist[..., :3], ref32[..., :3]) <= FAST_RELL2
        assert rel_l2(hist[..., :3], thist[..., :3]) <= FAST_RELL2
        assert np.all(hist[..., 3] == 0.0)
    else:
        # parameters outside the benchmark mode: the exact forms, their bits
        assert used == tused
        np.testing.assert_array_equal(hist, thist)


def test_auto_selects_the_fast_form_in_the_benchmark_mode(cuda):
    ctx = T.Taa(64, 32)
    for params, want in ((dict(), T.TAA_FORM_FAST), (dict(mDepthCulling=1, mRejectOutside=1), T.TAA_FORM_FAST),
                         (dict(mInterpolationMode=0), T.TAA_FORM_FAST), (dict(mInterpolationMode=1), T.TAA_FORM_TILED),
                         (dict(mToneMapLumaKaris=1), T.TAA_FORM_TILED),
                         (dict(mColorClampingOrClipping=1), T.TAA_FORM_FAST),
                         (dict(mColorClampingOrClipping=3), T.TAA_FORM_TILED),
                         (dict(mShapedNeighbourhood=1, mVarianceClipping=0), T.TAA_FORM_TILED)):
        ctx.set_uniforms(T.make_uniforms(WL.base_parameters(**params)))
        assert ctx.selected_form() == want, params
    ctx.close()
    # RGBA16F history (the reference's own storage) runs in the fast form too, but not
    # with the one-launch sharpener
    ctx = T.Taa(64, 32, history_format=T.TAA_HISTORY_RGBA16F, form=T.TAA_FORM_FAST)
    ctx.set_uniforms(T.make_uniforms(WL.base_parameters()))
    assert ctx.selected_form() == T.TAA_FORM_FAST
    ctx.close()
    ctx = T.Taa(64, 32, history_format=T.TAA_HISTORY_RGBA16F, sharpener=T.TAA_SHARPEN_CAS,
                flags=T.TAA_FLAG_FUSED_SHARPEN)
    ctx.set_uniforms(T.make_uniforms(WL.base_parameters()))
    assert ctx.selected_form() == T.TAA_FORM_TILED
    ctx.close()


@pytest.mark.parametrize("size", [(70, 41), (17, 9), (33, 31), (256, 144), (1, 1), (40, 1), (1, 40)])
@pytest.mark.parametrize("mode", ["c2", "bilinear", "rgba16f_motion", "first_frame"])
def test_fast_form_against_the_exact_form(cuda, size, mode):
    w, h = size
    params = dict(mDepthCulling=1, mRejectOutside=1) if mode == "c2" else \
        dict(mInterpolationMode=0) if mode == "bilinear" else {}
    mc = 4 if mode == "rgba16f_motion" else 2
    wl = WL.small(w, h, frames=2, seed=w * 7 + h, params=params)
    fr = cpu_frames(wl, range(2), motion_channels=mc)
    hist = None if mode == "first_frame" else fr[0]["color"].astype(np.float32)
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"], mResetHistory=1 if mode == "first_frame" else 0)
    outs = {}
    for form in (T.TAA_FORM_FAST, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, form=form, motion_format=T.TAA_MOTION_RGBA16F if mc == 4 else T.TAA_MOTION_RG16F)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == form
        outs[form] = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"])
        ctx.close()
    f, t = outs[T.TAA_FORM_FAST], outs[T.TAA_FORM_TILED]
    assert np.all(np.isfinite(f["history_out"]))
    # on frames of a few dozen pixels one pixel whose clip is ill-conditioned
    # (a near-degenerate box channel, taa.comp:335-340) decides the frame norm:
    # there the fast form must be as close to the FP64 oracle as the exact form
    r64 = O.resolve(u, fr[1]["color"].astype(np.float32), fr[1]["depth"], fr[1]["motion"].astype(np.float32),
                    history=hist, history_depth=fr[0]["depth"], precision=64)["history"][..., :3]
    e_fast, e_exact = rel_l2(f["history_out"][..., :3], r64), rel_l2(t["history_out"][..., :3], r64)
    assert e_fast <= max(FAST_RELL2, 3.0 * e_exact), (e_fast, e_exact)
    assert rel_l2(f["history_out"][..., :3], t["history_out"][..., :3]) <= 1e-3
    assert rel_l2(f["result"][..., :3], t["result"][..., :3]) <= 1e-3  # after the RGBA16F store
    assert np.all(f["result"][..., 3] == 1.0)
    assert T.device_status(clear=True) == 0


def render(wl, sc, f, dev):
    H, W = wl.height, wl.width
    col = torch.empty(H, W, 4, dtype=torch.float16, device=dev)
    dep = torch.empty(H, W, dtype=torch.float32, device=dev)
    mot = torch.empty(H, W, 2, dtype=torch.float16, device=dev)
    T.synth_render(sc, f, color=col, depth=dep, motion=mot)
    return col, dep, mot


@pytest.mark.parametrize("name,frames,check", [("c1", 16, range(1, 16)), ("c2", 6, (1, 5)), ("c3", 6, (1, 5))])
def test_fast_form_sequences_against_fp64(cuda, name, frames, check):
    """Each checked frame against the FP64 oracle fed the same history: relative
    L2 <= 1e-4 and PSNR >= 50 dB (the exact forms' bar); and within 1e-4 of
    the exact FP32 oracle's resolve of the same frame."""
    wl = {"c1": WL.c1, "c2": WL.c2, "c3": WL.c3}[name]()
    sc = wl.scene()
    H, W = wl.height, wl.width
    ctx = T.Taa(W, H, form=T.TAA_FORM_FAST)
    hist = torch.zeros(H, W, 4, device=cuda)
    hout = torch.empty_like(hist)
    prev = None
    rep = []
    for f in range(frames):
        col, dep, mot = render(wl, sc, f, cuda)
        u = T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(sc, f)[1], mResetHistory=1 if f == 0 else 0)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == T.TAA_FORM_FAST
        pd = prev if prev is not None else dep
        ctx.resolve(color=col, depth=dep, velocity=mot, history=hist, history_depth=pd, history_out=hout)
        torch.cuda.synchronize()
        if f in check:
            args = (u, col.float().cpu().numpy(), dep.cpu().numpy(), mot.float().cpu().numpy())
            kw = dict(history=hist.cpu().numpy(), history_depth=pd.cpu().numpy())
            got = hout.cpu().numpy()[..., :3]
            r32 = O.resolve(*args, **kw)["history"][..., :3]
            r64 = O.resolve(*args, precision=64, **kw)["history"][..., :3]
            rep.append((f, rel_l2(got, r32), rel_l2(got, r64), psnr(got, r64)))
        hist, hout = hout, hist
        prev = dep
    ctx.close()
    print(f"{name} fast form (frame, relL2 vs FP32 oracle, relL2 vs FP64, PSNR vs FP64):", rep)
    assert max(r[1] for r in rep) <= 1e-4
    assert max(r[2] for r in rep) <= 1e-4
    assert min(r[3] for r in rep) >= 50.0


@pytest.mark.parametrize("form", [T.TAA_FORM_FAST, T.TAA_FORM_TILED], ids=["fast", "tiled"])
def test_result_in_pinned_host_memory(cuda, form):
    """The result binding may be pinned host memory: the kernel's stores cross
    the host link and give the same bits as a device image."""
    wl = WL.small(200, 120, frames=2, seed=21)
    sc = wl.scene()
    H, W = wl.height, wl.width
    col = torch.empty(2, H, W, 4, dtype=torch.float16, device=cuda)
    dep = torch.empty(2, H, W, device=cuda)
    mot = torch.empty(2, H, W, 2, dtype=torch.float16, device=cuda)
    for f in range(2):
        T.synth_render(sc, f, color=col[f], depth=dep[f], motion=mot[f])
    ctx = T.Taa(W, H, form=form)
    ctx.set_uniforms(T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(sc, 1)[1]))
    hist = col[0].float()
    host = torch.full((H, W, 4), float("nan"), dtype=torch.float16).pin_memory()
    dev_res = torch.full((H, W, 4), float("nan"), dtype=torch.float16, device=cuda)
    outs = []
    for res in (host, dev_res):
        h = torch.empty(H, W, 4, device=cuda)
        ctx.resolve(color=col[1], depth=dep[1], velocity=mot[1], history=hist, history_depth=dep[0], history_out=h,
                    result=res)
        torch.cuda.synchronize()
        outs.append(res.cpu())
    ctx.close()
    assert torch.equal(outs[0], outs[1]) and not torch.isnan(outs[0]).any()


@pytest.mark.parametrize("size", [(200, 120), (61, 37), (256, 160), (1, 1), (40, 1), (1, 40), (31, 15)],
                         ids=lambda s: f"{s[0]}x{s[1]}")
@pytest.mark.parametrize("interp", [2, 0], ids=["catmull_rom", "bilinear"])
@pytest.mark.parametrize("sharpener", [T.TAA_SHARPEN_CAS, T.TAA_SHARPEN_SIMPLE], ids=["cas", "simple"])
def test_fused_sharpen_equals_two_passes(cuda, size, interp, sharpener):
    """TAA_FLAG_FUSED_SHARPEN on the fast form (one launch, each 30x14 tile
    resolved with its ring) gives the two-pass form's bits: history, result
    and sharpened image, over a 4-frame chain."""
    W, H = size
    wl = WL.small(W, H, frames=4, seed=23, params=dict(mInterpolationMode=interp))
    sc = wl.scene()
    F = 4
    col = torch.empty(F, H, W, 4, dtype=torch.float16, device=cuda)
    dep = torch.empty(F, H, W, device=cuda)
    mot = torch.empty(F, H, W, 2, dtype=torch.float16, device=cuda)
    for f in range(F):
        T.synth_render(sc, f, color=col[f], depth=dep[f], motion=mot[f])
    outs = []
    for flags in (0, T.TAA_FLAG_FUSED_SHARPEN):
        ctx = T.Taa(W, H, form=T.TAA_FORM_AUTO, sharpener=sharpener, sharpen_factor=0.5, flags=flags)
        hist = [torch.zeros(H, W, 4, device=cuda) for _ in range(2)]
        frames = []
        for f in range(F):
            ctx.set_uniforms(T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(sc, f)[1],
                                             mResetHistory=1 if f == 0 else 0))
            assert ctx.selected_form() == T.TAA_FORM_FAST
            res = torch.full((H, W, 4), float("nan"), dtype=torch.float16, device=cuda)
            shp = torch.full((H, W, 4), float("nan"), dtype=torch.float16, device=cuda)
            ctx.resolve(color=col[f], depth=dep[f], velocity=mot[f], history=hist[f & 1],
                        history_depth=dep[f - 1] if f else dep[0], history_out=hist[(f + 1) & 1], result=res,
                        sharpened=shp)
            torch.cuda.synchronize()
            frames.append((hist[(f + 1) & 1][..., :3].clone(), res.clone(), shp.clone()))
        outs.append(frames)
        ctx.close()
    for f in range(F):
        for two, one, name in zip(outs[0][f], outs[1][f], ("history", "result", "sharpened")):
            assert not torch.isnan(one).any(), (f, name)
            assert torch.equal(two, one), (f, name, float((two.float() - one.float()).abs().max()))
    assert T.device_status(clear=True) == 0


def test_fp16_context_with_fused_sharpener_runs_the_fast_one_launch_kernel(cuda):
    W, H = 96, 64
    wl = WL.small(W, H, frames=2, seed=29)
    sc = wl.scene()
    col = torch.empty(2, H, W, 4, dtype=torch.float16, device=cuda)
    dep = torch.empty(2, H, W, device=cuda)
    mot = torch.empty(2, H, W, 2, dtype=torch.float16, device=cuda)
    for f in range(2):
        T.synth_render(sc, f, color=col[f], depth=dep[f], motion=mot[f])
    u = T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(sc, 1)[1])
    outs = []
    for form in (T.TAA_FORM_FP16, T.TAA_FORM_FAST):
        ctx = T.Taa(W, H, form=form, sharpener=T.TAA_SHARPEN_CAS, flags=T.TAA_FLAG_FUSED_SHARPEN)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == T.TAA_FORM_FAST
        h = torch.empty(H, W, 4, device=cuda)
        shp = torch.empty(H, W, 4, dtype=torch.float16, device=cuda)
        ctx.resolve(color=col[1], depth=dep[1], velocity=mot[1], history=col[0].float(), history_depth=dep[0],
                    history_out=h, sharpened=shp)
        torch.cuda.synchronize()
        outs.append((h.clone(), shp.clone()))
        ctx.close()
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])


def skew_matrices(u, seed):
    """Non-trivial inverse view-projection and history view-projection matrices
    (identity plus small seeded terms, w kept near 1) for the reprojection path."""
    rng = np.random.default_rng(seed)
    for name in ("mInverseViewProjMatrix", "mHistoryViewProjMatrix"):
        m = np.eye(4) + rng.uniform(-0.03, 0.03, (4, 4))
        m[3, 3] = 1.0
        arr = getattr(u, name)
        for i, v in enumerate(m.T.ravel()):  # column-major
            arr[i] = float(v)
    return u


@pytest.mark.parametrize("size", [(70, 41), (33, 31), (256, 144), (1, 1), (40, 1), (1, 40)],
                         ids=lambda s: f"{s[0]}x{s[1]}")
@pytest.mark.parametrize("vel", [0, 1, 2], ids=["reproject", "movers", "velocity"])
@pytest.mark.parametrize("interp,mc", [(0, 2), (2, 4), (0, 4)], ids=["bilinear-rg", "cr-rgba", "bilinear-rgba"])
def test_fast_form_in_the_reference_default_mode(cuda, size, vel, interp, mc):
    """The reference's default parameter block (RGB, 3x3 min/max box, clamp,
    alpha 0.05) with each velocity use runs in the fast form (AUTO's choice)
    and is as close to the FP64 oracle as the exact form (within 1e-5 relative
    L2, or three times the exact form's distance on frames whose norm one
    pixel decides), and within 1e-4 of the exact form."""
    w, h = size
    p = T.default_parameters()
    p.mUseVelocityVectors, p.mInterpolationMode = vel, interp
    wl = WL.small(w, h, frames=2, seed=w * 5 + h + vel)
    fr = cpu_frames(wl, range(2), motion_channels=mc)
    u = skew_matrices(T.make_uniforms(p, jitter_ndc=fr[1]["jitter"]), seed=vel + 3)
    hist = fr[0]["color"].astype(np.float32)
    outs = {}
    for form in (T.TAA_FORM_AUTO, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, form=form, motion_format=T.TAA_MOTION_RGBA16F if mc == 4 else T.TAA_MOTION_RG16F)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == (T.TAA_FORM_FAST if form == T.TAA_FORM_AUTO else T.TAA_FORM_TILED)
        outs[form] = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"])
        ctx.close()
    f, t = outs[T.TAA_FORM_AUTO], outs[T.TAA_FORM_TILED]
    assert np.all(np.isfinite(f["history_out"]))
    r64 = O.resolve(u, fr[1]["color"].astype(np.float32), fr[1]["depth"], fr[1]["motion"].astype(np.float32),
                    history=hist, history_depth=fr[0]["depth"], precision=64)["history"][..., :3]
    e_fast, e_exact = rel_l2(f["history_out"][..., :3], r64), rel_l2(t["history_out"][..., :3], r64)
    assert e_fast <= max(FAST_RELL2, 3.0 * e_exact), (e_fast, e_exact)
    assert rel_l2(f["history_out"][..., :3], t["history_out"][..., :3]) <= 1e-4
    assert np.all(f["history_out"][..., 3] == t["history_out"][..., 3])
    assert T.device_status(clear=True) == 0


def test_reference_default_mode_sequence_against_fp64(cuda):
    """C1 (1280x720) with the reference's default parameter block, 8 frames:
    every frame from frame 1 within 1e-4 relative L2 of the FP32 and the FP64
    oracle fed the same history."""
    wl = WL.c1()
    sc = wl.scene()
    H, W = wl.height, wl.width
    p = T.default_parameters()
    ctx = T.Taa(W, H)
    hist = torch.zeros(H, W, 4, device=cuda)
    hout = torch.empty_like(hist)
    prev = None
    rep = []
    for f in range(8):
        col, dep, mot = render(wl, sc, f, cuda)
        u = T.make_uniforms(p, jitter_ndc=T.synth_jitter(sc, f)[1], mResetHistory=1 if f == 0 else 0)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == T.TAA_FORM_FAST
        pd = prev if prev is not None else dep
        ctx.resolve(color=col, depth=dep, velocity=mot, history=hist, history_depth=pd, history_out=hout)
        torch.cuda.synchronize()
        if f >= 1:
            args = (u, col.float().cpu().numpy(), dep.cpu().numpy(), mot.float().cpu().numpy())
            kw = dict(history=hist.cpu().numpy(), history_depth=pd.cpu().numpy())
            got = hout.cpu().numpy()[..., :3]
            r32 = O.resolve(*args, **kw)["history"][..., :3]
            r64 = O.resolve(*args, precision=64, **kw)["history"][..., :3]
            rep.append((f, rel_l2(got, r32), rel_l2(got, r64)))
        hist, hout = hout, hist
        prev = dep
    ctx.close()
    print("C1 reference defaults, fast form (frame, relL2 vs FP32, vs FP64):", rep)
    assert max(r[1] for r in rep) <= 1e-4 and max(r[2] for r in rep) <= 1e-4


@pytest.mark.parametrize("size", [(70, 41), (256, 144), (33, 31), (1, 1), (40, 1)], ids=lambda s: f"{s[0]}x{s[1]}")
@pytest.mark.parametrize("mode", ["benchmark", "defaults"])
def test_fast_form_with_rgba16f_history(cuda, size, mode):
    """RGBA16F history (the reference's TAA_IMAGE_FORMAT_RGB) in the fast form: the
    window holds RGBA16F texels, the history is stored as RGBA16F.  Against the
    exact form with the same storage: most pixels round to the same FP16 value,
    the rest one FP16 step apart (frame relative L2 within 5e-4); against the
    FP64 oracle fed the same FP16 history, within 5e-4 after the store as well."""
    w, h = size
    if mode == "defaults":
        p = T.default_parameters()
        wl = WL.small(w, h, frames=2, seed=w + 3 * h)
    else:
        wl = WL.small(w, h, frames=2, seed=w + 3 * h, params=dict(mDepthCulling=1, mRejectOutside=1))
        p = wl.parameters()
    fr = cpu_frames(wl, range(2))
    hist = fr[0]["color"].astype(np.float16).astype(np.float32)
    u = T.make_uniforms(p, jitter_ndc=fr[1]["jitter"])
    outs = {}
    for form in (T.TAA_FORM_AUTO, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, form=form, history_format=T.TAA_HISTORY_RGBA16F)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == (T.TAA_FORM_FAST if form == T.TAA_FORM_AUTO else T.TAA_FORM_TILED)
        outs[form] = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"],
                                 history_fp16=True)
        ctx.close()
    f, t = outs[T.TAA_FORM_AUTO]["history_out"], outs[T.TAA_FORM_TILED]["history_out"]
    assert np.all(np.isfinite(f))
    assert rel_l2(f[..., :3], t[..., :3]) <= 5e-4
    r64 = O.resolve(u, fr[1]["color"].astype(np.float32), fr[1]["depth"], fr[1]["motion"].astype(np.float32),
                    history=hist, history_depth=fr[0]["depth"], precision=64)["history"][..., :3]
    r64h = r64.astype(np.float16).astype(np.float64)
    assert rel_l2(f[..., :3], r64h) <= max(5e-4, 3.0 * rel_l2(t[..., :3], r64h))
    assert T.device_status(clear=True) == 0


def test_rgba16f_history_chain_at_4k(cuda):
    """The C2 workload's first 16 frames with RGBA16F history, fast form against the
    exact form, each on its own history.  FP16 storage has a dead band: a blend step
    smaller than half an FP16 step of the history (|alpha (c - h)| < 2^-12 |h|) does
    not move it, so two chains whose arithmetic differs by a rounding settle up to
    about 2^-12 / alpha = 2.4e-3 relative apart per pixel (measured frame relative
    L2 1.2e-3 at frame 8, 2.2e-3 at frame 15).  Bar 5e-3; each single resolve from
    the same history is within 5e-4 (the test above)."""
    wl = WL.c2()
    sc = wl.scene()
    H, W = wl.height, wl.width
    ctxs = {f: T.Taa(W, H, form=f, history_format=T.TAA_HISTORY_RGBA16F) for f in (T.TAA_FORM_AUTO, T.TAA_FORM_TILED)}
    hists = {f: [torch.zeros(H, W, 4, dtype=torch.float16, device=cuda) for _ in range(2)] for f in ctxs}
    prev = None
    rep = []
    for fi in range(16):
        col, dep, mot = render(wl, sc, fi, cuda)
        u = T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(sc, fi)[1], mResetHistory=1 if fi == 0 else 0)
        for f, ctx in ctxs.items():
            ctx.set_uniforms(u)
            hb = hists[f]
            ctx.resolve(color=col, depth=dep, velocity=mot, history=hb[fi & 1], history_depth=prev if prev is not None else dep,
                        history_out=hb[(fi + 1) & 1])
        torch.cuda.synchronize()
        if fi in (8, 15):
            a = hists[T.TAA_FORM_AUTO][(fi + 1) & 1][..., :3].float().cpu().numpy()
            b = hists[T.TAA_FORM_TILED][(fi + 1) & 1][..., :3].float().cpu().numpy()
            rep.append((fi, rel_l2(a, b)))
        prev = dep
    assert ctxs[T.TAA_FORM_AUTO].selected_form() == T.TAA_FORM_FAST
    for ctx in ctxs.values():
        ctx.close()
    print("C2 RGBA16F history, fast vs exact (frame, relL2):", rep)
    assert all(e <= 5e-3 for _, e in rep), rep


@pytest.mark.parametrize("sizes", [((48, 32), (96, 64)), ((64, 40), (96, 60)), ((80, 45), (97, 61)),
                                   ((40, 40), (40, 72)), ((960, 540), (1920, 1080)), ((7, 5), (13, 9))],
                         ids=["2x", "1.5x", "odd", "one_axis", "1080p", "tiny"])
@pytest.mark.parametrize("mode", ["base", "c2", "bilinear", "rgba16f_motion", "first_frame"])
def test_fast_upsampling(cuda, sizes, mode):
    """TAAU in the fast form (AUTO's choice in the benchmark mode): as close to the
    FP64 oracle as the exact tiled form's upsampling path (within 1e-5 relative L2,
    or three times the exact form's distance on frames a few pixels decide), and
    within 1e-4 of it."""
    (w, h), (ow, oh) = sizes
    params = dict(mDepthCulling=1, mRejectOutside=1) if mode == "c2" else \
        dict(mInterpolationMode=0) if mode == "bilinear" else {}
    mc = 4 if mode == "rgba16f_motion" else 2
    wl = WL.small(w, h, frames=2, seed=ow + 7 * oh, params=params)
    fr = cpu_frames(wl, range(2), motion_channels=mc)
    rng = np.random.default_rng(ow)
    hist = None if mode == "first_frame" else np.ascontiguousarray(rng.uniform(0.0, 2.0, (oh, ow, 4)).astype(np.float32))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"], mUpsampling=1,
                        mResetHistory=1 if mode == "first_frame" else 0)
    outs = {}
    for form in (T.TAA_FORM_AUTO, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, ow, oh, form=form, motion_format=T.TAA_MOTION_RGBA16F if mc == 4 else T.TAA_MOTION_RG16F)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == (T.TAA_FORM_FAST if form == T.TAA_FORM_AUTO else T.TAA_FORM_TILED)
        outs[form] = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"])
        ctx.close()
    f, t = outs[T.TAA_FORM_AUTO], outs[T.TAA_FORM_TILED]
    assert np.all(np.isfinite(f["history_out"]))
    r64 = O.resolve(u, fr[1]["color"].astype(np.float32), fr[1]["depth"], fr[1]["motion"].astype(np.float32),
                    history=hist, history_depth=fr[0]["depth"], out_size=(ow, oh), precision=64)["history"][..., :3]
    e_fast, e_exact = rel_l2(f["history_out"][..., :3], r64), rel_l2(t["history_out"][..., :3], r64)
    assert e_fast <= max(FAST_RELL2, 3.0 * e_exact), (e_fast, e_exact)
    assert rel_l2(f["history_out"][..., :3], t["history_out"][..., :3]) <= 1e-4
    assert np.all(f["history_out"][..., 3] == 0.0)
    assert T.device_status(clear=True) == 0


GEN_MODES = {f"{'ycocg' if yc else 'rgb'}-{'var' if var else 'minmax'}-{'clamp' if rect == 1 else 'clip'}":
             dict(mUseYCoCg=yc, mVarianceClipping=var, mColorClampingOrClipping=rect)
             for yc in (0, 1) for var in (0, 1) for rect in (1, 2)}


@pytest.mark.parametrize("mode", list(GEN_MODES))
@pytest.mark.parametrize("vel", [0, 2], ids=["reproject", "velocity"])
@pytest.mark.parametrize("interp", [2, 0], ids=["catmull_rom", "bilinear"])
def test_fast_form_in_every_rectification_mode(cuda, mode, vel, interp):
    """Every combination of colour space (YCoCg, RGB), box (variance, min/max)
    and rectification (clamp, clip toward the centre) with either velocity use
    runs in the fast form (AUTO's choice), as close to the FP64 oracle as the
    exact form and within 1e-4 of it."""
    w, h = 96, 56
    p = T.default_parameters()
    for k, v in GEN_MODES[mode].items():
        setattr(p, k, v)
    p.mUseVelocityVectors, p.mInterpolationMode, p.mAlpha = vel, interp, 0.1
    wl = WL.small(w, h, frames=2, seed=len(mode) * 7 + vel + interp)
    fr = cpu_frames(wl, range(2), motion_channels=2)
    u = skew_matrices(T.make_uniforms(p, jitter_ndc=fr[1]["jitter"]), seed=vel + interp)
    hist = fr[0]["color"].astype(np.float32)
    outs = {}
    for form in (T.TAA_FORM_AUTO, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, form=form)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == (T.TAA_FORM_FAST if form == T.TAA_FORM_AUTO else T.TAA_FORM_TILED)
        outs[form] = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"])
        ctx.close()
    f, t = outs[T.TAA_FORM_AUTO], outs[T.TAA_FORM_TILED]
    assert np.all(np.isfinite(f["history_out"]))
    r64 = O.resolve(u, fr[1]["color"].astype(np.float32), fr[1]["depth"], fr[1]["motion"].astype(np.float32),
                    history=hist, history_depth=fr[0]["depth"], precision=64)["history"][..., :3]
    e_fast, e_exact = rel_l2(f["history_out"][..., :3], r64), rel_l2(t["history_out"][..., :3], r64)
    assert e_fast <= max(FAST_RELL2, 3.0 * e_exact), (e_fast, e_exact)
    assert rel_l2(f["history_out"][..., :3], t["history_out"][..., :3]) <= 1e-4
    assert T.device_status(clear=True) == 0


@pytest.mark.parametrize("extra", [dict(mVelBasedAlpha=1), dict(mLumaWeightingLottes=1), dict(mReduceBlendNearClamp=1),
                                   dict(mShrinkChromaAxis=1), dict(mVelBasedAlpha=1, mLumaWeightingLottes=1,
                                                                   mReduceBlendNearClamp=1, mShrinkChromaAxis=1)],
                         ids=["vel_alpha", "lottes", "near_clamp", "shrink_chroma", "all"])
@pytest.mark.parametrize("mode", ["ycocg-var-clip", "ycocg-minmax-clamp", "rgb-minmax-clamp", "rgb-var-clip"])
def test_fast_form_with_blend_modifiers(cuda, extra, mode):
    """The blend-weight modifiers (velocity-based alpha, luma weighting, near-clamp
    reduction) and the chroma-axis shrink in the fast form, against the exact form
    and FP64 as above."""
    w, h = 96, 56
    p = WL.base_parameters(**GEN_MODES[mode], **extra)
    wl = WL.small(w, h, frames=2, seed=len(mode) + len(extra))
    fr = cpu_frames(wl, range(2), motion_channels=2)
    u = T.make_uniforms(p, jitter_ndc=fr[1]["jitter"])
    hist = fr[0]["color"].astype(np.float32)
    outs = {}
    for form in (T.TAA_FORM_AUTO, T.TAA_FORM_TILED):
        ctx = T.Taa(w, h, form=form)
        ctx.set_uniforms(u)
        assert ctx.selected_form() == (T.TAA_FORM_FAST if form == T.TAA_FORM_AUTO else T.TAA_FORM_TILED)
        outs[form] = gpu_resolve(ctx, cuda, fr[1]["color"], fr[1]["depth"], fr[1]["motion"], hist, fr[0]["depth"])
        ctx.close()
    f, t = outs[T.TAA_FORM_AUTO], outs[T.TAA_FORM_TILED]
    assert np.all(np.isfinite(f["history_out"]))
    r64 = O.resolve(u, fr[1]["color"].astype(np.float32), fr[1]["depth"], fr[1]["motion"].astype(np.float32),
                    history=hist, history_depth=fr[0]["depth"], precision=64)["history"][..., :3]
    e_fast, e_exact = rel_l2(f["history_out"][..., :3], r64), rel_l2(t["history_out"][..., :3], r64)
    assert e_fast <= max(FAST_RELL2, 3.0 * e_exact), (e_fast, e_exact)
    assert rel_l2(f["history_out"][..., :3], t["history_out"][..., :3]) <= 1e-4
    assert T.device_status(clear=True) == 0
