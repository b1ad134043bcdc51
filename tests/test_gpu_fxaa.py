"""The FXAA pass (taa_fxaa) and the standalone sharpen pass (taa_sharpen) on the
GPU against the oracle (run with -m gpu).

* FXAA: the kernels compute the prepare pass's FP16 luma and FXAA 3.11 quality
  preset 12 with the oracle's operations in the same order, so their RGBA16F
  output equals the FP32 oracle's value rounded to FP16, bit for bit: on the
  golden fixture's frame and masks, on rendered frames at sizes that are not
  multiples of the block (odd widths, whose rows are not 16-byte aligned, take
  the scalar path), on degenerate sizes, with other settings and with padded
  pitches; on the segmentation mask a resolve writes
  (the reference's ray-trace-assist chain, source/taa.hpp:1063-1104).  With
  and without a context's work list (TAA_FLAG_FXAA).
* sharpen: taa_sharpen equals the oracle's sharpen.comp / CAS to one FP16 ulp,
  like the sharpener fused into the resolve.
"""
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle as O
import taa_abi as T
import workloads as WL
from helpers import cpu_frames, half_ulp, to_dev

pytestmark = pytest.mark.gpu

G = Path(__file__).resolve().parent / "golden"


_CTX = {}


def list_ctx(w, h):
    """A context with the FXAA work list for images up to w x h."""
    if (w, h) not in _CTX:
        _CTX[(w, h)] = T.Taa(w, h, form=T.TAA_FORM_PLAIN, flags=T.TAA_FLAG_FXAA)
    return _CTX[(w, h)]


def run_fxaa(dev, img, seg, params=None, pad=0, ctx=None):
    """taa_fxaa on a numpy RGBA image (FP16 values) and mask; returns the output as float32."""
    h, w = img.shape[:2]
    src = torch.zeros(h, w + pad, 4, dtype=torch.float16, device=dev)
    src[:, :w] = to_dev(img, torch.float16, dev)
    out = torch.full((h, w + pad, 4), float("nan"), dtype=torch.float16, device=dev)
    m = None
    if seg is not None:
        m = torch.zeros(h, w + pad, dtype=torch.int32, device=dev)
        m[:, :w] = torch.from_numpy(np.ascontiguousarray(seg).view(np.int32)).to(dev)
    T.fxaa(src[:, :w], out[:, :w], None if m is None else m[:, :w], params, ctx=ctx)
    torch.cuda.synchronize()
    res = out.float().cpu().numpy()
    if pad:
        assert np.all(np.isnan(res[:, w:])), "the pass wrote outside the image"
    return res[:, :w]


def expected(img, seg, params=None):
    kw = {} if params is None else dict(subpix=params.subpix, edge_threshold=params.edge_threshold,
                                        edge_threshold_min=params.edge_threshold_min)
    ref = O.fxaa(img, seg, precision=32, **kw)
    return ref.astype(np.float32).astype(np.float16).astype(np.float32)


def assert_equal(got, ref):
    bad = np.argwhere(np.any(got != ref, axis=-1))
    assert bad.size == 0, f"{len(bad)} pixels differ, first {bad[:3].tolist()}: {got[tuple(bad[0])]} vs {ref[tuple(bad[0])]}"


def rendered(w, h, seed=3):
    wl = WL.small(w, h, frames=1, seed=seed)
    return cpu_frames(wl, range(1))[0]["color"].astype(np.float32)


def test_golden_frame_and_masks(cuda):
    g = np.load(G / "fxaa_golden.npz")
    img = g["image"]
    h, w = img.shape[:2]
    for name in ("random", "all", "none"):
        seg = g[f"{name}/segmask"]
        got = run_fxaa(cuda, img, seg)
        assert_equal(got, expected(img, seg))
        assert_equal(run_fxaa(cuda, img, seg, ctx=list_ctx(w, h)), got)
        # and close to the reference shader's own FP32 evaluation (its sampler
        # positions in double: a handful of pixels may take another branch)
        ref32 = g[f"{name}/ref32"].astype(np.float64)
        rel = np.abs(got - ref32) / np.maximum(1.0, np.abs(ref32))
        assert np.mean(np.all(rel <= 2e-3, axis=-1)) >= 0.995


@pytest.mark.parametrize("size", [(256, 160), (97, 33), (33, 17), (1, 1), (1, 9), (13, 1), (2, 2)])
def test_rendered_frames(cuda, size):
    w, h = size
    img = rendered(max(w, 8), max(h, 8))[:h, :w]
    img = np.ascontiguousarray(img)
    rng = np.random.default_rng(w * 1000 + h)
    seg = rng.integers(0, 1 << 16, (h, w)).astype(np.uint32)
    for m in (seg, None):
        ref = expected(img, m)
        # without a work list, with one, and with a context too small to lend it
        for c in (None, list_ctx(w, h), list_ctx(max(1, w // 2), h)):
            got = run_fxaa(cuda, img, m, ctx=c)
            assert_equal(got, ref)
    if (w, h) == (256, 160):
        # the pass changes the marked edge pixels only
        changed = np.any(got != expected(img, np.zeros((h, w), np.uint32)), axis=-1)
        assert changed.mean() > 0.05


def test_settings_and_padded_pitch(cuda):
    img = rendered(120, 72, seed=5)
    seg = np.ones((72, 120), np.uint32)
    rng = np.random.default_rng(2)
    half = rng.integers(0, 4, (72, 120)).astype(np.uint32)
    for sub, thr, tmin in ((0.0, 0.166, 0.0625), (1.0, 0.063, 0.0312), (0.75, 0.333, 0.0833)):
        p = T.FxaaParams(sub, thr, tmin)
        for m in (seg, half):
            ref = expected(img, m, p)
            assert_equal(run_fxaa(cuda, img, m, p, pad=24), ref)
            assert_equal(run_fxaa(cuda, img, m, p, pad=24, ctx=list_ctx(120, 72)), ref)


def test_on_the_mask_a_resolve_writes(cuda):
    # the ray-trace-assist chain: resolve (writes the segmentation mask) -> FXAA on its result
    w, h = 160, 96
    wl = WL.small(w, h, frames=2, seed=11, params=dict(mRayTraceAugment=1, mRayTraceAugmentFlags=0x3F | 0x200))
    fr = cpu_frames(wl, range(2))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    ctx = T.Taa(w, h, form=T.TAA_FORM_PLAIN)
    ctx.set_uniforms(u)
    b = dict(color=to_dev(fr[1]["color"], torch.float16, cuda), depth=to_dev(fr[1]["depth"], torch.float32, cuda),
             velocity=to_dev(fr[1]["motion"], torch.float16, cuda),
             history=to_dev(fr[0]["color"].astype(np.float32), torch.float32, cuda),
             history_depth=to_dev(fr[0]["depth"], torch.float32, cuda),
             history_out=torch.empty(h, w, 4, device=cuda), result=torch.empty(h, w, 4, dtype=torch.float16, device=cuda),
             segmask=torch.zeros(h, w, dtype=torch.int32, device=cuda))
    ctx.resolve(**b)
    out = torch.empty(h, w, 4, dtype=torch.float16, device=cuda)
    fctx = T.Taa(w, h, form=T.TAA_FORM_PLAIN, flags=T.TAA_FLAG_FXAA)
    T.fxaa(b["result"], out, b["segmask"], ctx=fctx)
    torch.cuda.synchronize()
    fctx.close()
    seg = b["segmask"].cpu().numpy().view(np.uint32)
    marked = (seg & 3) == 1
    assert 0.0 < marked.mean() < 1.0
    res = b["result"].float().cpu().numpy()
    assert_equal(out.float().cpu().numpy(), expected(res, seg))
    ctx.close()


def test_errors(cuda):
    lib = T.load()
    a = torch.zeros(8, 8, 4, dtype=torch.float16, device=cuda)
    o = torch.zeros(8, 8, 4, dtype=torch.float16, device=cuda)
    pa, po = a.data_ptr(), o.data_ptr()
    f = lambda *args: lib.taa_fxaa(None, None, *args)
    assert f(pa, 64, None, 0, pa, 64, 8, 8, None) == T.TAA_E_INVAL           # output is the input
    assert f(pa, 64, None, 0, pa + 32, 64, 8, 8, None) == T.TAA_E_INVAL      # overlapping rows
    assert f(pa + 2, 64, None, 0, po, 64, 8, 8, None) == T.TAA_E_ALIGN       # misaligned
    assert f(pa, 32, None, 0, po, 64, 8, 8, None) == T.TAA_E_INVAL           # pitch < width * 8
    assert f(pa, 64, None, 0, po, 64, 0, 8, None) == T.TAA_E_INVAL           # empty
    assert f(None, 64, None, 0, po, 64, 8, 8, None) == T.TAA_E_INVAL
    bad = T.FxaaParams(float("nan"), 0.1, 0.1)
    assert f(pa, 64, None, 0, po, 64, 8, 8, bad) == T.TAA_E_INVAL
    assert lib.taa_sharpen(None, 3, 0.5, pa, 64, po, 64, 8, 8) == T.TAA_E_INVAL
    assert lib.taa_sharpen(None, 1, 0.5, pa, 64, pa, 64, 8, 8) == T.TAA_E_INVAL
    d = T.fxaa_default_params()
    assert (d.subpix, d.edge_threshold, d.edge_threshold_min) == (0.75, np.float32(0.116), np.float32(0.0833))


@pytest.mark.parametrize("sharpener", [T.TAA_SHARPEN_SIMPLE, T.TAA_SHARPEN_CAS])
def test_standalone_sharpen(cuda, sharpener):
    img = rendered(75, 41, seed=9)
    img = np.clip(img, 0, 1.5).astype(np.float16).astype(np.float32)
    src = to_dev(img, torch.float16, cuda)
    out = torch.empty_like(src)
    T.sharpen(src, out, sharpener, 0.6)
    torch.cuda.synchronize()
    got = out.float().cpu().numpy()
    if sharpener == T.TAA_SHARPEN_CAS:
        _, c1 = O.cas_setup(0.6, 75, 41, 75, 41)
        ref = O.cas(img, c1[0])
    else:
        ref = O.sharpen(img, 0.6)
    q = ref.astype(np.float32).astype(np.float16).astype(np.float64)
    assert np.all(np.abs(got[..., :3] - q[..., :3]) <= half_ulp(ref[..., :3]) + 1e-12)
    assert np.all(got[..., 3] == 1.0)


CASF = np.load(Path(__file__).resolve().parent / "golden" / "cas_golden.npz")


@pytest.mark.parametrize("key", list(CASF["cases"]))
def test_standalone_cas_matches_the_reference_shader(cuda, key):
    """taa_sharpen with CAS against shaders/sharpen_cas.comp compiled here
    (tests/golden/cas_golden.npz): within one FP16 ulp of the shader's FP32
    result after the RGBA16F store."""
    img, ref = CASF[f"{key}/image"], CASF[f"{key}/ref32"].astype(np.float64)
    h, w = img.shape[:2]
    s = float(key.split("_s")[1])
    src = to_dev(img, torch.float16, cuda)
    out = torch.empty_like(src)
    T.sharpen(src, out, T.TAA_SHARPEN_CAS, s)
    torch.cuda.synchronize()
    got = out.float().cpu().numpy()
    assert np.all(np.abs(got[..., :3] - ref) <= half_ulp(ref) + 1e-12)
    assert np.all(got[..., 3] == 1.0)
