"""The ray-trace-assist classification (segmentation mask, taa.comp:558-702) in
the tiled forms, run with -m gpu: on rendered frames with seeded material ids
and normals, every flag alone and together, with the history count and with a
previous mask, at ragged sizes, the tiled FP32 form gives the plain form's
history and mask bit for bit (both classify through segmentation.cuh, the
plain form on global memory, the tiled form on a staged tile), and the FP16
form the plain form's mask."""
import numpy as np
import pytest
import torch

import taa_abi as T
import workloads as WL
from helpers import cpu_frames, psnr, to_dev

pytestmark = pytest.mark.gpu

F = T.RTFLAG
FLAGS = {
    "out": F["OUT"], "dis": F["DIS"], "nrm": F["NRM"], "dpt": F["DPT"], "mid": F["MID"], "lum": F["LUM"],
    "edges": F["NRM"] | F["DPT"] | F["MID"] | F["LUM"],
    "all_tests_count": 0x7F, "fixed_border": F["FXD"] | 0x3F, "everything": F["ALL"],
}


def inputs(w, h, seed):
    wl = WL.small(w, h, frames=2, seed=seed, params=dict(mDepthCulling=1, mRejectOutside=1))
    fr = cpu_frames(wl, range(2), motion_channels=2)
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    mat = (((yy // 20) * 31 + (xx // 24) * 17) % 5 + 1).astype(np.uint32)
    mat[(mat % 3) == 0] |= np.uint32(0x80000000)  # movers: whole blocks
    pmat = np.roll(mat, 2, axis=1)
    blk = rng.uniform(size=(h // 16 + 1, w // 16 + 1, 4)).astype(np.float32)
    uvn = np.repeat(np.repeat(blk, 16, 0), 16, 1)[:h, :w].copy()
    uvn[..., 2] *= 6.28
    uvn[..., 3] = uvn[..., 3] * 3.0 - 1.5
    pseg = ((rng.integers(0, 5, (h, w)).astype(np.uint32) << 16) | rng.integers(0, 3, (h, w)).astype(np.uint32))
    return wl, fr, mat, pmat, uvn, pseg


def run(dev, form, wl, fr, mat, pmat, uvn, pseg, flags):
    h, w = wl.height, wl.width
    p = wl.parameters()
    p.mRayTraceAugment = 1
    p.mRayTraceAugmentFlags = flags
    p.mRayTraceHistoryCount = 6
    p.mRayTraceAugment_WNrm, p.mRayTraceAugment_WDpt = 1.0, 0.01
    p.mRayTraceAugment_WMId, p.mRayTraceAugment_WLum = 0.7, 0.02
    p.mRayTraceAugment_Thresh = 0.5
    u = T.make_uniforms(p, jitter_ndc=fr[1]["jitter"], mCamNearPlane=0.1, mCamFarPlane=100.0)
    ctx = T.Taa(w, h, form=form)
    ctx.set_uniforms(u)
    i32 = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)
    b = dict(color=to_dev(fr[1]["color"], torch.float16, dev), depth=to_dev(fr[1]["depth"], torch.float32, dev),
             velocity=to_dev(fr[1]["motion"], torch.float16, dev),
             history=to_dev(fr[0]["color"].astype(np.float32), torch.float32, dev),
             history_depth=to_dev(fr[0]["depth"], torch.float32, dev), material=i32(mat), prev_material=i32(pmat),
             uvnrm=to_dev(uvn, torch.float32, dev), prev_segmask=i32(pseg),
             history_out=torch.full((h, w, 4), float("nan"), device=dev),
             result=torch.full((h, w, 4), float("nan"), dtype=torch.float16, device=dev),
             segmask=torch.full((h, w), -1, dtype=torch.int32, device=dev))
    used = ctx.selected_form()
    ctx.resolve(**b)
    torch.cuda.synchronize()
    ctx.close()
    return used, b["history_out"].cpu().numpy(), b["segmask"].cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("size", [(64, 36), (33, 31), (97, 50)])
@pytest.mark.parametrize("flags", list(FLAGS))
def test_tiled_classification_matches_the_plain_form(cuda, size, flags):
    w, h = size
    data = inputs(w, h, seed=w + h)
    used_p, hist_p, seg_p = run(cuda, T.TAA_FORM_PLAIN, *data, FLAGS[flags])
    used_t, hist_t, seg_t = run(cuda, T.TAA_FORM_TILED, *data, FLAGS[flags])
    assert used_p == T.TAA_FORM_PLAIN and used_t == T.TAA_FORM_TILED
    np.testing.assert_array_equal(seg_t, seg_p)
    np.testing.assert_array_equal(hist_t, hist_p)
    if flags in ("edges", "all_tests_count"):
        classes = np.bincount((seg_p & 3).ravel(), minlength=3)
        assert classes[2] > 0 and classes[0] > 0  # the inputs exercise both outcomes
    used_h, hist_h, seg_h = run(cuda, T.TAA_FORM_FP16, *data, FLAGS[flags])
    assert used_h == T.TAA_FORM_FP16
    np.testing.assert_array_equal(seg_h, seg_p)
    assert psnr(hist_h[..., :3], hist_p[..., :3]) >= 50.0


def test_a_fused_sharpener_keeps_the_classification_in_the_plain_form(cuda):
    """The tiled form's single resolve-and-sharpen launch has no classifier;
    a sharpener run as a pass of its own after the resolve (the default)
    leaves the classification in the tiled form."""
    p = WL.base_parameters(mRayTraceAugment=1, mRayTraceAugmentFlags=0x3F)
    for flags, form in ((T.TAA_FLAG_FUSED_SHARPEN, T.TAA_FORM_PLAIN), (0, T.TAA_FORM_TILED)):
        ctx = T.Taa(32, 16, sharpener=T.TAA_SHARPEN_CAS, flags=flags)
        ctx.set_uniforms(T.make_uniforms(p))
        assert ctx.selected_form() == form
        ctx.close()
