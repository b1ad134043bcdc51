"""The largest image sizes the C ABI accepts (32768 texels on a side), run with
-m gpu: 32768 x 40 and 40 x 32768 frames through the plain, tiled and FP16
forms against the FP32 oracle (the FP32 forms to its bits), the FXAA pass at
the full width (its work list packs x and y into 16 bits each), and the
rejection of 32769.  Rows 32768 texels wide exercise the TMA window at its
largest coordinates; columns 40 texels wide and 32768 tall, the copy by
cp.async (the window does not fit) and the last tile row."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle as O
import taa_abi as T
import workloads as WL
from helpers import cpu_frames, half_ulp, psnr, to_dev

pytestmark = pytest.mark.gpu

SIZES = [(32768, 40), (40, 32768)]


@pytest.fixture(scope="module", params=SIZES, ids=lambda s: f"{s[0]}x{s[1]}")
def extreme(request):
    w, h = request.param
    wl = WL.small(w, h, frames=2, seed=23, params=dict(mDepthCulling=1, mRejectOutside=1))
    fr = cpu_frames(wl, range(2), motion_channels=2)
    hist = fr[0]["color"].astype(np.float32)
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    ref = O.resolve(u, fr[1]["color"].astype(np.float32), fr[1]["depth"], fr[1]["motion"].astype(np.float32),
                    history=hist, history_depth=fr[0]["depth"])
    return w, h, fr, hist, u, ref


def resolve(dev, form, w, h, fr, hist, u):
    ctx = T.Taa(w, h, form=form)
    ctx.set_uniforms(u)
    b = dict(color=to_dev(fr[1]["color"], torch.float16, dev), depth=to_dev(fr[1]["depth"], torch.float32, dev),
             velocity=to_dev(fr[1]["motion"], torch.float16, dev), history=to_dev(hist, torch.float32, dev),
             history_depth=to_dev(fr[0]["depth"], torch.float32, dev),
             history_out=torch.full((h, w, 4), float("nan"), device=dev),
             result=torch.full((h, w, 4), float("nan"), dtype=torch.float16, device=dev))
    ctx.resolve(**b)
    torch.cuda.synchronize()
    assert ctx.selected_form() == (form if form != T.TAA_FORM_AUTO else T.TAA_FORM_TILED)
    ctx.close()
    return b["history_out"].cpu().numpy(), b["result"].float().cpu().numpy()


@pytest.mark.parametrize("form", [T.TAA_FORM_PLAIN, T.TAA_FORM_TILED])
def test_fp32_forms_give_the_oracle_bits(cuda, extreme, form):
    w, h, fr, hist, u, ref = extreme
    got, res = resolve(cuda, form, w, h, fr, hist, u)
    np.testing.assert_array_equal(got, ref["history"].astype(np.float32))
    scr = ref["screen"][..., :3]
    q = scr.astype(np.float32).astype(np.float16).astype(np.float64)
    assert np.all(np.abs(res[..., :3] - q) <= half_ulp(scr) + 1e-12)
    assert T.device_status(clear=True) == 0


def test_fast_form_within_its_contract(cuda, extreme):
    w, h, fr, hist, u, ref = extreme
    got, _ = resolve(cuda, T.TAA_FORM_FAST, w, h, fr, hist, u)
    r = ref["history"][..., :3]
    assert np.linalg.norm(got[..., :3] - r) <= 1e-5 * np.linalg.norm(r)
    assert T.device_status(clear=True) == 0


def test_fp16_form_within_its_contract(cuda, extreme):
    w, h, fr, hist, u, ref = extreme
    got, _ = resolve(cuda, T.TAA_FORM_FP16, w, h, fr, hist, u)
    assert np.all(np.isfinite(got[..., :3]))
    assert psnr(got[..., :3], ref["history"][..., :3]) >= 50.0


def test_fxaa_at_the_full_width(cuda, extreme):
    w, h, fr, _, _, _ = extreme
    img = fr[1]["color"].astype(np.float32)
    seg = np.random.default_rng(5).integers(0, 4, (h, w)).astype(np.uint32)
    src = to_dev(img, torch.float16, cuda)
    out = torch.empty_like(src)
    m = torch.from_numpy(seg.view(np.int32)).to(cuda)
    ctx = T.Taa(w, h, form=T.TAA_FORM_PLAIN, flags=T.TAA_FLAG_FXAA)
    T.fxaa(src, out, m, ctx=ctx)
    torch.cuda.synchronize()
    ctx.close()
    ref = O.fxaa(img, seg, precision=32).astype(np.float32).astype(np.float16).astype(np.float32)
    np.testing.assert_array_equal(out.float().cpu().numpy(), ref)


def test_one_past_the_largest_size_is_rejected(cuda):
    lib = T.load()
    h = C.c_void_p()
    for w_, h_ in ((32769, 8), (8, 32769)):
        d = T.Desc(C.sizeof(T.Desc), w_, h_, w_, h_, 0, 1, 0, 0, 0.5, 0)
        assert lib.taa_create(C.byref(d), C.byref(h)) == T.TAA_E_INVAL
    a = torch.zeros(1, 16, 4, dtype=torch.float16, device=cuda)
    assert lib.taa_fxaa(None, None, a.data_ptr(), 32769 * 8, None, 0, a.data_ptr() + 8, 32769 * 8, 32769, 1,
                        None) == T.TAA_E_INVAL
