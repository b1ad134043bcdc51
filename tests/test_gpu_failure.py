"""The bounded waits' give-up path, made to run without a fault (run with -m gpu).

Every wait of a resolve kernel on an mbarrier (the TMA copy of a tile's
history window) is bounded; a wait that gives up sets
TAA_DEVICE_WINDOW_TIMEOUT in the device status word, waits once more (always
with the full bound, so the copy has landed before the tile's threads leave)
and leaves the tile's pixels unwritten.  The test hook
taa_debug_set_window_wait(0) makes every first wait give up at once.  Then:

* the status word reports the timeout bit, and clearing it reads 0 after;
* some pixels are left as they were (NaN here): the tiles whose window came
  by TMA; every pixel that was written has the bits of a normal run (tiles
  whose window crosses the image border are copied without the barrier);
* with the default limit back, the same launch writes every pixel with the
  normal bits and leaves the status word at 0;
* a persistent batch CTA whose wait gave up stops after that tile.
"""
import numpy as np
import pytest
import torch

import taa_abi as T
import workloads as WL
from helpers import cpu_frames, to_dev

pytestmark = pytest.mark.gpu

W, H = 160, 96  # 5 x 6 tiles of 32 x 16: the inner ones copy their window by TMA


def inputs(dev, w=W, h=H, seed=3, params=None):
    wl = WL.small(w, h, frames=2, seed=seed, params=params or {})
    fr = cpu_frames(wl, range(2))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    b = dict(color=to_dev(fr[1]["color"], torch.float16, dev), depth=to_dev(fr[1]["depth"], torch.float32, dev),
             velocity=to_dev(fr[1]["motion"], torch.float16, dev),
             history=to_dev(fr[0]["color"].astype(np.float32), torch.float32, dev),
             history_depth=to_dev(fr[0]["depth"], torch.float32, dev))
    return u, b


def outputs(dev, w=W, h=H):
    return dict(history_out=torch.full((h, w, 4), float("nan"), device=dev),
                result=torch.full((h, w, 4), float("nan"), dtype=torch.float16, device=dev))


def run(ctx, b, dev, w=W, h=H):
    o = outputs(dev, w, h)
    ctx.resolve(**b, **o)
    torch.cuda.synchronize()
    return o["history_out"].cpu().numpy(), o["result"].float().cpu().numpy()


def check_gave_up(normal, failed):
    h_n, r_n = normal
    h_f, r_f = failed
    unwritten = np.isnan(h_f[..., 0])
    assert unwritten.any(), "no tile gave up"
    assert (~unwritten).any(), "the border tiles copy their window without the barrier"
    assert np.all(np.isnan(r_f[unwritten]))
    np.testing.assert_array_equal(h_f[~unwritten], h_n[~unwritten])
    np.testing.assert_array_equal(r_f[~unwritten], r_n[~unwritten])


@pytest.fixture
def give_up(cuda):
    T.device_status(clear=True)
    T.set_window_wait(0)
    yield
    T.set_window_wait(None)
    T.device_status(clear=True)


@pytest.mark.parametrize("form", [T.TAA_FORM_TILED, T.TAA_FORM_FP16, T.TAA_FORM_FAST])
def test_window_wait_gives_up_and_leaves_the_tile_unwritten(cuda, form):
    u, b = inputs(cuda)
    ctx = T.Taa(W, H, form=form)
    ctx.set_uniforms(u)
    assert ctx.selected_form() == form
    T.device_status(clear=True)
    normal = run(ctx, b, cuda)
    assert T.device_status(clear=True) == 0
    assert not np.isnan(normal[0]).any()
    T.set_window_wait(0)
    try:
        failed = run(ctx, b, cuda)
        assert T.device_status(clear=False) & T.TAA_DEVICE_WINDOW_TIMEOUT
        assert T.device_status(clear=True) & T.TAA_DEVICE_WINDOW_TIMEOUT  # read and clear
        assert T.device_status(clear=False) == 0
    finally:
        T.set_window_wait(None)
    check_gave_up(normal, failed)
    again = run(ctx, b, cuda)
    assert T.device_status(clear=True) == 0
    np.testing.assert_array_equal(again[0], normal[0])
    np.testing.assert_array_equal(again[1], normal[1])
    ctx.close()


def test_upsampling_window_wait_gives_up(cuda, give_up):
    """The tiled form's upsampling path (1.5x) waits on its window the same way."""
    lo_w, lo_h = W * 2 // 3, H * 2 // 3
    wl = WL.small(lo_w, lo_h, frames=2, seed=4)
    fr = cpu_frames(wl, range(2))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"], mUpsampling=1)
    b = dict(color=to_dev(fr[1]["color"], torch.float16, cuda), depth=to_dev(fr[1]["depth"], torch.float32, cuda),
             velocity=to_dev(fr[1]["motion"], torch.float16, cuda),
             history=torch.rand((H, W, 4), device=cuda), history_depth=to_dev(fr[0]["depth"], torch.float32, cuda))
    ctx = T.Taa(lo_w, lo_h, W, H, form=T.TAA_FORM_TILED)
    ctx.set_uniforms(u)
    assert ctx.selected_form() == T.TAA_FORM_TILED
    T.set_window_wait(None)
    normal = run(ctx, b, cuda)
    T.set_window_wait(0)
    failed = run(ctx, b, cuda)
    assert T.device_status(clear=True) & T.TAA_DEVICE_WINDOW_TIMEOUT
    check_gave_up(normal, failed)
    ctx.close()


@pytest.mark.parametrize("shape", [(32, 16, T.TAA_FORM_TILED), (16, 8, T.TAA_FORM_TILED), (32, 16, T.TAA_FORM_FAST)])
def test_batch_cta_stops_after_a_wait_gave_up(cuda, give_up, shape):
    sizes = [(W, H), (128, 64)]
    views = []
    for i, (w, h) in enumerate(sizes):
        u, b = inputs(cuda, w, h, seed=30 + i)
        views.append(dict(size=(w, h), u=u, b=b))
    batch = T.Batch(sizes)
    for i, v in enumerate(views):
        batch.set_uniforms(i, v["u"])
    outs = [outputs(cuda, *v["size"]) for v in views]
    batch.prepare(0, [dict(v["b"], **o) for v, o in zip(views, outs)])
    # one persistent CTA per SM: a CTA whose first tile gives up leaves its later tiles too
    batch.set_tuning(shape[0], shape[1], T.TAA_SCHEDULE_VIEW_ORDER, 1, form=shape[2])
    T.set_window_wait(None)
    batch.launch(0)
    torch.cuda.synchronize()
    assert T.device_status(clear=True) == 0
    normal = [(o["history_out"].cpu().numpy(), o["result"].float().cpu().numpy()) for o in outs]
    for o in outs:
        for t in o.values():
            t.fill_(float("nan"))
    T.set_window_wait(0)
    batch.launch(0)
    torch.cuda.synchronize()
    assert T.device_status(clear=True) & T.TAA_DEVICE_WINDOW_TIMEOUT
    failed = [(o["history_out"].cpu().numpy(), o["result"].float().cpu().numpy()) for o in outs]
    unwritten = sum(int(np.isnan(f[0][..., 0]).sum()) for f in failed)
    assert unwritten > 0
    for n, f in zip(normal, failed):
        ok = ~np.isnan(f[0][..., 0])
        np.testing.assert_array_equal(f[0][ok], n[0][ok])
        np.testing.assert_array_equal(f[1][ok], n[1][ok])
    batch.close()


def test_fused_sharpen_window_wait_gives_up(cuda):
    """The fast form's fused sharpener (30x14 tiles with their ring) leaves a
    tile whose wait gave up unwritten in all three images."""
    u, b = inputs(cuda)
    ctx = T.Taa(W, H, form=T.TAA_FORM_FAST, sharpener=T.TAA_SHARPEN_CAS, flags=T.TAA_FLAG_FUSED_SHARPEN)
    ctx.set_uniforms(u)
    assert ctx.selected_form() == T.TAA_FORM_FAST

    def go():
        o = outputs(cuda)
        o["sharpened"] = torch.full((H, W, 4), float("nan"), dtype=torch.float16, device=cuda)
        ctx.resolve(**b, **o)
        torch.cuda.synchronize()
        return [o[k].float().cpu().numpy() for k in ("history_out", "result", "sharpened")]

    T.device_status(clear=True)
    normal = go()
    assert T.device_status(clear=True) == 0 and not np.isnan(normal[2]).any()
    T.set_window_wait(0)
    try:
        failed = go()
        assert T.device_status(clear=True) & T.TAA_DEVICE_WINDOW_TIMEOUT
    finally:
        T.set_window_wait(None)
    unwritten = np.isnan(failed[0][..., 0])
    assert unwritten.any() and (~unwritten).any()
    for n, f in zip(normal, failed):
        assert np.all(np.isnan(f[unwritten]))
        np.testing.assert_array_equal(f[~unwritten], n[~unwritten])
    ctx.close()
