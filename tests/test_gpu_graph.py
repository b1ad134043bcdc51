"""A single-view frame captured in a CUDA graph, run with -m gpu: the resolve
(tiled FP32, FP16 and plain forms), the FXAA pass with the context's work list
(a programmatic dependent launch) and the post-process pass are enqueued on a
capturing stream - none of the calls synchronises the host or allocates - and
the replayed graph writes the same bits as the eager calls."""
import numpy as np
import pytest
import torch

import taa_abi as T
import workloads as WL
from helpers import cpu_frames, to_dev

pytestmark = pytest.mark.gpu


def frame_inputs(dev, w, h):
    wl = WL.small(w, h, frames=2, seed=41, params=dict(mDepthCulling=1, mRejectOutside=1, mRayTraceAugment=1,
                                                        mRayTraceAugmentFlags=0x3F))
    fr = cpu_frames(wl, range(2), motion_channels=2)
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    b = dict(color=to_dev(fr[1]["color"], torch.float16, dev), depth=to_dev(fr[1]["depth"], torch.float32, dev),
             velocity=to_dev(fr[1]["motion"], torch.float16, dev),
             history=to_dev(fr[0]["color"].astype(np.float32), torch.float32, dev),
             history_depth=to_dev(fr[0]["depth"], torch.float32, dev))
    return u, b


def outputs(dev, w, h):
    return dict(history_out=torch.full((h, w, 4), float("nan"), device=dev),
                result=torch.full((h, w, 4), float("nan"), dtype=torch.float16, device=dev),
                segmask=torch.full((h, w), -1, dtype=torch.int32, device=dev),
                fxaa=torch.full((h, w, 4), float("nan"), dtype=torch.float16, device=dev),
                post=torch.full((h, w, 4), float("nan"), dtype=torch.float16, device=dev))


def enqueue(ctx, b, o, pp, stream):
    ctx.resolve(stream=stream, history_out=o["history_out"], result=o["result"], segmask=o["segmask"], **b)
    T.fxaa(o["result"], o["fxaa"], o["segmask"], stream=stream, ctx=ctx)
    T.post_process(o["fxaa"], o["post"], pp, stream=stream)


@pytest.mark.parametrize("form", [T.TAA_FORM_TILED, T.TAA_FORM_FP16, T.TAA_FORM_PLAIN])
def test_graph_replay_equals_eager(cuda, form):
    w, h = 160, 96
    u, b = frame_inputs(cuda, w, h)
    ctx = T.Taa(w, h, form=form, flags=T.TAA_FLAG_FXAA)
    ctx.set_uniforms(u)
    assert ctx.selected_form() == form
    pp = T.post_process_default_params(w, h)
    pp.zoom, pp.split_x = 1, w // 3
    eager, replay = outputs(cuda, w, h), outputs(cuda, w, h)
    enqueue(ctx, b, eager, pp, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            enqueue(ctx, b, replay, pp, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for _ in range(3):  # replays are idempotent: the FXAA work list resets itself
        g.replay()
    torch.cuda.synchronize()
    for k in eager:
        np.testing.assert_array_equal(replay[k].cpu().numpy(), eager[k].cpu().numpy(), err_msg=k)
    marked = int(((eager["segmask"].cpu().numpy() & 3) == 1).sum())
    assert marked > 0  # the FXAA pass had pixels to work on
    assert T.device_status(clear=True) == 0
    ctx.close()


@pytest.mark.parametrize("form", [T.TAA_FORM_TILED, T.TAA_FORM_FP16])
def test_graph_replay_with_a_sharpener(cuda, form):
    """A resolve with CAS (the resolve, then the sharpen pass launched as its
    programmatic dependent, the screen image in the context's buffer) captured
    in a CUDA graph replays to the eager bits."""
    w, h = 160, 96
    u, b = frame_inputs(cuda, w, h)
    ctx = T.Taa(w, h, form=form, sharpener=T.TAA_SHARPEN_CAS, sharpen_factor=0.5)
    ctx.set_uniforms(u)
    assert ctx.selected_form() == form

    def outs():
        return dict(history_out=torch.full((h, w, 4), float("nan"), device=cuda),
                    sharpened=torch.full((h, w, 4), float("nan"), dtype=torch.float16, device=cuda))

    eager, replay = outs(), outs()
    ctx.resolve(stream=torch.cuda.current_stream().cuda_stream, **eager, **b)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            ctx.resolve(stream=torch.cuda.current_stream().cuda_stream, **replay, **b)
    torch.cuda.synchronize()
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    for k in eager:
        np.testing.assert_array_equal(replay[k].cpu().numpy(), eager[k].cpu().numpy(), err_msg=k)
    assert not torch.isnan(eager["sharpened"].float()).any()
    ctx.close()
