"""taa_resolve_static_scratch against taa_resolve through the C ABI (run with -m gpu).

The entry point runs a resolve and then the sharpen pass with the screen
image between them in the library's fixed device buffer instead of an image
the context allocates.  Its outputs must equal those of taa_resolve on a
context created with the same sharpener (the same kernels; the tests'
tolerance for a form against itself is equality), on two calls in a row with
the history chained.  This file is collected last, so it also runs after every
other GPU test has used the device.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import taa_abi as T
import workloads as WL
from helpers import cpu_frames, to_dev

pytestmark = pytest.mark.gpu

W, H = 70, 41


def frame_io(**bindings):
    io = T.FrameIO()
    for name, t in bindings.items():
        if t is not None:
            p, pitch = T.tensor_ptr_pitch(t)
            setattr(io, name, p)
            setattr(io, name + "_pitch", pitch)
    return io


def run_pair(ctx_ref, ctx_static, u, frames, sharpener, factor, dev):
    """Two calls in a row on each entry point, each chaining its own history."""
    lib = T.load()
    hist_ref = hist_static = None
    for cur, prev in ((frames[1], frames[0]), (frames[2], frames[1])):
        ins = dict(color=to_dev(cur["color"], torch.float16, dev), depth=to_dev(cur["depth"], torch.float32, dev),
                   velocity=to_dev(cur["motion"], torch.float16, dev),
                   history_depth=to_dev(prev["depth"], torch.float32, dev))
        outs = {}
        for key, ctx, hist in (("ref", ctx_ref, hist_ref), ("static", ctx_static, hist_static)):
            h_out = torch.full((H, W, 4), float("nan"), device=dev)
            sharp = torch.full((H, W, 4), float("nan"), dtype=torch.float16, device=dev)
            io = frame_io(history=hist, history_out=h_out, sharpened=sharp, **ins)
            if key == "ref":
                T.check(lib.taa_resolve(ctx.handle, None, C.byref(io)))
            else:
                T.check(lib.taa_resolve_static_scratch(ctx.handle, None, C.byref(io), sharpener, factor))
            outs[key] = (h_out, sharp)
        torch.cuda.synchronize()
        for a, b in zip(outs["ref"], outs["static"]):
            np.testing.assert_array_equal(b.float().cpu().numpy(), a.float().cpu().numpy())
        assert torch.all(outs["static"][1][..., 3] == 1.0)
        hist_ref, hist_static = outs["ref"][0], outs["static"][0]


CASES = {
    "plain_cas": (T.TAA_FORM_PLAIN, T.TAA_SHARPEN_CAS, {}),
    "plain_simple": (T.TAA_FORM_PLAIN, T.TAA_SHARPEN_SIMPLE, {}),
    # split screen is a plain-form feature, so AUTO runs the plain form here
    "auto_split_screen_cas": (T.TAA_FORM_AUTO, T.TAA_SHARPEN_CAS, dict(splitScreen=1, splitX=30)),
    # the tiled FP32 and FP16 forms: the resolve, then the sharpen pass
    "tiled_cas": (T.TAA_FORM_TILED, T.TAA_SHARPEN_CAS, {}),
    "fp16_simple": (T.TAA_FORM_FP16, T.TAA_SHARPEN_SIMPLE, {}),
}
FORM_RUN = {"tiled_cas": T.TAA_FORM_TILED, "fp16_simple": T.TAA_FORM_FP16}


@pytest.mark.parametrize("case", list(CASES))
def test_static_scratch_matches_taa_resolve(cuda, case):
    form, sharpener, extra = CASES[case]
    wl = WL.small(W, H, frames=3)
    fr = cpu_frames(wl, range(3))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"], **extra)
    ctx_ref = T.Taa(W, H, form=form, sharpener=sharpener, sharpen_factor=0.4)
    ctx_static = T.Taa(W, H, form=form)  # no sharpener: taa_create allocates no device memory
    for c in (ctx_ref, ctx_static):
        c.set_uniforms(u)
    assert ctx_static.selected_form() == FORM_RUN.get(case, T.TAA_FORM_PLAIN)
    run_pair(ctx_ref, ctx_static, u, fr, sharpener, 0.4, cuda)
    ctx_ref.close()
    ctx_static.close()


def test_static_scratch_rejects_outputs_beyond_its_buffer(cuda):
    lib = T.load()
    ctx = T.Taa(3841, 2160, form=T.TAA_FORM_PLAIN)
    ctx.set_uniforms(T.make_uniforms(T.default_parameters()))
    io = T.FrameIO()  # refused before any binding is read
    rc = lib.taa_resolve_static_scratch(ctx.handle, None, C.byref(io), T.TAA_SHARPEN_CAS, 0.5)
    assert rc == T.TAA_E_INVAL
    assert b"exceeds the static buffer" in lib.taa_last_error()
    ctx.close()
