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


def run_pair(ctx_ref, ctx_static, u, frames, sharpener, factor, dev, bind_result=False):
    """Two calls in a row on each entry point, each chaining its own history;
    bind_result: both calls also get a result image (the static buffer is then
    not used)."""
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
            res = torch.full((H, W, 4), float("nan"), dtype=torch.float16, device=dev) if bind_result else None
            io = frame_io(history=hist, history_out=h_out, sharpened=sharp, result=res, **ins)
            if key == "ref":
                T.check(lib.taa_resolve(ctx.handle, None, C.byref(io)))
            else:
                T.check(lib.taa_resolve_static_scratch(ctx.handle, None, C.byref(io), sharpener, factor))
            outs[key] = (h_out, sharp) + ((res,) if bind_result else ())
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


# The branches that do not use the buffer, and a context that has a sharpener
# of its own: (form, flags, sharpener the context is created with, sharpener
# the call names, whether a result image is bound).
BRANCHES = {
    # a bound result image carries the screen image to the sharpen pass
    "result_bound": (T.TAA_FORM_TILED, 0, T.TAA_SHARPEN_OFF, T.TAA_SHARPEN_CAS, True),
    # the tiled form's single launch with the sharpener needs no screen image
    "fused_tiled": (T.TAA_FORM_TILED, T.TAA_FLAG_FUSED_SHARPEN, T.TAA_SHARPEN_OFF, T.TAA_SHARPEN_CAS, False),
    # a context created with CAS; the call names the simple sharpener and uses the buffer
    "own_sharpener": (T.TAA_FORM_TILED, 0, T.TAA_SHARPEN_CAS, T.TAA_SHARPEN_SIMPLE, False),
}


@pytest.mark.parametrize("case", list(BRANCHES))
def test_static_scratch_branches_match_taa_resolve(cuda, case):
    form, flags, own, named, bind_result = BRANCHES[case]
    wl = WL.small(W, H, frames=3)
    fr = cpu_frames(wl, range(3))
    u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
    ctx_ref = T.Taa(W, H, form=form, sharpener=named, sharpen_factor=0.4, flags=flags)
    ctx_static = T.Taa(W, H, form=form, sharpener=own, sharpen_factor=0.7, flags=flags)
    for c in (ctx_ref, ctx_static):
        c.set_uniforms(u)
    run_pair(ctx_ref, ctx_static, u, fr, named, 0.4, cuda, bind_result=bind_result)
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
