"""The batched resolve (taa_batch_*) against per-view taa_resolve (run with -m gpu).

A batch resolves views of different sizes in one persistent launch; every
view must get exactly the bits its own taa_resolve gives in the form of the
batch's tile body - the tiled FP32 form for the exact tile shapes, the fast
form for the four-pixel strips - whatever tile shape and job order the batch
runs with, when the launch is replayed from a CUDA graph, and after
taa_batch_autotune has picked its configuration.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import taa_abi as T
import workloads as WL
from helpers import cpu_frames, to_dev

pytestmark = pytest.mark.gpu

SIZES = [(70, 41), (17, 9), (256, 96), (33, 31), (128, 72), (64, 36)]
SHAPES = [(32, 8), (16, 16), (32, 16), (16, 8), (8, 8)]


def make_views(dev, sizes, params=None, motion_channels=2):
    views = []
    for i, (w, h) in enumerate(sizes):
        wl = WL.small(w, h, frames=2, seed=20 + i, params=params or {})
        fr = cpu_frames(wl, range(2), motion_channels=motion_channels)
        u = T.make_uniforms(wl.parameters(), jitter_ndc=fr[1]["jitter"])
        b = dict(color=to_dev(fr[1]["color"], torch.float16, dev), depth=to_dev(fr[1]["depth"], torch.float32, dev),
                 velocity=to_dev(fr[1]["motion"], torch.float16, dev),
                 history=to_dev(fr[0]["color"].astype(np.float32), torch.float32, dev),
                 history_depth=to_dev(fr[0]["depth"], torch.float32, dev),
                 history_out=torch.full((h, w, 4), float("nan"), device=dev),
                 result=torch.full((h, w, 4), float("nan"), dtype=torch.float16, device=dev))
        views.append(dict(size=(w, h), u=u, b=b))
    return views


def reference(views, motion_format, form=T.TAA_FORM_TILED):
    out = []
    for v in views:
        w, h = v["size"]
        ctx = T.Taa(w, h, motion_format=motion_format, form=form)
        ctx.set_uniforms(v["u"])
        b = dict(v["b"])
        b["history_out"] = torch.full_like(b["history_out"], float("nan"))
        b["result"] = torch.full_like(b["result"], float("nan"))
        ctx.resolve(**b)
        torch.cuda.synchronize()
        out.append((b["history_out"].cpu().numpy(), b["result"].float().cpu().numpy()))
        ctx.close()
    return out


def reset_outputs(views):
    for v in views:
        v["b"]["history_out"].fill_(float("nan"))
        v["b"]["result"].fill_(float("nan"))


def check_equal(views, ref):
    torch.cuda.synchronize()
    for v, (h_ref, r_ref) in zip(views, ref):
        np.testing.assert_array_equal(v["b"]["history_out"].cpu().numpy(), h_ref, err_msg=str(v["size"]))
        np.testing.assert_array_equal(v["b"]["result"].float().cpu().numpy(), r_ref, err_msg=str(v["size"]))


def make_batch(views, motion_format):
    batch = T.Batch([v["size"] for v in views], motion_format=motion_format)
    for i, v in enumerate(views):
        batch.set_uniforms(i, v["u"])
    batch.prepare(0, [v["b"] for v in views])
    return batch


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("schedule", [T.TAA_SCHEDULE_VIEW_ORDER, T.TAA_SCHEDULE_LARGEST_FIRST,
                                      T.TAA_SCHEDULE_INTERLEAVED])
def test_batch_equals_per_view_resolve(cuda, shape, schedule):
    views = make_views(cuda, SIZES)
    ref = reference(views, T.TAA_MOTION_RG16F)
    batch = make_batch(views, T.TAA_MOTION_RG16F)
    for grid_mode in (0, T.TAA_BATCH_CTA_PER_TILE, 1):
        batch.set_tuning(shape[0], shape[1], schedule, grid_mode)
        reset_outputs(views)
        batch.launch(0)
        check_equal(views, ref)
    batch.close()


@pytest.mark.parametrize("schedule", [T.TAA_SCHEDULE_VIEW_ORDER, T.TAA_SCHEDULE_LARGEST_FIRST,
                                      T.TAA_SCHEDULE_INTERLEAVED])
@pytest.mark.parametrize("params,mc", [({}, 2), (dict(mInterpolationMode=0, mDepthCulling=1, mRejectOutside=1), 2),
                                       ({}, 4)], ids=["cr", "bilinear_c2", "rgba16f_motion"])
def test_fast_strips_equal_per_view_fast_resolve(cuda, schedule, params, mc):
    """The four-pixel strips (TAA_FORM_FAST's body) over many views: each view
    gets the bits of its own taa_resolve in TAA_FORM_FAST, persistent or one
    CTA per tile."""
    mf = T.TAA_MOTION_RGBA16F if mc == 4 else T.TAA_MOTION_RG16F
    views = make_views(cuda, SIZES, params=params, motion_channels=mc)
    ref = reference(views, mf, form=T.TAA_FORM_FAST)
    batch = make_batch(views, mf)
    for grid_mode in (0, T.TAA_BATCH_CTA_PER_TILE, 1):
        batch.set_tuning(32, 16, schedule, grid_mode, form=T.TAA_FORM_FAST)
        reset_outputs(views)
        batch.launch(0)
        check_equal(views, ref)
    batch.close()


def test_fast_strips_need_a_fast_batch_and_the_benchmark_mode(cuda):
    lib = T.load()
    views = make_views(cuda, SIZES[:2])
    tb = T.Batch([v["size"] for v in views], form=T.TAA_FORM_TILED)
    bad = T.BatchTuning(32, 16, 0, 0, 0.0, T.TAA_FORM_FAST)
    assert lib.taa_batch_set_tuning(tb.handle, C.byref(bad)) == T.TAA_E_UNSUPPORTED
    tb.close()
    views = make_views(cuda, SIZES[:2], params=dict(mColorClampingOrClipping=1))  # not the benchmark mode
    batch = make_batch(views, T.TAA_MOTION_RG16F)
    batch.set_tuning(32, 16, 0, 0, form=T.TAA_FORM_FAST)
    assert lib.taa_batch_launch(batch.handle, None, 0) == T.TAA_E_UNSUPPORTED
    best = batch.autotune(0, reps=1)
    assert best.form in (0, T.TAA_FORM_TILED)  # the strips are not candidates
    batch.close()


@pytest.mark.parametrize("mode", ["bilinear_clamp", "rgba16f_motion"])
def test_batch_other_modes(cuda, mode):
    params = dict(mInterpolationMode=0, mColorClampingOrClipping=1) if mode == "bilinear_clamp" else {}
    mc, mf = (4, T.TAA_MOTION_RGBA16F) if mode == "rgba16f_motion" else (2, T.TAA_MOTION_RG16F)
    views = make_views(cuda, SIZES[:4], params=params, motion_channels=mc)
    ref = reference(views, mf)
    batch = make_batch(views, mf)
    for shape in ((16, 16), (8, 8)):
        batch.set_tuning(shape[0], shape[1], T.TAA_SCHEDULE_INTERLEAVED)
        reset_outputs(views)
        batch.launch(0)
        check_equal(views, ref)
    batch.close()


def test_autotune_then_graph_replay(cuda):
    views = make_views(cuda, SIZES)
    batch = make_batch(views, T.TAA_MOTION_RG16F)
    best = batch.autotune(0, reps=2)
    assert best.ms > 0
    assert ((best.tile_w, best.tile_h) in SHAPES and best.form in (0, T.TAA_FORM_TILED)) or \
        ((best.tile_w, best.tile_h) == (32, 16) and best.form == T.TAA_FORM_FAST)
    t = batch.tuning()
    assert (t.tile_w, t.tile_h, t.schedule, t.form) == (best.tile_w, best.tile_h, best.schedule, best.form)
    ref = reference(views, T.TAA_MOTION_RG16F, form=T.TAA_FORM_FAST if best.form == T.TAA_FORM_FAST else T.TAA_FORM_TILED)
    reset_outputs(views)
    batch.launch(0)
    check_equal(views, ref)
    # the launch captured into a CUDA graph, replayed
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        batch.launch(0, stream=torch.cuda.current_stream().cuda_stream)
    reset_outputs(views)
    torch.cuda.synchronize()
    g.replay()
    check_equal(views, ref)
    reset_outputs(views)
    g.replay()
    check_equal(views, ref)
    assert T.device_status(clear=True) == 0
    batch.close()


def test_batch_rejects_what_it_does_not_run(cuda):
    lib = T.load()
    d = (T.Desc * 2)()
    d[0] = T.Desc(C.sizeof(T.Desc), 64, 32, 64, 32, T.TAA_HISTORY_RGBA32F, T.TAA_MOTION_RG16F, 0, 0, 0.5, 0)
    d[1] = T.Desc(C.sizeof(T.Desc), 64, 32, 64, 32, T.TAA_HISTORY_RGBA32F, T.TAA_MOTION_RGBA16F, 0, 0, 0.5, 0)
    h = C.c_void_p()
    assert lib.taa_batch_create(d, 2, C.byref(h)) == T.TAA_E_UNSUPPORTED  # mixed motion formats
    d[1] = T.Desc(C.sizeof(T.Desc), 32, 16, 64, 32, T.TAA_HISTORY_RGBA32F, T.TAA_MOTION_RG16F, 0, 0, 0.5, 0)
    assert lib.taa_batch_create(d, 2, C.byref(h)) == T.TAA_E_UNSUPPORTED  # upsampling
    d[1] = T.Desc(C.sizeof(T.Desc), 64, 32, 64, 32, T.TAA_HISTORY_RGBA16F, T.TAA_MOTION_RG16F, 0, 0, 0.5, 0)
    assert lib.taa_batch_create(d, 2, C.byref(h)) == T.TAA_E_UNSUPPORTED  # RGBA16F history
    batch = T.Batch([(64, 32), (32, 16)])
    assert lib.taa_batch_launch(batch.handle, None, 0) == T.TAA_E_INVAL  # slot never prepared
    bad = T.BatchTuning(24, 8, 0, 0, 0.0)
    assert lib.taa_batch_set_tuning(batch.handle, C.byref(bad)) == T.TAA_E_INVAL
    batch.close()


def test_c4_views_from_a_graph_match_the_oracle(cuda):
    """The C4 configuration: 48 views (log-uniform 320x180 .. 3840x2160, each
    with its own scene, jitter phase and pan), frame 1 of each resolved on the
    history of its frame 0, all in one batch launch captured in a CUDA graph
    and replayed.  The 6 smallest and the 2 largest views get the FP32 oracle's
    bits; every view has the bits of its own taa_resolve."""
    import oracle as O
    wls = WL.c4_views()
    views = []
    for wl in wls:
        sc = wl.scene()
        w, h = wl.width, wl.height
        fr = []
        for f in range(2):
            col = torch.empty(h, w, 4, dtype=torch.float16, device=cuda)
            dep = torch.empty(h, w, device=cuda)
            mot = torch.empty(h, w, 2, dtype=torch.float16, device=cuda)
            T.synth_render(sc, f, color=col, depth=dep, motion=mot)
            fr.append((col, dep, mot))
        u = T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(sc, 1)[1])
        b = dict(color=fr[1][0], depth=fr[1][1], velocity=fr[1][2], history=fr[0][0].float().contiguous(),
                 history_depth=fr[0][1], history_out=torch.full((h, w, 4), float("nan"), device=cuda),
                 result=torch.full((h, w, 4), float("nan"), dtype=torch.float16, device=cuda))
        views.append(dict(size=(w, h), u=u, b=b))
    assert len(views) == 48
    batch = make_batch(views, T.TAA_MOTION_RG16F)
    # the exact tiles: the oracle's bits
    batch.set_tuning(16, 16, T.TAA_SCHEDULE_LARGEST_FIRST)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        batch.launch(0, stream=torch.cuda.current_stream().cuda_stream)
    reset_outputs(views)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    assert T.device_status(clear=True) == 0
    order = sorted(range(48), key=lambda i: views[i]["size"][0] * views[i]["size"][1])
    for i in order[:6] + order[-2:]:
        v = views[i]
        b = v["b"]
        ref = O.resolve(v["u"], b["color"].float().cpu().numpy(), b["depth"].cpu().numpy(),
                        b["velocity"].float().cpu().numpy(), history=b["history"].cpu().numpy(),
                        history_depth=b["history_depth"].cpu().numpy())
        np.testing.assert_array_equal(b["history_out"].cpu().numpy(), ref["history"].astype(np.float32),
                                      err_msg=str(v["size"]))
        np.testing.assert_array_equal(b["result"].float().cpu().numpy(),
                                      ref["screen"].astype(np.float32).astype(np.float16).astype(np.float32),
                                      err_msg=str(v["size"]))
    got = [(v["b"]["history_out"].cpu().numpy(), v["b"]["result"].float().cpu().numpy()) for v in views]
    ref = reference(views, T.TAA_MOTION_RG16F)
    for (h_g, r_g), (h_r, r_r), v in zip(got, ref, views):
        np.testing.assert_array_equal(h_g, h_r, err_msg=str(v["size"]))
        np.testing.assert_array_equal(r_g, r_r, err_msg=str(v["size"]))
    # the autotuned configuration (the fast strips where they win), from a graph:
    # the bits of each view's own taa_resolve in that form, and within 1e-4
    # relative L2 of the FP64 oracle on the checked views
    best = batch.autotune(0, reps=1)
    form = T.TAA_FORM_FAST if best.form == T.TAA_FORM_FAST else T.TAA_FORM_TILED
    g2 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g2, stream=s):
        batch.launch(0, stream=torch.cuda.current_stream().cuda_stream)
    reset_outputs(views)
    torch.cuda.synchronize()
    g2.replay()
    torch.cuda.synchronize()
    assert T.device_status(clear=True) == 0
    got = [(v["b"]["history_out"].cpu().numpy(), v["b"]["result"].float().cpu().numpy()) for v in views]
    ref = reference(views, T.TAA_MOTION_RG16F, form=form)
    for (h_g, r_g), (h_r, r_r), v in zip(got, ref, views):
        np.testing.assert_array_equal(h_g, h_r, err_msg=str(v["size"]))
        np.testing.assert_array_equal(r_g, r_r, err_msg=str(v["size"]))
    report = []
    for i in order[:6] + order[-2:]:
        v = views[i]
        b = v["b"]
        args = (v["u"], b["color"].float().cpu().numpy(), b["depth"].cpu().numpy(), b["velocity"].float().cpu().numpy())
        kw = dict(history=b["history"].cpu().numpy(), history_depth=b["history_depth"].cpu().numpy())
        r64 = O.resolve(*args, precision=64, **kw)["history"][..., :3]
        r32 = O.resolve(*args, **kw)["history"][..., :3]
        n64 = np.linalg.norm(r64)
        e_got, e_exact = np.linalg.norm(got[i][0][..., :3] - r64) / n64, np.linalg.norm(r32 - r64) / n64
        report.append((v["size"], e_got, e_exact))
        # as close to FP64 as the exact FP32 form (whose bits the FP32 oracle has), or within 1e-4
        assert e_got <= max(1e-4, 3.0 * e_exact), (v["size"], e_got, e_exact)
    print("C4 views (size, relL2 of the autotuned form vs FP64, of the exact FP32 form vs FP64):", report)
    batch.close()
