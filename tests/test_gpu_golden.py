"""The CUDA forms on the golden fixtures of the reference shader (run with -m gpu).

Every fixture case (tests/golden, produced by the reference's taa.comp compiled
as C++) is resolved on the GPU through the C ABI.  The plain form handles
every parameter (segmentation mask, upsampling, debug output, split screen):
it must give the FP32 oracle's bits (except where the shader calls sin/cos,
whose CUDA and libm roundings differ), stay within a frame relative L2 of 1e-5
of the reference shader's own FP32 output, and produce the reference's
segmentation mask.  Cases the tiled form implements are checked the same way.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle as O
import taa_abi as T

pytestmark = pytest.mark.gpu

G = Path(__file__).resolve().parent / "golden"
FIX = np.load(G / "taa_comp_golden.npz")
CASES = [str(c) for c in FIX["cases"]]
TRANSCENDENTAL = ("noise", "segmask_all_tests", "segmask_no_history_count", "segmask_fixed_border", "debug_8")


def rel_bound(key):
    # taa.comp:551-556 hashes with fract(sin(x) * 43758.5453): one ulp of sin
    # moves the noise anywhere within its amplitude (2 * mNoiseFactor = 2/510),
    # so CUDA's and libm's sinf differ by up to that much per pixel
    return 3e-3 if key.endswith(":noise") else 1e-5


def uniforms_of(key):
    u = T.Uniforms()
    C.memmove(C.addressof(u), FIX[f"{key}/uniforms"].tobytes(), C.sizeof(u))
    return u


def gpu(key, form, dev, debug=False):
    scene = key.split(":")[0]
    g = lambda k: FIX[f"{scene}/{k}"]
    hist = g("history")
    oh, ow = hist.shape[:2]
    h, w = g("color").shape[:2]
    ctx = T.Taa(w, h, ow, oh, motion_format=T.TAA_MOTION_RGBA16F, form=form)
    u = uniforms_of(key)
    ctx.set_uniforms(u)
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    b = dict(color=t(g("color"), torch.float16), depth=t(g("depth"), torch.float32),
             velocity=t(g("velocity"), torch.float16), history=t(hist, torch.float32),
             history_depth=t(g("history_depth"), torch.float32),
             material=t(g("material").view(np.int32), torch.int32),
             prev_material=t(g("prev_material").view(np.int32), torch.int32),
             prev_segmask=t(g("prev_segmask").view(np.int32), torch.int32), uvnrm=t(g("uvnrm"), torch.float32),
             history_out=torch.full((oh, ow, 4), float("nan"), device=dev),
             result=torch.full((oh, ow, 4), float("nan"), dtype=torch.float16, device=dev),
             debug=torch.full((oh, ow, 4), float("nan"), dtype=torch.float16, device=dev) if debug else None,
             segmask=torch.zeros((oh, ow), dtype=torch.int32, device=dev))
    used = ctx.selected_form()
    ctx.resolve(**b)
    torch.cuda.synchronize()
    if debug:
        # taa_selected_form answers for calls without a debug binding; with one the
        # tiled FP32 form writes it unless the parameters need the plain form
        # (upsampling with a debug binding runs in the plain form)
        up = ow != w or oh != h
        used = T.TAA_FORM_PLAIN if used == T.TAA_FORM_PLAIN or up else T.TAA_FORM_TILED
    ctx.close()
    seg = b["segmask"].cpu().numpy().view(np.uint32) if b["segmask"] is not None else None
    if debug:
        return used, b["history_out"].cpu().numpy(), seg, b["debug"].cpu().numpy()
    return used, b["history_out"].cpu().numpy(), seg


def oracle32(key):
    scene = key.split(":")[0]
    g = lambda k: FIX[f"{scene}/{k}"]
    hist = g("history")
    return O.resolve(uniforms_of(key), g("color"), g("depth"), g("velocity"), history=hist,
                     history_depth=g("history_depth"), out_size=(hist.shape[1], hist.shape[0]), material=g("material"),
                     prev_material=g("prev_material"), prev_segmask=g("prev_segmask"), uvnrm=g("uvnrm"))


@pytest.mark.parametrize("key", CASES)
def test_plain_form_on_reference_fixtures(cuda, key):
    used, hist, seg = gpu(key, T.TAA_FORM_PLAIN, cuda)
    assert used == T.TAA_FORM_PLAIN
    ref32 = FIX[f"{key}/ref32_history"].astype(np.float64)
    rel = np.linalg.norm(hist - ref32) / max(np.linalg.norm(ref32), 1e-30)
    assert rel <= rel_bound(key), rel
    name = key.split(":")[1]
    if name.startswith("segmask"):
        assert np.mean(seg == FIX[f"{key}/ref64_segmask"]) >= 0.99
    if name not in TRANSCENDENTAL:
        np.testing.assert_array_equal(hist, oracle32(key)["history"].astype(np.float32))


@pytest.mark.parametrize("key", CASES)
def test_tiled_form_on_reference_fixtures(cuda, key):
    used, hist, seg = gpu(key, T.TAA_FORM_TILED, cuda)
    ref32 = FIX[f"{key}/ref32_history"].astype(np.float64)
    rel = np.linalg.norm(hist - ref32) / max(np.linalg.norm(ref32), 1e-30)
    assert rel <= rel_bound(key), (used, rel)
    name = key.split(":")[1]
    if name.startswith("segmask"):
        # the ray-trace-assist classification runs in the tiled form on a staged
        # neighbourhood: the plain form's bits (both call CUDA's sinf/cosf for the
        # normals) and the reference's mask
        assert used == T.TAA_FORM_TILED
        _, phist, pseg = gpu(key, T.TAA_FORM_PLAIN, cuda)
        np.testing.assert_array_equal(hist, phist)
        np.testing.assert_array_equal(seg, pseg)
        assert np.mean(seg == FIX[f"{key}/ref64_segmask"]) >= 0.99
    elif used == T.TAA_FORM_TILED and name in TRANSCENDENTAL:
        # the noise hashes CUDA's sinf like the plain form: the plain form's bits
        _, phist, _ = gpu(key, T.TAA_FORM_PLAIN, cuda)
        np.testing.assert_array_equal(hist, phist)
    elif used == T.TAA_FORM_TILED:
        np.testing.assert_array_equal(hist, oracle32(key)["history"].astype(np.float32))


# parameter modes the tiled forms run since they gained noise, dynamic
# anti-ghosting (the mask in the history alpha) and the 3x3-longest velocity
TILED_NOW = ("noise", "anti_ghosting", "velocity_longest")


@pytest.mark.parametrize("name", TILED_NOW)
def test_tiled_form_runs_the_extra_modes(cuda, name):
    key = f"s:{name}"
    used, hist, _ = gpu(key, T.TAA_FORM_TILED, cuda)
    assert used == T.TAA_FORM_TILED
    _, phist, _ = gpu(key, T.TAA_FORM_PLAIN, cuda)
    np.testing.assert_array_equal(hist, phist)  # alpha included: the dynamic mask
    used16, hist16, _ = gpu(key, T.TAA_FORM_FP16, cuda)
    assert used16 == T.TAA_FORM_FP16
    np.testing.assert_array_equal(hist16[..., 3], phist[..., 3])
    assert np.linalg.norm(hist16[..., :3] - phist[..., :3]) <= 1e-2 * np.linalg.norm(phist[..., :3])



@pytest.mark.parametrize("key", [k for k in CASES if k.split(":")[1].startswith("debug") or
                                 k.split(":")[1] in ("base", "c2_depth_reject", "segmask_all_tests")])
def test_debug_output_of_the_tiled_form(cuda, key):
    """With a debug binding the tiled FP32 form writes the debug image
    (taa.comp:912-942) with the plain form's bits, and the history is unchanged."""
    used, hist, seg, dbg = gpu(key, T.TAA_FORM_TILED, cuda, debug=True)
    assert used == T.TAA_FORM_TILED
    pused, phist, pseg, pdbg = gpu(key, T.TAA_FORM_PLAIN, cuda, debug=True)
    assert pused == T.TAA_FORM_PLAIN
    np.testing.assert_array_equal(dbg, pdbg)
    np.testing.assert_array_equal(hist, phist)
    _, hist_nodebug, _ = gpu(key, T.TAA_FORM_TILED, cuda)
    np.testing.assert_array_equal(hist, hist_nodebug)
