"""The oracle against golden fixtures produced by the reference's own code (CPU).

tests/golden/make_golden.py compiles the reference's shaders/taa.comp and
shaders/sharpen.comp as C++ (through oracle/ref_shim, with only mechanical
rewrites) and CasSetup from shaders/ffx_cas.h, runs them on seeded inputs for
every parameter mode, and stores inputs and outputs here.  These tests need
no reference tree: they hold the oracle's restatement to
  * FP64: the reference shader evaluated in double, to 1e-9 (relative to
    max(1, |value|)) on history, screen and debug, and exactly on the
    segmentation mask - the algorithmic pin;
  * FP32: the reference shader evaluated in float (no FMA contraction), to a
    frame relative L2 of 1e-5 (the oracle fuses the moment and Catmull-Rom
    sums where the shader's text does not, and evaluates the 9-tap
    Catmull-Rom as its 16-tap form);
  * CasSetup: equal bits;
  * FXAA (shaders/antialias_fxaa_prepare.comp then shaders/antialias_fxaa.comp
    with Fxaa3_11_mod.h, through an RGBA16F image): the FP64 oracle equals the
    shader in double exactly; the FP32 oracle (sampler positions in float, the
    shader's in double) agrees on all but a handful of pixels;
  * the post-process pass (shaders/post_process.comp): the FP32 and FP64
    oracle equal the shader exactly for every push-constant case.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import oracle as O
import taa_abi as T

G = Path(__file__).resolve().parent / "golden"
FIX = np.load(G / "taa_comp_golden.npz")
CASES = [str(c) for c in FIX["cases"]]


def uniforms_of(key):
    u = T.Uniforms()
    C.memmove(C.addressof(u), FIX[f"{key}/uniforms"].tobytes(), C.sizeof(u))
    return u


def run_oracle(key, precision):
    scene = key.split(":")[0]
    g = lambda k: FIX[f"{scene}/{k}"]
    hist = g("history")
    return O.resolve(uniforms_of(key), g("color"), g("depth"), g("velocity"), history=hist,
                     history_depth=g("history_depth"), out_size=(hist.shape[1], hist.shape[0]), precision=precision,
                     material=g("material"), prev_material=g("prev_material"), prev_segmask=g("prev_segmask"),
                     uvnrm=g("uvnrm"), want_debug=True)


def rel_err(a, ref):
    return float(np.max(np.abs(a - ref) / np.maximum(1.0, np.abs(ref))))


def test_fixture_covers_the_parameter_modes():
    assert len(CASES) >= 39
    names = {c.split(":")[1] for c in CASES}
    for must in ("base", "bspline", "clip_slow_shaped", "segmask_all_tests", "upsample", "pass_through",
                 "split_screen", "debug_8", "anti_ghosting", "velocity_longest", "reprojection_only"):
        assert must in names


@pytest.mark.parametrize("key", CASES)
def test_fp64_oracle_matches_the_reference_shader(key):
    r = run_oracle(key, 64)
    assert rel_err(r["history"], FIX[f"{key}/ref64_history"]) <= 1e-9
    assert rel_err(r["screen"], FIX[f"{key}/ref64_screen"]) <= 1e-9
    assert rel_err(r["debug"], FIX[f"{key}/ref64_debug"]) <= 1e-9
    np.testing.assert_array_equal(r["segmask"], FIX[f"{key}/ref64_segmask"])


@pytest.mark.parametrize("key", CASES)
def test_fp32_oracle_tracks_the_reference_shader(key):
    r = run_oracle(key, 32)
    ref = FIX[f"{key}/ref32_history"].astype(np.float64)
    got = r["history"]
    n = np.linalg.norm(ref)
    assert np.linalg.norm(got - ref) / max(n, 1e-30) <= 1e-5
    # the bulk of the pixels agree to FP32 rounding
    close = np.abs(got - ref) <= 1e-5 * np.maximum(1.0, np.abs(ref))
    assert close.mean() >= 0.98


def test_cas_setup_matches_the_reference_header():
    lib = T.load()
    for row in json.loads((G / "cas_setup_golden.json").read_text()):
        c0, c1 = O.cas_setup(row["sharpness"], *row["dims"])
        assert c0 == row["const0"] and c1 == row["const1"], row
        p0 = (C.c_uint32 * 4)()
        p1 = (C.c_uint32 * 4)()
        assert lib.taa_cas_setup(row["sharpness"], *row["dims"], p0, p1) == 0
        assert list(p0) == row["const0"] and list(p1) == row["const1"], row


def test_sharpen_matches_the_reference_shader():
    s = np.load(G / "sharpen_golden.npz")
    for prec in (64, 32):
        got = O.sharpen(s["image"], float(s["factor"]), precision=prec)
        ref = s[f"ref{prec}"]
        if prec == 64:
            assert rel_err(got, ref) <= 1e-12
        else:
            np.testing.assert_array_equal(got.astype(np.float32), ref.astype(np.float32))


CASF = np.load(G / "cas_golden.npz")


@pytest.mark.parametrize("key", list(CASF["cases"]))
def test_cas_filter_matches_the_reference_shader(key):
    """The FP32 restatement of CasFilter (ffx_cas.h:424-537 with ffx_a.h's
    approximations) gives the bits of shaders/sharpen_cas.comp compiled here,
    HDR inputs above 1 included."""
    img, c1, ref = CASF[f"{key}/image"], CASF[f"{key}/const1"], CASF[f"{key}/ref32"]
    w, s = key.split("_s")
    _, setup1 = O.cas_setup(float(s), *([float(v) for v in w.split("x")] * 2))
    assert setup1[0] == int(c1[0])
    got = O.cas(img, int(c1[0]), precision=32)[..., :3].astype(np.float32)
    np.testing.assert_array_equal(got, ref)


FXAA = np.load(G / "fxaa_golden.npz")


@pytest.mark.parametrize("mask", ["random", "all", "none"])
def test_fxaa_oracle_matches_the_reference_shaders(mask):
    img, seg = FXAA["image"], FXAA[f"{mask}/segmask"]
    sub, thr, tmin = FXAA["params"].tolist()
    assert np.array_equal(FXAA["rcp"], np.float32(1.0) / np.array([img.shape[1], img.shape[0]], np.float32))
    r64 = O.fxaa(img, seg, sub, thr, tmin, precision=64)
    np.testing.assert_array_equal(r64, FXAA[f"{mask}/ref64"])
    r32 = O.fxaa(img, seg, sub, thr, tmin, precision=32)
    ref32 = FXAA[f"{mask}/ref32"].astype(np.float64)
    rel = np.abs(r32 - ref32) / np.maximum(1.0, np.abs(ref32))
    per_px = np.max(rel, axis=-1)
    assert np.mean(per_px <= 1e-5) >= 0.99
    assert np.sum(per_px > 1e-3) <= 2  # another branch of the edge search
    assert rel_err(r32, ref32) <= 0.05


def test_fxaa_fixture_exercises_the_edge_paths():
    img = FXAA["image"].astype(np.float64)
    prepared = img.copy()  # the FP64 reading: luma in double, stored as FP16
    prepared[..., 3] = (img[..., 0] * 0.299 + img[..., 1] * 0.587 + img[..., 2] * 0.114).astype(np.float16)
    # unmarked pixels are the prepared texels; marked ones change on edges
    np.testing.assert_array_equal(FXAA["none/ref64"], prepared)
    for mask, lo in (("random", 0.1), ("all", 0.5)):
        changed = np.any(np.abs(FXAA[f"{mask}/ref64"] - prepared) > 1e-3, axis=-1)
        assert changed.mean() >= lo
        marked = (FXAA[f"{mask}/segmask"] & 3) == 1
        assert not np.any(changed & ~marked)


POST = np.load(G / "post_golden.npz")
POST_CASES = sorted({k.split("/")[0] for k in POST.files if "/" in k})


def post_params(name):
    pp = json.loads(str(POST[f"{name}/params"]))
    return {k: tuple(v) if isinstance(v, list) else v for k, v in pp.items()}


@pytest.mark.parametrize("name", POST_CASES)
def test_post_process_oracle_matches_the_reference_shader(name):
    pp = post_params(name)
    for prec in (64, 32):
        got = O.post_process(POST["image"], POST["debug"], precision=prec, **pp)
        np.testing.assert_array_equal(got, POST[f"{name}/ref{prec}"].astype(np.float64))


def test_post_process_fixture_covers_each_branch():
    img, dbg = POST["image"].astype(np.float64), POST["debug"].astype(np.float64)
    assert len(POST_CASES) == 7
    np.testing.assert_array_equal(POST["defaults/ref64"], img)  # no split, zoom or debug: a copy
    r = POST["split_debug_left_alpha/ref64"]
    assert np.all(r[:, 36] == 0)  # the split line
    np.testing.assert_array_equal(r[:, :36, 0], dbg[:, :36, 0] + dbg[:, :36, 3])  # alpha shown in red and blue
    np.testing.assert_array_equal(r[:, :36, 3], 1.0)
    np.testing.assert_array_equal(r[:, 37:], img[:, 37:])
    z = POST["zoom_box/ref64"]
    assert np.all(z[7, 9:18] == (1, 0, 0, 0))  # the red box one texel outside (10, 8, 7, 5)
    assert np.all(z[20, 40:65] == (1, 1, 1, 0))  # the inset's white border
    inner = z[21:37, 41:64]
    assert len({tuple(v) for v in inner.reshape(-1, 4)}) <= 35  # magnified: the 7 x 5 source texels
