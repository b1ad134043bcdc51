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
  * CasSetup: equal bits.
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
