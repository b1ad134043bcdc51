"""The .ini settings of the TAA class (taa_settings_*; source/taa.hpp:1198-1339,
source/IniUtil.cpp) and the C++ mirror's writeSettingsToIni/readSettingsFromIni.
Host code only (no GPU)."""
import ctypes as C
import subprocess

import numpy as np
import pytest

import build as lib_build
import taa_abi as T

PARAM_KEYS = ["mPassThrough", "mColorClampingOrClipping", "mShapedNeighbourhood", "mVarianceClipping",
              "mVarClipGamma", "mUseYCoCg", "mLumaWeightingLottes", "mDepthCulling", "mRejectOutside",
              "mUnjitterNeighbourhood", "mUnjitterCurrentSample", "mUnjitterFactor", "mAlpha", "mMinAlpha",
              "mMaxAlpha", "mRejectionAlpha", "mUseVelocityVectors", "mVelocitySampleMode", "mInterpolationMode",
              "mToneMapLumaKaris", "mAddNoise", "mNoiseFactor", "mReduceBlendNearClamp", "mDynamicAntiGhosting",
              "mDebugMask.x", "mDebugMask.y", "mDebugMask.z", "mDebugMask.w", "mDebugMode", "mDebugScale",
              "mDebugCenter", "mDebugToScreenOutput", "mVelBasedAlpha", "mVelBasedAlphaMax", "mVelBasedAlphaFactor",
              "mRayTraceAugment"]
PRIMARY_KEYS = ["mTaaEnabled", "mSampleDistribution", "mSharpener", "mSharpenFactor", "mSplitScreen", "mSplitX",
                "mFixedJitterIndex", "mJitterExtraScale", "mJitterSlowMotion", "mJitterRotateDegrees",
                "mResetHistoryOnChange", "mDebugSampleOffsets.size"]
POST_KEYS = ["mPostProcessEnabled", "zoom", "showZoomBox"] + [f"zoom{w}LTWH.{c}" for w in ("Src", "Dst")
                                                               for c in "xyzw"]


def sections(text):
    out, cur = {}, None
    for line in text.split("\n"):
        if line.startswith("["):
            cur = line[1:-1]
            out[cur] = []
        else:
            k, v = line.split("=", 1)
            out[cur].append((k, v))
    return out


def test_defaults_are_the_reference_members(built):
    s = T.settings_default()
    # source/taa.hpp:1350-1420 and the post-processing push constants 101-111
    assert (s.mTaaEnabled, s.mSampleDistribution, s.mSharpener, s.mSplitScreen, s.mSplitX) == (1, 1, 0, 0, 0)
    assert s.mSharpenFactor == pytest.approx(0.5)
    assert (s.mFixedJitterIndex, s.mJitterSlowMotion, s.mResetHistoryOnChange) == (-1, 1, 1)
    assert (s.mJitterExtraScale, s.mJitterRotateDegrees) == (1.0, 0.0)
    assert s.mDebugSampleOffsetsCount == 1 and list(s.mDebugSampleOffsets[0]) == [0.0, 0.0]
    assert (s.mPostProcessEnabled, s.zoom, s.showZoomBox) == (1, 0, 1)
    assert list(s.zoomSrcLTWH) == [950, 530, 20, 20] and list(s.zoomDstLTWH) == [1710, 10, 200, 200]
    assert bytes(s.param[0]) == bytes(T.default_parameters()) == bytes(s.param[1])


def test_written_text_has_the_reference_layout(built):
    s = T.settings_default()
    s.mDebugSampleOffsetsCount = 2
    s.mDebugSampleOffsets[1][0], s.mDebugSampleOffsets[1][1] = 0.25, -0.5
    text = T.settings_to_ini(s)
    assert not text.endswith("\n") and "\r" not in text and " " not in text
    sec = sections(text)
    # the INI library lower-cases section and key names; sections in the order written
    assert list(sec) == ["taa_param_0", "taa_param_1", "taa_primary", "taa_postprocess"]
    for i in range(2):
        assert [k for k, _ in sec[f"taa_param_{i}"]] == [k.lower() for k in PARAM_KEYS]
    prim = [k.lower() for k in PRIMARY_KEYS] + [f"mdebugsampleoffsets_{i}.{c}" for i in range(2) for c in "xy"]
    assert [k for k, _ in sec["taa_primary"]] == prim
    assert [k for k, _ in sec["taa_postprocess"]] == [k.lower() for k in POST_KEYS]
    d = dict(sec["taa_param_0"])
    # std::to_string: floats with six decimals, VkBool32 and int as integers
    assert d["malpha"] == "0.050000" and d["mcolorclampingorclipping"] == "1" and d["mpassthrough"] == "0"
    assert d["mdebugmask.x"] == "1.000000" and d["mdebugmask.w"] == "0.000000"
    p = dict(sec["taa_primary"])
    assert p["mtaaenabled"] == "1" and p["mfixedjitterindex"] == "-1" and p["msharpenfactor"] == "0.500000"
    assert p["mdebugsampleoffsets.size"] == "2" and p["mdebugsampleoffsets_1.y"] == "-0.500000"
    assert dict(sec["taa_postprocess"])["zoomdstltwh.x"] == "1710"


def randomized(seed):
    rng = np.random.default_rng(seed)
    s = T.settings_default()
    for i in range(2):
        p = s.param[i]
        for name, kind in T._PARAM_FIELDS:
            if kind == "f":
                setattr(p, name, float(np.float32(rng.uniform(-3, 3))))
            elif kind == "i":
                setattr(p, name, int(rng.integers(-2, 5)))
            elif kind == "u":
                setattr(p, name, int(rng.integers(0, 2)))
            else:
                for c in range(4):
                    getattr(p, name)[c] = float(np.float32(rng.uniform(0, 1)))
    s.mTaaEnabled, s.mSampleDistribution, s.mSharpener = 0, 5, 2
    s.mSharpenFactor, s.mSplitScreen, s.mSplitX = 0.25, 1, 321
    s.mFixedJitterIndex, s.mJitterExtraScale, s.mJitterSlowMotion, s.mJitterRotateDegrees = 3, 1.5, 4, 12.5
    s.mResetHistoryOnChange = 0
    s.mDebugSampleOffsetsCount = 5
    for k in range(5):
        s.mDebugSampleOffsets[k][0], s.mDebugSampleOffsets[k][1] = rng.uniform(-0.5, 0.5, 2)
    s.mPostProcessEnabled, s.zoom, s.showZoomBox = 0, 1, 0
    for k in range(4):
        s.zoomSrcLTWH[k], s.zoomDstLTWH[k] = int(rng.integers(0, 2000)), int(rng.integers(-5, 2000))
    return s


# members the settings file does not hold (source/taa.hpp:1205-1238 writes 33 of the 40)
NOT_STORED = {"mShrinkChromaAxis", "mRayTraceAugmentFlags", "mRayTraceAugment_WNrm", "mRayTraceAugment_WDpt",
              "mRayTraceAugment_WMId", "mRayTraceAugment_WLum", "mRayTraceAugment_Thresh", "mRayTraceHistoryCount"}


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_round_trip(built, seed):
    s = randomized(seed)
    back = T.settings_from_ini(T.settings_to_ini(s))
    for i in range(2):
        for name, kind in T._PARAM_FIELDS:
            a, b = getattr(s.param[i], name), getattr(back.param[i], name)
            if name in NOT_STORED:
                assert b == getattr(T.default_parameters(), name)  # untouched: the defaults read over
            elif kind == "f4":
                np.testing.assert_allclose(list(b), list(a), atol=5e-7)
            elif kind == "f":
                assert abs(a - b) <= 5e-7 + 1e-6 * abs(a), name  # six decimals
            else:
                assert a == b, name
    for name in ("mTaaEnabled", "mSampleDistribution", "mSharpener", "mSplitScreen", "mSplitX", "mFixedJitterIndex",
                 "mJitterSlowMotion", "mResetHistoryOnChange", "mDebugSampleOffsetsCount", "mPostProcessEnabled",
                 "zoom", "showZoomBox"):
        assert getattr(back, name) == getattr(s, name), name
    assert list(back.zoomSrcLTWH) == list(s.zoomSrcLTWH) and list(back.zoomDstLTWH) == list(s.zoomDstLTWH)
    np.testing.assert_allclose(np.array(back.mDebugSampleOffsets)[:5], np.array(s.mDebugSampleOffsets)[:5],
                               atol=5e-7)
    # what was read back writes the same text again
    assert T.settings_to_ini(back) == T.settings_to_ini(T.settings_from_ini(T.settings_to_ini(back)))


def test_reads_a_settings_file_as_the_reference_does(built):
    # a whole settings file: other sections of the application, mixed-case names,
    # blanks around '=', comments, CRLF line ends, a key before any section,
    # a repeated key (the last wins), "true" for a C++ bool, a partial vector
    text = "\r\n".join([
        "stray=1",
        "[Lights]",
        "mMaxPointLightCount=16",
        "; a comment line",
        "[TAA_Param_0]",
        "  mAlpha = 0.25  ",
        "MCOLORCLAMPINGORCLIPPING=2",
        "mUseYCoCg=1",
        "mUseYCoCg=0",
        "mDebugMask.y=0.5",
        "mInterpolationMode=2trailing",
        "mVarClipGamma=",
        "[taa_param_1]",
        "mPassThrough=7",
        "[TAA_Primary] ; note",
        "mTaaEnabled=true",
        "mSplitScreen=2",
        "mSharpener=2",
        "mDebugSampleOffsets.size=3",
        "mDebugSampleOffsets_0.x=0.125",
        "mDebugSampleOffsets_2.y=-0.25",
        "[TAA_Postprocess]",
        "zoomSrcLTWH.z=64",
        "mPostProcessEnabled=0",
    ])
    base = T.settings_default()
    base.param[0].mVarClipGamma = 1.25
    s = T.settings_from_ini(text, base)
    p0, p1 = s.param[0], s.param[1]
    assert p0.mAlpha == pytest.approx(0.25) and p0.mColorClampingOrClipping == 2
    assert p0.mUseYCoCg == 0
    assert list(p0.mDebugMask) == [1.0, 0.5, 1.0, 0.0]
    assert p0.mInterpolationMode == 2           # std::stol reads the leading number
    assert p0.mVarClipGamma == 1.25             # empty value: member unchanged
    assert p1.mPassThrough == 7                 # VkBool32 through std::stoul
    assert s.mTaaEnabled == 1 and s.mSplitScreen == 0  # bool: "1" or "true" only
    assert s.mSharpener == 2
    assert s.mDebugSampleOffsetsCount == 3
    assert list(s.mDebugSampleOffsets[0]) == [0.125, 0.0] and list(s.mDebugSampleOffsets[2]) == [0.0, -0.25]
    assert list(s.zoomSrcLTWH) == [950, 530, 64, 20] and s.mPostProcessEnabled == 0
    # everything else kept its value
    d = T.default_parameters()
    assert p0.mMaxAlpha == d.mMaxAlpha and p1.mAlpha == d.mAlpha and s.mSampleDistribution == 1


def test_sample_offset_list_follows_the_stored_size(built):
    s = T.settings_default()
    s.mDebugSampleOffsetsCount = 4
    for k in range(4):
        s.mDebugSampleOffsets[k][0] = k + 1.0
    # the reference resizes to max(1, stored size), 0 when the key is absent
    assert T.settings_from_ini("[TAA_Primary]\nmSharpener=1", s).mDebugSampleOffsetsCount == 1
    assert T.settings_from_ini("[TAA_Primary]\nmDebugSampleOffsets.size=-3", s).mDebugSampleOffsetsCount == 1
    r = T.settings_from_ini("[TAA_Primary]\nmDebugSampleOffsets.size=6", s)
    assert r.mDebugSampleOffsetsCount == 6
    assert [r.mDebugSampleOffsets[k][0] for k in range(6)] == [1.0, 2.0, 3.0, 4.0, 0.0, 0.0]
    with pytest.raises(T.TaaError):
        T.settings_from_ini("[TAA_Primary]\nmDebugSampleOffsets.size=65", s)


@pytest.mark.parametrize("line", ["[TAA_Param_0]\nmAlpha=abc", "[TAA_Param_1]\nmDepthCulling=x1",
                                  "[TAA_Primary]\nmSplitX=--4", "[TAA_Param_0]\nmAlpha=1e60",
                                  "[TAA_Postprocess]\nzoomDstLTWH.w=99999999999999999999"])
def test_unreadable_numbers_fail_and_change_nothing(built, line):
    # std::stof/stoi/stoul throw on these; the settings stay as they were
    s = randomized(4)
    before = bytes(s)
    raw = line.encode()
    rc = T.load().taa_settings_read_ini(C.byref(s), raw, len(raw))
    assert rc == T.TAA_E_INVAL and bytes(s) == before
    assert "not a number" in T.load().taa_last_error().decode()


def test_write_buffer_and_argument_errors(built):
    lib = T.load()
    s = T.settings_default()
    n = C.c_size_t()
    assert lib.taa_settings_write_ini(C.byref(s), None, 0, C.byref(n)) == 0 and n.value > 1000
    small = C.create_string_buffer(n.value)  # no room for the NUL
    assert lib.taa_settings_write_ini(C.byref(s), small, n.value, C.byref(n)) == T.TAA_E_INVAL
    assert small.value == b""
    s.mDebugSampleOffsetsCount = 0
    assert lib.taa_settings_write_ini(C.byref(s), None, 0, C.byref(n)) == T.TAA_E_INVAL
    assert lib.taa_settings_read_ini(None, b"", 0) == T.TAA_E_INVAL
    assert lib.taa_settings_default(None) == T.TAA_E_INVAL


def test_custom_sample_offsets_jitter(built):
    # sample distribution 5: the debug offsets in pixels times the NDC pixel size
    offs = [(0.25, -0.25), (-0.375, 0.125), (0.0, 0.5)]
    w, h = 1920, 1080
    sx, sy = np.float32(2.0) / np.float32(w), np.float32(2.0) / np.float32(h)
    for f in range(7):
        x, y = offs[f % 3]
        got = T.jitter_offset_custom(offs, f, w, h)
        assert got == (float(np.float32(x) * sx), float(np.float32(y) * sy))
    # the debugging knobs apply as for the tables
    opts = T.JitterOpts(1, 1, 0.0, 2.0)
    assert T.jitter_offset_custom(offs, 5, w, h, opts) == (float(np.float32(offs[1][0]) * sx * 2),
                                                          float(np.float32(offs[1][1]) * sy * 2))
    with pytest.raises(T.TaaError):
        T.jitter_offset_custom([], 0, w, h)


def test_mirror_reads_and_writes_settings(built, tmp_path):
    lib = lib_build.build_library()
    exe = tmp_path / "settings_roundtrip"
    src = lib_build.PKG / "examples" / "settings_roundtrip.cpp"
    subprocess.run([lib_build.nvcc(), "-std=c++17", "-O2", "-x", "cu", str(src), "-o", str(exe), "-L",
                    str(lib.parent), "-ltaa_gb300", f"-Xlinker=-rpath,{lib.parent}"], check=True, capture_output=True)
    # defaults: the mirror writes what the library writes for the default settings
    r = subprocess.run([str(exe)], capture_output=True, text=True, check=True)
    assert r.stdout == T.settings_to_ini(T.settings_default())
    # a file read in and written out again
    s = randomized(7)
    f = tmp_path / "in.ini"
    f.write_text(T.settings_to_ini(s))
    r = subprocess.run([str(exe), str(f)], capture_output=True, text=True, check=True)
    assert r.stdout == T.settings_to_ini(T.settings_from_ini(f.read_text()))
    bad = tmp_path / "bad.ini"
    bad.write_text("[TAA_Param_0]\nmAlpha=oops\n")
    r = subprocess.run([str(exe), str(bad)], capture_output=True, text=True)
    assert r.returncode == 2 and "not a number" in r.stderr
