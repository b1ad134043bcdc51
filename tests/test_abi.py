"""The C ABI: exported symbols, struct layouts and the host-only entry points (no GPU)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import taa_abi as T

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(taa_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(built):
    lib = T.load()
    names = declared_functions()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(T.EXPORTS) == names


def test_binding_constants_match_the_header():
    """Every TAA_FORM_*, TAA_FLAG_*, TAA_SHARPEN_*, TAA_HISTORY_* and
    TAA_MOTION_* value the ctypes binding names equals the header's."""
    text = (ROOT / "include" / "taa_gb300.h").read_text()
    defs = {m.group(1): int(m.group(2), 0)
            for m in re.finditer(r"^#define\s+(TAA_(?:FORM|FLAG|SHARPEN|HISTORY|MOTION|DEVICE|WINDOW)_\w+)\s+(0x[0-9a-fA-F]+|\d+)u?\b",
                                 text, flags=re.M)}
    assert "TAA_FLAG_FUSED_SHARPEN" in defs and "TAA_FORM_FP16" in defs and "TAA_WINDOW_WAIT_POLLS" in defs
    for name, value in defs.items():
        if hasattr(T, name):
            assert getattr(T, name) == value, name
    flags = [v for k, v in defs.items() if k.startswith("TAA_FLAG_")]
    assert len(set(flags)) == len(flags) and all(f & (f - 1) == 0 for f in flags)


def test_struct_layout_matches_reference_block():
    # std140 offsets of the reference blocks (source/taa.hpp:30-129)
    assert C.sizeof(T.Parameters) == 176
    assert T.Parameters.mDebugMask.offset == 144
    assert T.Parameters.mRayTraceHistoryCount.offset == 140
    assert C.sizeof(T.Uniforms) == 544
    assert T.Uniforms.param.offset == 128
    assert T.Uniforms.mJitterNdc.offset == 480
    assert T.Uniforms.splitScreen.offset == 512
    assert T.Uniforms.mCamFarPlane.offset == 536


def test_header_compiles_as_c_and_cxx(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "taa_gb300.h"\n#include "taa_synth.h"\nint main(void){return sizeof(taa_uniforms_t)==544?0:1;}\n')
    for cc, std in (("gcc", "-std=c11"), ("g++", "-std=c++17")):
        exe = tmp_path / ("a_" + cc.replace("+", "p"))
        lang = ["-x", "c++"] if cc == "g++" else []
        subprocess.run([cc, std, *lang, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
        assert subprocess.run([str(exe)]).returncode == 0


def test_default_parameters_are_reference_defaults(built):
    p = T.default_parameters()
    # source/taa.hpp:31-76
    assert p.mAlpha == pytest.approx(0.05)
    assert p.mColorClampingOrClipping == 1
    assert p.mMinAlpha == np.float32(1.0) - np.float32(0.97)  # float arithmetic, as 1.0f - 0.97f
    assert p.mMaxAlpha == np.float32(1.0) - np.float32(0.88)
    assert p.mUseVelocityVectors == 1 and p.mInterpolationMode == 0
    assert p.mNoiseFactor == np.float32(1.0 / 510.0)
    assert p.mRayTraceAugmentFlags == (0xFFFFFFFF & ~(0x80 | 0x100))
    assert list(p.mDebugMask) == [1.0, 1.0, 1.0, 0.0]
    assert p.mRayTraceHistoryCount == -1


def test_jitter_matches_oracle(built):
    import oracle as O
    lib = T.load()
    for dist in range(5):
        for frame in range(20):
            out = (C.c_float * 2)()
            n = C.c_int32()
            assert lib.taa_get_jitter_offset(dist, frame, 1280, 720, None, out, C.byref(n)) == 0
            ref, rn = O.jitter_offset(dist, frame, 1280, 720)
            assert (out[0], out[1]) == ref and n.value == rn
    # debug knobs: slow motion, fixed index, rotation, scale (taa.hpp:219-232)
    opts = T.JitterOpts(3, 2, 30.0, 1.5)
    out = (C.c_float * 2)()
    assert lib.taa_get_jitter_offset(2, 11, 640, 360, C.byref(opts), out, None) == 0
    assert (out[0], out[1]) == O.jitter_offset(2, 11, 640, 360, 3, 2, 30.0, 1.5)[0]


def test_halton_2_3_first_eight(built):
    import oracle as O
    # helpers::halton(i, 2), (i, 3) for i = 1..8 (helper_functions.hpp:9-26)
    assert [O.halton(i, 2) for i in range(1, 9)] == [0.5, 0.25, 0.75, 0.125, 0.625, 0.375, 0.875, 0.0625]
    h3 = [O.halton(i, 3) for i in range(1, 9)]
    np.testing.assert_allclose(h3, [1 / 3, 2 / 3, 1 / 9, 4 / 9, 7 / 9, 2 / 9, 5 / 9, 8 / 9], rtol=1e-6)


def test_jitter_errors(built):
    lib = T.load()
    out = (C.c_float * 2)()
    assert lib.taa_get_jitter_offset(9, 0, 64, 64, None, out, None) == T.TAA_E_INVAL
    assert b"sample distribution" in lib.taa_last_error()
    assert lib.taa_get_jitter_offset(2, 0, 0, 64, None, out, None) == T.TAA_E_INVAL


def test_jittered_projection_is_translate_times_p(built):
    lib = T.load()
    rng = np.random.default_rng(0)
    P = rng.standard_normal(16).astype(np.float32)
    j = np.array([0.01, -0.02], np.float32)
    out = (C.c_float * 16)()
    assert lib.taa_jittered_projection(P.ctypes.data_as(C.POINTER(C.c_float)),
                                       j.ctypes.data_as(C.POINTER(C.c_float)), out) == 0
    Tm = np.eye(4, dtype=np.float64)
    Tm[0, 3], Tm[1, 3] = j
    ref = (Tm @ P.reshape(4, 4).T.astype(np.float64)).T.reshape(16)
    np.testing.assert_allclose(np.array(out[:]), ref, rtol=1e-6, atol=1e-7)


def test_compose_matrices_fp64(built):
    rng = np.random.default_rng(1)
    pc, vc, pp, vp = (rng.standard_normal(16) + 4 * np.eye(4).reshape(16) for _ in range(4))
    inv, hist = T.compose_matrices(pc, vc, pp, vp)
    M = lambda a: np.asarray(a, np.float64).reshape(4, 4).T  # column-major
    ref_inv = np.linalg.inv(M(pc) @ M(vc)).T.reshape(16).astype(np.float32)
    ref_hist = (M(pp) @ M(vp)).T.reshape(16).astype(np.float32)
    np.testing.assert_allclose(inv, ref_inv, rtol=2e-6, atol=1e-7)
    np.testing.assert_array_equal(hist, ref_hist)
    with pytest.raises(T.TaaError):
        T.compose_matrices(np.zeros(16), vc, pp, vp)


def test_cas_setup_matches_oracle_and_peak(built):
    import oracle as O
    lib = T.load()
    for s in (0.0, 0.25, 0.5, 1.0, 1.7, -1.0):
        c0 = (C.c_uint32 * 4)()
        c1 = (C.c_uint32 * 4)()
        assert lib.taa_cas_setup(s, 1920, 1080, 1920, 1080, c0, c1) == 0
        r0, r1 = O.cas_setup(s, 1920, 1080, 1920, 1080)
        assert list(c0) == r0 and list(c1) == r1
    c0, c1 = O.cas_setup(0.5, 2560, 1440, 2560, 1440)
    peak = np.frombuffer(np.uint32(c1[0]).tobytes(), np.float32)[0]
    assert peak == np.float32(-1.0 / 6.5)  # -1/lerp(8, 5, 0.5)


def test_create_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = T.load()
    d = T.Desc(C.sizeof(T.Desc), 64, 64, 64, 64, 0, 1, 0, 0, 0.5, 0)
    h = C.c_void_p()
    assert lib.taa_create(C.byref(d), C.byref(h)) == T.TAA_E_CUDA
    assert not h.value


def test_create_rejects_bad_descriptions(built):
    lib = T.load()
    h = C.c_void_p()
    bad = [
        T.Desc(C.sizeof(T.Desc), 0, 64, 64, 64, 0, 1, 0, 0, 0.5, 0),
        T.Desc(C.sizeof(T.Desc), 64, 64, 64, 64, 2, 1, 0, 0, 0.5, 0),
        T.Desc(C.sizeof(T.Desc), 64, 64, 64, 64, 0, 2, 0, 0, 0.5, 0),
        T.Desc(C.sizeof(T.Desc), 64, 64, 64, 64, 0, 1, 9, 0, 0.5, 0),
        T.Desc(C.sizeof(T.Desc), 64, 64, 64, 64, 0, 1, 0, 3, 0.5, 0),
        T.Desc(C.sizeof(T.Desc), 64, 64, 64, 64, 0, 1, 0, 0, float("nan"), 0),
        T.Desc(12, 64, 64, 64, 64, 0, 1, 0, 0, 0.5, 0),
        T.Desc(C.sizeof(T.Desc), 64, 64, 64, 64, 0, 1, T.TAA_FORM_TILED, 0, 0.5, T.TAA_FLAG_FP16_GUARD),
        T.Desc(C.sizeof(T.Desc), 64, 64, 64, 64, 0, 1, T.TAA_FORM_AUTO, 0, 0.5, T.TAA_FLAG_FP16_GUARD),
        T.Desc(C.sizeof(T.Desc), 64, 64, 64, 64, 0, 1, 0, 0, 0.5, 0x10),
    ]
    for d in bad:
        assert lib.taa_create(C.byref(d), C.byref(h)) == T.TAA_E_INVAL
        assert lib.taa_last_error()


def test_null_arguments(built):
    lib = T.load()
    assert lib.taa_resolve(None, None, None) == T.TAA_E_INVAL
    assert lib.taa_set_uniforms(None, None) == T.TAA_E_INVAL
    assert lib.taa_destroy(None) == 0
