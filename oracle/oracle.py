"""numpy face of the oracle (test infrastructure: the checker, never the product).

Loads ``oracle/_build/liboracle.so`` (built by ``oracle/build_oracle.py``) and wraps
its entry points for numpy arrays.  Images are (H, W, C) arrays; FP16 inputs
are widened to float32 exactly before they are handed over.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from importlib import util
            spec = util.spec_from_file_location("build_oracle", HERE / "build_oracle.py")
            mod = util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_oracle()
        lib = C.CDLL(str(LIB_PATH))
        P = C.POINTER
        fp, dp, up = P(C.c_float), P(C.c_double), P(C.c_uint32)
        lib.oracle_resolve.restype = C.c_int
        lib.oracle_resolve.argtypes = [C.c_int, C.c_void_p] + [C.c_int] * 4 + [fp] * 5 + [up] * 3 + [fp] + \
                                      [dp] * 3 + [up, C.c_int]
        lib.oracle_cas.argtypes = [C.c_int, fp, C.c_int, C.c_int, C.c_uint32, dp, C.c_int]
        lib.oracle_sharpen.argtypes = [C.c_int, fp, C.c_int, C.c_int, C.c_float, dp, C.c_int]
        lib.oracle_fxaa.argtypes = [C.c_int, fp, up, C.c_int, C.c_int] + [C.c_float] * 5 + [dp, C.c_int]
        lib.oracle_cas_setup.argtypes = [C.c_float] * 5 + [up, up]
        ip = C.POINTER(C.c_int)
        lib.oracle_post_process.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, ip, ip, fp, fp] + [C.c_int] * 5 + \
            [dp, C.c_int]
        lib.oracle_cas_setup.restype = None
        lib.oracle_halton.argtypes = [C.c_int, C.c_int]
        lib.oracle_halton.restype = C.c_float
        lib.oracle_jitter_offset.argtypes = [C.c_int, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                             C.c_float, fp, P(C.c_int)]
        lib.oracle_jitter_offset.restype = None
        lib.oracle_quantize_half.argtypes = [fp, fp, C.c_size_t]
        lib.oracle_quantize_half.restype = None
        lib.oracle_check_div_const.argtypes = [C.c_float, C.c_uint32, C.c_uint32, C.c_int]
        lib.oracle_check_div_const.restype = C.c_longlong
        lib.oracle_synth_frame.argtypes = [C.c_void_p, fp, C.c_int, dp, dp, dp, dp, C.c_int]
        _lib = lib
    return _lib


def _fp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _up(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint32))


def _f32(a, ch=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float32)
    if ch is not None and a.ndim == 3 and a.shape[2] < ch:
        pad = np.zeros(a.shape[:2] + (ch - a.shape[2],), np.float32)
        a = np.ascontiguousarray(np.concatenate([a, pad], axis=2))
    return a


def _u32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.uint32)


def nthreads_default() -> int:
    return max(1, os.cpu_count() or 1)


def resolve(uniforms, color, depth, velocity, history=None, history_depth=None, out_size=None, precision=32,
            material=None, prev_material=None, prev_segmask=None, uvnrm=None, want_debug=False, nthreads=None):
    """Run the oracle resolve.  Returns dict(history, screen, debug, segmask)
    of float64 arrays holding the FP32 (precision=32) or FP64 values before
    any FP16 store."""
    lib = load()
    in_h, in_w = color.shape[:2]
    out_w, out_h = out_size if out_size else (in_w, in_h)
    col = _f32(color, 4)
    dep = _f32(depth).reshape(in_h, in_w)
    vel = _f32(velocity, 4)
    his = _f32(history, 4)
    hdp = _f32(history_depth)
    mat, pmat, pseg = _u32(material), _u32(prev_material), _u32(prev_segmask)
    nrm = _f32(uvnrm, 4)
    out_hist = np.zeros((out_h, out_w, 4))
    out_scr = np.zeros((out_h, out_w, 4))
    out_dbg = np.zeros((out_h, out_w, 4)) if want_debug else None
    out_seg = np.zeros((out_h, out_w), np.uint32)
    rc = lib.oracle_resolve(precision, C.addressof(uniforms), in_w, in_h, out_w, out_h, _fp(col), _fp(dep), _fp(his),
                            _fp(hdp), _fp(vel), _up(mat), _up(pmat), _up(pseg), _fp(nrm), _dp(out_hist),
                            _dp(out_scr), _dp(out_dbg), _up(out_seg), nthreads or nthreads_default())
    if rc != 0:
        raise ValueError("oracle_resolve rejected its arguments")
    return dict(history=out_hist, screen=out_scr, debug=out_dbg, segmask=out_seg)


def cas(img, peak_bits, precision=32, nthreads=None):
    lib = load()
    a = _f32(img, 4)
    h, w = a.shape[:2]
    out = np.zeros((h, w, 4))
    lib.oracle_cas(precision, _fp(a), w, h, peak_bits, _dp(out), nthreads or nthreads_default())
    return out


def sharpen(img, factor, precision=32, nthreads=None):
    lib = load()
    a = _f32(img, 4)
    h, w = a.shape[:2]
    out = np.zeros((h, w, 4))
    lib.oracle_sharpen(precision, _fp(a), w, h, factor, _dp(out), nthreads or nthreads_default())
    return out


FXAA_DEFAULTS = (0.75, 0.116, 0.0833)  # fxaaQualitySubpix, EdgeThreshold, EdgeThresholdMin (taa.hpp:95-97)


def fxaa(img, segmask=None, subpix=0.75, edge_threshold=0.116, edge_threshold_min=0.0833, precision=32,
         nthreads=None):
    """FXAA prepare + FXAA 3.11 quality preset 12 on the pixels with (segmask & 3) == 1
    (every pixel when segmask is None); returns rgb and the FP16-stored luma."""
    lib = load()
    a = _f32(img, 4)
    h, w = a.shape[:2]
    seg = None if segmask is None else _u32(segmask)
    if seg is not None and seg.shape != (h, w):
        raise ValueError("segmask must be (H, W)")
    rcp = np.float32(1.0) / np.array([w, h], np.float32)
    out = np.zeros((h, w, 4))
    rc = lib.oracle_fxaa(precision, _fp(a), _up(seg), w, h, float(rcp[0]), float(rcp[1]), subpix, edge_threshold,
                         edge_threshold_min, _dp(out), nthreads or nthreads_default())
    if rc != 0:
        raise ValueError("oracle_fxaa rejected its arguments")
    return out


POST_DEFAULTS = dict(zoom_src=(950, 530, 20, 20), zoom_dst=(1710, 10, 200, 200), mask_l=(1.0, 1.0, 1.0, 0.0),
                     mask_r=(1.0, 1.0, 1.0, 0.0), zoom=False, show_zoom_box=True, split_x=-1, show_l=False,
                     show_r=False)


def post_process(img, debug=None, precision=32, nthreads=None, **params):
    """The post-process pass (shaders/post_process.comp) on an RGBA image and an
    RGBA debug image: split line, zoom box and inset, debug image per side.
    Parameters as POST_DEFAULTS (the push constants of source/taa.hpp:101-111);
    returns the RGBA output unrounded."""
    lib = load()
    pp = dict(POST_DEFAULTS)
    unknown = set(params) - set(pp)
    if unknown:
        raise TypeError(f"unknown post-process parameters {sorted(unknown)}")
    pp.update(params)
    a = _f32(img, 4)
    h, w = a.shape[:2]
    d = None if debug is None else _f32(debug, 4)
    if d is not None and d.shape != a.shape:
        raise ValueError("debug must match the image")
    iv = lambda v: (C.c_int * 4)(*[int(x) for x in v])
    fv = lambda v: np.ascontiguousarray(v, dtype=np.float32)
    ml, mr = fv(pp["mask_l"]), fv(pp["mask_r"])
    out = np.zeros((h, w, 4))
    rc = lib.oracle_post_process(precision, _fp(a), _fp(d), w, h, iv(pp["zoom_src"]), iv(pp["zoom_dst"]), _fp(ml),
                                 _fp(mr), int(bool(pp["zoom"])), int(bool(pp["show_zoom_box"])), int(pp["split_x"]),
                                 int(bool(pp["show_l"])), int(bool(pp["show_r"])), _dp(out),
                                 nthreads or nthreads_default())
    if rc != 0:
        raise ValueError("oracle_post_process rejected its arguments")
    return out


def cas_setup(sharpness, in_w, in_h, out_w, out_h):
    c0 = (C.c_uint32 * 4)()
    c1 = (C.c_uint32 * 4)()
    load().oracle_cas_setup(sharpness, in_w, in_h, out_w, out_h, c0, c1)
    return list(c0), list(c1)


def halton(i, b):
    return load().oracle_halton(i, b)


def jitter_offset(dist, frame, w, h, fixed_index=-1, slow_motion=1, rotate_degrees=0.0, extra_scale=1.0):
    out = (C.c_float * 2)()
    n = C.c_int()
    load().oracle_jitter_offset(dist, frame, w, h, fixed_index, slow_motion, rotate_degrees, extra_scale, out,
                                C.byref(n))
    return (out[0], out[1]), n.value


def quantize_half(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    out = np.empty_like(a)
    load().oracle_quantize_half(_fp(a), _fp(out), a.size)
    return out


def check_div_const(d, lo_bits, hi_bits, nthreads=None):
    return load().oracle_check_div_const(d, lo_bits, hi_bits, nthreads or nthreads_default())


def synth_frame(scene, spheres, frame, truth=False, nthreads=None):
    """FP64 evaluation of the analytic scene; returns dict(color, depth, motion, truth)."""
    lib = load()
    w, h = scene.width, scene.height
    sph = np.ascontiguousarray(spheres, dtype=np.float32)
    col = np.zeros((h, w, 4))
    dep = np.zeros((h, w))
    mot = np.zeros((h, w, 4))
    tru = np.zeros((h, w, 4)) if truth else None
    lib.oracle_synth_frame(C.addressof(scene), _fp(sph), frame, _dp(col), _dp(dep), _dp(mot), _dp(tru),
                           nthreads or nthreads_default())
    return dict(color=col, depth=dep, motion=mot, truth=tru)


# ---------------------------------------------------------------- inputs without the library
# The parameter block, the uniform block and the scene description as the
# oracle's own ctypes types (the layouts of include/taa_params.h and
# include/taa_synth.h), so that a caller that must not load the library - the
# benchmark's reference arm - builds the same inputs from the oracle alone.
_PF = "f i u u u f u u u u u u f f f f u i i i u u f u u u f f u u f f f f f i f4 i f u u".split()
_PN = ("mAlpha mColorClampingOrClipping mDepthCulling mUnjitterNeighbourhood mUnjitterCurrentSample "
       "mUnjitterFactor mPassThrough mUseYCoCg mShrinkChromaAxis mVarianceClipping mShapedNeighbourhood "
       "mLumaWeightingLottes mVarClipGamma mMinAlpha mMaxAlpha mRejectionAlpha mRejectOutside mUseVelocityVectors "
       "mVelocitySampleMode mInterpolationMode mToneMapLumaKaris mAddNoise mNoiseFactor mReduceBlendNearClamp "
       "mDynamicAntiGhosting mVelBasedAlpha mVelBasedAlphaMax mVelBasedAlphaFactor mRayTraceAugment "
       "mRayTraceAugmentFlags mRayTraceAugment_WNrm mRayTraceAugment_WDpt mRayTraceAugment_WMId "
       "mRayTraceAugment_WLum mRayTraceAugment_Thresh mRayTraceHistoryCount mDebugMask mDebugMode mDebugScale "
       "mDebugCenter mDebugToScreenOutput").split()
_T = {"f": C.c_float, "i": C.c_int32, "u": C.c_uint32, "f4": C.c_float * 4}


class Parameters(C.Structure):
    """Parameters of source/taa.hpp:30-77 (176 bytes)."""
    _fields_ = [(n, _T[t]) for n, t in zip(_PN, _PF)]


class Uniforms(C.Structure):
    """uniforms_for_taa of source/taa.hpp:113-129 (544 bytes)."""
    _fields_ = [("mHistoryViewProjMatrix", C.c_float * 16), ("mInverseViewProjMatrix", C.c_float * 16),
                ("param", Parameters * 2), ("mJitterNdc", C.c_float * 4), ("mSinTime", C.c_float * 4),
                ("splitScreen", C.c_uint32), ("splitX", C.c_int32), ("mUpsampling", C.c_uint32),
                ("mBypassHistoryUpdate", C.c_uint32), ("mResetHistory", C.c_uint32), ("mCamNearPlane", C.c_float),
                ("mCamFarPlane", C.c_float), ("pad1", C.c_float)]


class SynthScene(C.Structure):
    """taa_synth_scene_t (include/taa_synth.h)."""
    _fields_ = [("struct_size", C.c_uint32), ("width", C.c_int32), ("height", C.c_int32), ("seed", C.c_uint64),
                ("num_spheres", C.c_int32), ("radius_min", C.c_float), ("radius_max", C.c_float),
                ("sphere_speed_max", C.c_float), ("spin_max", C.c_float), ("cam_v0", C.c_float * 2),
                ("cam_accel", C.c_float * 2), ("checker_period", C.c_float), ("firefly_fraction", C.c_float),
                ("firefly_max", C.c_float), ("jitter_phase", C.c_int32), ("jitter_enabled", C.c_int32)]


assert C.sizeof(Parameters) == 176 and C.sizeof(Uniforms) == 544


def default_parameters() -> Parameters:
    p = Parameters()
    lib = load()
    lib.oracle_default_parameters.argtypes = [C.c_void_p]
    lib.oracle_default_parameters(C.addressof(p))
    return p


def make_uniforms(p0: Parameters, jitter_ndc=(0.0, 0.0), **kw) -> Uniforms:
    """The uniform block of a frame: identity matrices, both parameter sets p0,
    the jitter, near 0.1 and far 1000, and any field given by name."""
    u = Uniforms()
    for m in (u.mHistoryViewProjMatrix, u.mInverseViewProjMatrix):
        for i in range(4):
            m[i * 5] = 1.0
    u.param[0] = p0
    u.param[1] = p0
    u.mJitterNdc[0], u.mJitterNdc[1] = jitter_ndc
    u.mCamNearPlane, u.mCamFarPlane = 0.1, 1000.0
    for k, v in kw.items():
        setattr(u, k, v)
    return u


def synth_scene(width, height, seed, **fields) -> SynthScene:
    s = SynthScene()
    lib = load()
    lib.oracle_synth_default_scene.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_uint64]
    lib.oracle_synth_default_scene(C.addressof(s), width, height, seed)
    for k, v in fields.items():
        if k in ("cam_v0", "cam_accel"):
            getattr(s, k)[0], getattr(s, k)[1] = v
        else:
            setattr(s, k, v)
    return s


def synth_spheres(scene: SynthScene):
    t = np.zeros((max(1, scene.num_spheres), 12), np.float32)
    lib = load()
    lib.oracle_synth_spheres.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    lib.oracle_synth_spheres(C.addressof(scene), _fp(t))
    return t


def synth_jitter(scene: SynthScene, frame: int):
    """The frame's sub-pixel jitter in NDC."""
    ndc = (C.c_float * 2)()
    lib = load()
    lib.oracle_synth_jitter.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float)]
    lib.oracle_synth_jitter(C.addressof(scene), frame, ndc)
    return ndc[0], ndc[1]
