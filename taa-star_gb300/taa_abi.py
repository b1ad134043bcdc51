"""ctypes binding of libtaa_gb300 (include/taa_gb300.h, include/taa_synth.h).

This is the Python face of the C ABI, used by the tests and the benchmark.
It mirrors the structs byte for byte and adds a thin ``Taa`` context wrapper
that accepts torch CUDA tensors for the per-frame bindings.  It never falls
back to anything: if the shared library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libtaa_gb300.so"

TAA_OK = 0
TAA_E_INVAL = -1
TAA_E_ALIGN = -2
TAA_E_CUDA = -3
TAA_E_TIMEOUT = -4
TAA_E_UNSUPPORTED = -5
TAA_E_NOMEM = -6

TAA_HISTORY_RGBA32F = 0
TAA_HISTORY_RGBA16F = 1
TAA_MOTION_RGBA16F = 0
TAA_MOTION_RG16F = 1
TAA_FORM_AUTO, TAA_FORM_PLAIN, TAA_FORM_TILED, TAA_FORM_FP16, TAA_FORM_LEARNED, TAA_FORM_FAST = 0, 1, 2, 3, 4, 5
TAA_FLAG_LEARNED_TCGEN05 = 0x1
TAA_FLAG_FXAA = 0x2
TAA_FLAG_FP16_GUARD = 0x4
TAA_FLAG_FUSED_SHARPEN = 0x8
TAA_DEVICE_WINDOW_TIMEOUT = 0x1
TAA_WINDOW_WAIT_POLLS = 4096
TAA_SHARPEN_OFF, TAA_SHARPEN_SIMPLE, TAA_SHARPEN_CAS = 0, 1, 2

RTFLAG = dict(OUT=0x1, DIS=0x2, NRM=0x4, DPT=0x8, MID=0x10, LUM=0x20, CNT=0x40, ALL=0x80, FXD=0x100, FXA=0x200)

_PARAM_FIELDS = [
    ("mAlpha", "f"), ("mColorClampingOrClipping", "i"), ("mDepthCulling", "u"), ("mUnjitterNeighbourhood", "u"),
    ("mUnjitterCurrentSample", "u"), ("mUnjitterFactor", "f"), ("mPassThrough", "u"), ("mUseYCoCg", "u"),
    ("mShrinkChromaAxis", "u"), ("mVarianceClipping", "u"), ("mShapedNeighbourhood", "u"),
    ("mLumaWeightingLottes", "u"), ("mVarClipGamma", "f"), ("mMinAlpha", "f"), ("mMaxAlpha", "f"),
    ("mRejectionAlpha", "f"), ("mRejectOutside", "u"), ("mUseVelocityVectors", "i"), ("mVelocitySampleMode", "i"),
    ("mInterpolationMode", "i"), ("mToneMapLumaKaris", "u"), ("mAddNoise", "u"), ("mNoiseFactor", "f"),
    ("mReduceBlendNearClamp", "u"), ("mDynamicAntiGhosting", "u"), ("mVelBasedAlpha", "u"),
    ("mVelBasedAlphaMax", "f"), ("mVelBasedAlphaFactor", "f"), ("mRayTraceAugment", "u"),
    ("mRayTraceAugmentFlags", "u"), ("mRayTraceAugment_WNrm", "f"), ("mRayTraceAugment_WDpt", "f"),
    ("mRayTraceAugment_WMId", "f"), ("mRayTraceAugment_WLum", "f"), ("mRayTraceAugment_Thresh", "f"),
    ("mRayTraceHistoryCount", "i"), ("mDebugMask", "f4"), ("mDebugMode", "i"), ("mDebugScale", "f"),
    ("mDebugCenter", "u"), ("mDebugToScreenOutput", "u"),
]
_CT = {"f": C.c_float, "i": C.c_int32, "u": C.c_uint32, "f4": C.c_float * 4}
PARAM_NAMES = [n for n, _ in _PARAM_FIELDS]


class Parameters(C.Structure):
    """taa<CF>::Parameters (source/taa.hpp:30-77), 176 bytes."""
    _fields_ = [(n, _CT[t]) for n, t in _PARAM_FIELDS]


class Uniforms(C.Structure):
    """taa<CF>::uniforms_for_taa (source/taa.hpp:113-129), 544 bytes."""
    _fields_ = [
        ("mHistoryViewProjMatrix", C.c_float * 16), ("mInverseViewProjMatrix", C.c_float * 16),
        ("param", Parameters * 2), ("mJitterNdc", C.c_float * 4), ("mSinTime", C.c_float * 4),
        ("splitScreen", C.c_uint32), ("splitX", C.c_int32), ("mUpsampling", C.c_uint32),
        ("mBypassHistoryUpdate", C.c_uint32), ("mResetHistory", C.c_uint32), ("mCamNearPlane", C.c_float),
        ("mCamFarPlane", C.c_float), ("pad1", C.c_float),
    ]


class Desc(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("in_width", C.c_int32), ("in_height", C.c_int32), ("out_width", C.c_int32),
        ("out_height", C.c_int32), ("history_format", C.c_uint32), ("motion_format", C.c_uint32),
        ("form", C.c_uint32), ("sharpener", C.c_uint32), ("sharpen_factor", C.c_float), ("flags", C.c_uint32),
    ]


_IO_NAMES = ["color", "depth", "history", "history_depth", "result", "debug", "velocity", "history_out", "segmask",
             "material", "prev_material", "prev_segmask", "uvnrm", "sharpened"]


class FrameIO(C.Structure):
    _fields_ = [f for n in _IO_NAMES for f in ((n, C.c_void_p), (n + "_pitch", C.c_size_t))]


class JitterOpts(C.Structure):
    _fields_ = [("fixed_index", C.c_int32), ("slow_motion", C.c_int32), ("rotate_degrees", C.c_float),
                ("extra_scale", C.c_float)]


class BatchTuning(C.Structure):
    _fields_ = [("tile_w", C.c_int32), ("tile_h", C.c_int32), ("schedule", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("ms", C.c_float), ("form", C.c_int32)]


class MlpWeights(C.Structure):
    _fields_ = [("w1", C.c_float * 1024), ("b1", C.c_float * 32), ("w2", C.c_float * 1024), ("b2", C.c_float * 32),
                ("w3", C.c_float * 64), ("b3", C.c_float * 2)]


class MlpRecord(C.Structure):
    _fields_ = [("features", C.c_uint16 * 32), ("mean", C.c_float * 3), ("sigma", C.c_float * 3),
                ("history", C.c_float * 3), ("current", C.c_float * 3), ("truth", C.c_float * 3),
                ("gamma", C.c_float), ("alpha_fixed", C.c_float), ("flags", C.c_uint32), ("key", C.c_uint32 * 2)]


class FxaaParams(C.Structure):
    _fields_ = [("subpix", C.c_float), ("edge_threshold", C.c_float), ("edge_threshold_min", C.c_float)]


class PostProcessParams(C.Structure):
    """taa_post_process_params_t: the post-process pass's push constants."""
    _fields_ = [("zoom_src_ltwh", C.c_int32 * 4), ("zoom_dst_ltwh", C.c_int32 * 4), ("debug_l_mask", C.c_float * 4),
                ("debug_r_mask", C.c_float * 4), ("zoom", C.c_uint32), ("show_zoom_box", C.c_uint32),
                ("split_x", C.c_int32), ("debug_l_show", C.c_uint32), ("debug_r_show", C.c_uint32)]


SETTINGS_MAX_SAMPLE_OFFSETS = 64


class Settings(C.Structure):
    _fields_ = [("param", Parameters * 2), ("mTaaEnabled", C.c_uint32), ("mSampleDistribution", C.c_int32),
                ("mSharpener", C.c_int32), ("mSharpenFactor", C.c_float), ("mSplitScreen", C.c_uint32),
                ("mSplitX", C.c_int32), ("mFixedJitterIndex", C.c_int32), ("mJitterExtraScale", C.c_float),
                ("mJitterSlowMotion", C.c_int32), ("mJitterRotateDegrees", C.c_float),
                ("mResetHistoryOnChange", C.c_uint32), ("mDebugSampleOffsetsCount", C.c_int32),
                ("mDebugSampleOffsets", (C.c_float * 2) * SETTINGS_MAX_SAMPLE_OFFSETS),
                ("mPostProcessEnabled", C.c_uint32), ("zoom", C.c_uint32), ("showZoomBox", C.c_uint32),
                ("zoomSrcLTWH", C.c_int32 * 4), ("zoomDstLTWH", C.c_int32 * 4)]


TAA_SCHEDULE_VIEW_ORDER, TAA_SCHEDULE_LARGEST_FIRST, TAA_SCHEDULE_INTERLEAVED = 0, 1, 2
BATCH_SLOTS = 4
TAA_BATCH_CTA_PER_TILE = -1


class SynthScene(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("width", C.c_int32), ("height", C.c_int32), ("seed", C.c_uint64),
        ("num_spheres", C.c_int32), ("radius_min", C.c_float), ("radius_max", C.c_float),
        ("sphere_speed_max", C.c_float), ("spin_max", C.c_float), ("cam_v0", C.c_float * 2),
        ("cam_accel", C.c_float * 2), ("checker_period", C.c_float), ("firefly_fraction", C.c_float),
        ("firefly_max", C.c_float), ("jitter_phase", C.c_int32), ("jitter_enabled", C.c_int32),
    ]


class SynthFrame(C.Structure):
    _fields_ = [("color", C.c_void_p), ("color_pitch", C.c_size_t), ("depth", C.c_void_p),
                ("depth_pitch", C.c_size_t), ("motion", C.c_void_p), ("motion_pitch", C.c_size_t),
                ("motion_channels", C.c_int32), ("truth", C.c_void_p), ("truth_pitch", C.c_size_t)]


SYNTH_MAX_SPHERES = 256
SYNTH_SPHERE_FLOATS = 12

assert C.sizeof(Parameters) == 176 and C.sizeof(Uniforms) == 544

# Every symbol include/taa_gb300.h and include/taa_synth.h declare.
EXPORTS = ["taa_version", "taa_last_error", "taa_default_parameters", "taa_get_jitter_offset",
           "taa_get_jitter_offset_custom", "taa_fxaa_default_params", "taa_fxaa", "taa_sharpen",
           "taa_post_process_default_params", "taa_post_process",
           "taa_settings_default", "taa_settings_write_ini", "taa_settings_read_ini",
           "taa_jittered_projection", "taa_compose_matrices", "taa_cas_setup", "taa_create", "taa_destroy",
           "taa_set_uniforms", "taa_set_sharpener", "taa_selected_form", "taa_resolve",
           "taa_resolve_static_scratch", "taa_device_status", "taa_debug_set_window_wait", "taa_batch_create", "taa_batch_destroy",
           "taa_batch_set_uniforms", "taa_batch_prepare", "taa_batch_launch", "taa_batch_autotune",
           "taa_batch_get_tuning", "taa_batch_set_tuning", "taa_mlp_init_weights", "taa_set_mlp", "taa_mlp_forward",
           "taa_mlp_trainer_create", "taa_mlp_trainer_destroy", "taa_mlp_collect", "taa_mlp_record_count",
           "taa_mlp_records", "taa_mlp_gradients", "taa_mlp_train",
           "taa_synth_default_scene", "taa_synth_spheres", "taa_synth_jitter", "taa_synth_camera",
           "taa_synth_render"]

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: build it with taa-star_gb300/build.py")
    lib = C.CDLL(str(p))
    P = C.POINTER
    sig = {
        "taa_version": (C.c_char_p, [P(C.c_int)]),
        "taa_last_error": (C.c_char_p, []),
        "taa_default_parameters": (C.c_int, [P(Parameters)]),
        "taa_get_jitter_offset": (C.c_int, [C.c_int32, C.c_uint64, C.c_int32, C.c_int32, P(JitterOpts),
                                            P(C.c_float), P(C.c_int32)]),
        "taa_get_jitter_offset_custom": (C.c_int, [C.c_void_p, C.c_int32, C.c_uint64, C.c_int32, C.c_int32,
                                                   P(JitterOpts), P(C.c_float)]),
        "taa_fxaa_default_params": (C.c_int, [P(FxaaParams)]),
        "taa_fxaa": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p,
                               C.c_size_t, C.c_int32, C.c_int32, P(FxaaParams)]),
        "taa_sharpen": (C.c_int, [C.c_void_p, C.c_uint32, C.c_float, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t,
                                  C.c_int32, C.c_int32]),
        "taa_post_process_default_params": (C.c_int, [C.c_int32, C.c_int32, P(PostProcessParams)]),
        "taa_post_process": (C.c_int, [C.c_void_p, P(PostProcessParams), C.c_void_p, C.c_size_t, C.c_void_p,
                                       C.c_size_t, C.c_void_p, C.c_size_t, C.c_int32, C.c_int32]),
        "taa_settings_default": (C.c_int, [P(Settings)]),
        "taa_settings_write_ini": (C.c_int, [P(Settings), C.c_char_p, C.c_size_t, P(C.c_size_t)]),
        "taa_settings_read_ini": (C.c_int, [P(Settings), C.c_char_p, C.c_size_t]),
        "taa_jittered_projection": (C.c_int, [P(C.c_float), P(C.c_float), P(C.c_float)]),
        "taa_compose_matrices": (C.c_int, [P(C.c_double)] * 4 + [P(C.c_float)] * 2),
        "taa_cas_setup": (C.c_int, [C.c_float] * 5 + [P(C.c_uint32)] * 2),
        "taa_create": (C.c_int, [P(Desc), P(C.c_void_p)]),
        "taa_destroy": (C.c_int, [C.c_void_p]),
        "taa_set_uniforms": (C.c_int, [C.c_void_p, P(Uniforms)]),
        "taa_set_sharpener": (C.c_int, [C.c_void_p, C.c_uint32, C.c_float]),
        "taa_selected_form": (C.c_int, [C.c_void_p]),
        "taa_resolve": (C.c_int, [C.c_void_p, C.c_void_p, P(FrameIO)]),
        "taa_resolve_static_scratch": (C.c_int, [C.c_void_p, C.c_void_p, P(FrameIO), C.c_uint32, C.c_float]),
        "taa_device_status": (C.c_int, [P(C.c_uint32), C.c_int]),
        "taa_debug_set_window_wait": (C.c_int, [C.c_uint32]),
        "taa_batch_create": (C.c_int, [P(Desc), C.c_int32, P(C.c_void_p)]),
        "taa_batch_destroy": (C.c_int, [C.c_void_p]),
        "taa_batch_set_uniforms": (C.c_int, [C.c_void_p, C.c_int32, P(Uniforms)]),
        "taa_batch_prepare": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, P(FrameIO)]),
        "taa_batch_launch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
        "taa_batch_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, P(BatchTuning)]),
        "taa_batch_get_tuning": (C.c_int, [C.c_void_p, P(BatchTuning)]),
        "taa_batch_set_tuning": (C.c_int, [C.c_void_p, P(BatchTuning)]),
        "taa_mlp_init_weights": (C.c_int, [P(MlpWeights), C.c_uint64, C.c_float]),
        "taa_set_mlp": (C.c_int, [C.c_void_p, P(MlpWeights)]),
        "taa_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
        "taa_mlp_trainer_create": (C.c_int, [C.c_int32, P(C.c_void_p)]),
        "taa_mlp_trainer_destroy": (C.c_int, [C.c_void_p]),
        "taa_mlp_collect": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, P(FrameIO), C.c_void_p, C.c_size_t,
                                      C.c_float, C.c_uint32]),
        "taa_mlp_record_count": (C.c_int, [C.c_void_p, P(C.c_int32)]),
        "taa_mlp_records": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, P(MlpRecord)]),
        "taa_mlp_gradients": (C.c_int, [C.c_void_p, P(MlpWeights), C.c_int32, C.c_int32, P(MlpWeights), P(C.c_float)]),
        "taa_mlp_train": (C.c_int, [C.c_void_p, P(MlpWeights), C.c_int32, C.c_int32, C.c_float, C.c_uint64,
                                    P(C.c_float), P(C.c_float)]),
        "taa_synth_default_scene": (C.c_int, [P(SynthScene), C.c_int32, C.c_int32, C.c_uint64]),
        "taa_synth_spheres": (C.c_int, [P(SynthScene), P(C.c_float), C.c_int32]),
        "taa_synth_jitter": (C.c_int, [P(SynthScene), C.c_int32, P(C.c_float), P(C.c_float)]),
        "taa_synth_camera": (C.c_int, [P(SynthScene), C.c_int32, P(C.c_double), P(C.c_double)]),
        "taa_synth_render": (C.c_int, [P(SynthScene), C.c_int32, C.c_void_p, P(SynthFrame)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class TaaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{code}: {msg}")
        self.code = code


def check(rc: int) -> int:
    if rc < 0:
        raise TaaError(rc, load().taa_last_error().decode())
    return rc


def device_status(clear: bool = True) -> int:
    """The device status word (TAA_DEVICE_* bits); waits for the device."""
    bits = C.c_uint32()
    check(load().taa_device_status(C.byref(bits), int(clear)))
    return bits.value


def set_window_wait(first_wait_polls: int = None):
    """Test hook: the first window wait's poll limit on the current device
    (None: the default, TAA_WINDOW_WAIT_POLLS)."""
    check(load().taa_debug_set_window_wait(TAA_WINDOW_WAIT_POLLS if first_wait_polls is None else first_wait_polls))


def default_parameters() -> Parameters:
    p = Parameters()
    check(load().taa_default_parameters(C.byref(p)))
    return p


def fxaa_default_params() -> FxaaParams:
    p = FxaaParams()
    check(load().taa_fxaa_default_params(C.byref(p)))
    return p


def fxaa(input, output, segmask=None, params: FxaaParams | None = None, stream: int = 0, ctx: "Taa | None" = None):
    """taa_fxaa on (H, W, 4) FP16 tensors; segmask an (H, W) int32/uint32 tensor or None;
    ctx a context created with TAA_FLAG_FXAA lends its work list."""
    h, w = int(input.shape[0]), int(input.shape[1])
    ip, ipitch = tensor_ptr_pitch(input)
    op, opitch = tensor_ptr_pitch(output)
    sp, spitch = tensor_ptr_pitch(segmask) if segmask is not None else (None, 0)
    check(load().taa_fxaa(ctx.handle if ctx is not None else None, C.c_void_p(stream), C.c_void_p(ip), ipitch,
                          C.c_void_p(sp), spitch, C.c_void_p(op), opitch, w, h,
                          C.byref(params) if params is not None else None))


def sharpen(input, output, sharpener: int, factor: float, stream: int = 0):
    """taa_sharpen on (H, W, 4) FP16 tensors."""
    h, w = int(input.shape[0]), int(input.shape[1])
    ip, ipitch = tensor_ptr_pitch(input)
    op, opitch = tensor_ptr_pitch(output)
    check(load().taa_sharpen(C.c_void_p(stream), sharpener, factor, C.c_void_p(ip), ipitch, C.c_void_p(op), opitch,
                             w, h))


def post_process_default_params(w: int, h: int) -> PostProcessParams:
    p = PostProcessParams()
    check(load().taa_post_process_default_params(w, h, C.byref(p)))
    return p


def post_process(input, output, params: PostProcessParams, debug=None, stream: int = 0):
    """taa_post_process on (H, W, 4) FP16 tensors (debug may be None when no side shows it)."""
    h, w = int(input.shape[0]), int(input.shape[1])
    ip, ipitch = tensor_ptr_pitch(input)
    op, opitch = tensor_ptr_pitch(output)
    dp, dpitch = tensor_ptr_pitch(debug) if debug is not None else (None, 0)
    check(load().taa_post_process(C.c_void_p(stream), C.byref(params), C.c_void_p(ip), ipitch, C.c_void_p(dp), dpitch,
                                  C.c_void_p(op), opitch, w, h))


def jitter_offset_custom(offsets_px, frame: int, w: int, h: int, opts: JitterOpts | None = None):
    """taa_get_jitter_offset_custom: sample distribution 5 over the given pixel offsets."""
    n = len(offsets_px)
    arr = ((C.c_float * 2) * max(n, 1))(*[(C.c_float * 2)(float(x), float(y)) for x, y in offsets_px])
    out = (C.c_float * 2)()
    check(load().taa_get_jitter_offset_custom(C.cast(arr, C.c_void_p), n, frame, w, h,
                                               C.byref(opts) if opts is not None else None, out))
    return out[0], out[1]


def settings_default() -> Settings:
    s = Settings()
    check(load().taa_settings_default(C.byref(s)))
    return s


def settings_to_ini(s: Settings) -> str:
    """The .ini text of the settings, as the reference writes it."""
    lib = load()
    n = C.c_size_t()
    check(lib.taa_settings_write_ini(C.byref(s), None, 0, C.byref(n)))
    buf = C.create_string_buffer(n.value + 1)
    check(lib.taa_settings_write_ini(C.byref(s), buf, n.value + 1, C.byref(n)))
    return buf.value.decode()


def settings_from_ini(text: str, base: Settings | None = None) -> Settings:
    """Settings read from .ini text over `base` (the defaults when None)."""
    s = Settings()
    C.memmove(C.addressof(s), C.addressof(base if base is not None else settings_default()), C.sizeof(s))
    raw = text.encode()
    check(load().taa_settings_read_ini(C.byref(s), raw, len(raw)))
    return s


def identity16():
    return (C.c_float * 16)(*[1.0 if i % 5 == 0 else 0.0 for i in range(16)])


def make_uniforms(p0: Parameters, p1: Parameters | None = None, jitter_ndc=(0.0, 0.0), **kw) -> Uniforms:
    u = Uniforms()
    u.mHistoryViewProjMatrix = identity16()
    u.mInverseViewProjMatrix = identity16()
    u.param[0] = p0
    u.param[1] = p1 if p1 is not None else p0
    u.mJitterNdc[0], u.mJitterNdc[1] = jitter_ndc
    u.mCamNearPlane = 0.1
    u.mCamFarPlane = 1000.0
    for k, v in kw.items():
        if k in ("mHistoryViewProjMatrix", "mInverseViewProjMatrix"):
            setattr(u, k, (C.c_float * 16)(*[float(x) for x in v]))
        else:
            setattr(u, k, v)
    return u


def tensor_ptr_pitch(t) -> tuple[int, int]:
    """Device pointer and row pitch in bytes of an (H, W, ...) tensor with contiguous rows."""
    return int(t.data_ptr()), int(t.stride(0) * t.element_size())


class Taa:
    """One resolve context (taa_create ... taa_destroy)."""

    def __init__(self, in_w, in_h, out_w=None, out_h=None, history_format=TAA_HISTORY_RGBA32F,
                 motion_format=TAA_MOTION_RG16F, form=TAA_FORM_AUTO, sharpener=TAA_SHARPEN_OFF, sharpen_factor=0.5,
                 flags=0):
        self.lib = load()
        d = Desc(C.sizeof(Desc), in_w, in_h, out_w or in_w, out_h or in_h, history_format, motion_format, form,
                 sharpener, sharpen_factor, flags)
        h = C.c_void_p()
        check(self.lib.taa_create(C.byref(d), C.byref(h)))
        self.handle = h
        self.desc = d

    def close(self):
        if self.handle:
            self.lib.taa_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_uniforms(self, u: Uniforms):
        check(self.lib.taa_set_uniforms(self.handle, C.byref(u)))

    def set_sharpener(self, mode: int, factor: float):
        check(self.lib.taa_set_sharpener(self.handle, mode, factor))

    def set_mlp(self, w: MlpWeights):
        check(self.lib.taa_set_mlp(self.handle, C.byref(w)))

    def mlp_forward(self, features, outputs, stream: int = 0):
        check(self.lib.taa_mlp_forward(self.handle, C.c_void_p(stream), C.c_void_p(features.data_ptr()),
                                       C.c_void_p(outputs.data_ptr()), int(features.shape[0])))

    def selected_form(self) -> int:
        return check(self.lib.taa_selected_form(self.handle))

    def resolve(self, stream: int = 0, **bindings):
        """bindings: name=tensor (or None) for the names of taa_frame_io_t."""
        io = FrameIO()
        for name, t in bindings.items():
            if name not in _IO_NAMES:
                raise KeyError(name)
            if t is None:
                continue
            p, pitch = tensor_ptr_pitch(t)
            setattr(io, name, p)
            setattr(io, name + "_pitch", pitch)
        check(self.lib.taa_resolve(self.handle, C.c_void_p(stream), C.byref(io)))


def frame_io(**bindings) -> FrameIO:
    """A taa_frame_io_t from name=tensor (or None) bindings."""
    io = FrameIO()
    for name, t in bindings.items():
        if name not in _IO_NAMES:
            raise KeyError(name)
        if t is None:
            continue
        p, pitch = tensor_ptr_pitch(t)
        setattr(io, name, p)
        setattr(io, name + "_pitch", pitch)
    return io


class Batch:
    """A batch of views resolved by one persistent launch (taa_batch_*)."""

    def __init__(self, sizes, motion_format=TAA_MOTION_RG16F, form=TAA_FORM_AUTO):
        self.lib = load()
        self.n = len(sizes)
        descs = (Desc * self.n)()
        for i, (w, h) in enumerate(sizes):
            descs[i] = Desc(C.sizeof(Desc), w, h, w, h, TAA_HISTORY_RGBA32F, motion_format, form,
                            TAA_SHARPEN_OFF, 0.5, 0)
        h = C.c_void_p()
        check(self.lib.taa_batch_create(descs, self.n, C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.taa_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_uniforms(self, view: int, u: Uniforms):
        check(self.lib.taa_batch_set_uniforms(self.handle, view, C.byref(u)))

    def prepare(self, slot: int, views: list[dict], stream: int = 0):
        ios = (FrameIO * self.n)(*[frame_io(**v) for v in views])
        check(self.lib.taa_batch_prepare(self.handle, C.c_void_p(stream), slot, ios))

    def launch(self, slot: int, stream: int = 0):
        check(self.lib.taa_batch_launch(self.handle, C.c_void_p(stream), slot))

    def autotune(self, slot: int, reps: int = 3, stream: int = 0) -> BatchTuning:
        t = BatchTuning()
        check(self.lib.taa_batch_autotune(self.handle, C.c_void_p(stream), slot, reps, C.byref(t)))
        return t

    def tuning(self) -> BatchTuning:
        t = BatchTuning()
        check(self.lib.taa_batch_get_tuning(self.handle, C.byref(t)))
        return t

    def set_tuning(self, tile_w, tile_h, schedule, ctas_per_sm=0, form=TAA_FORM_TILED):
        t = BatchTuning(tile_w, tile_h, schedule, ctas_per_sm, 0.0, form)
        check(self.lib.taa_batch_set_tuning(self.handle, C.byref(t)))


def mlp_init_weights(seed: int = 1, alpha0: float = 0.1) -> MlpWeights:
    w = MlpWeights()
    check(load().taa_mlp_init_weights(C.byref(w), seed, alpha0))
    return w


def mlp_to_numpy(w: MlpWeights) -> dict:
    import numpy as np
    return dict(w1=np.ctypeslib.as_array(w.w1).reshape(32, 32).astype(np.float64), b1=np.ctypeslib.as_array(w.b1).astype(np.float64),
                w2=np.ctypeslib.as_array(w.w2).reshape(32, 32).astype(np.float64), b2=np.ctypeslib.as_array(w.b2).astype(np.float64),
                w3=np.ctypeslib.as_array(w.w3).reshape(2, 32).astype(np.float64), b3=np.ctypeslib.as_array(w.b3).astype(np.float64))


class MlpTrainer:
    """Record collection and training of the learned rectifier (taa_mlp_*)."""

    def __init__(self, capacity: int):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.taa_mlp_trainer_create(capacity, C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.taa_mlp_trainer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def collect(self, ctx: "Taa", truth, fraction: float, seed: int, stream: int = 0, **bindings):
        io = frame_io(**bindings)
        p, pitch = tensor_ptr_pitch(truth)
        check(self.lib.taa_mlp_collect(self.handle, ctx.handle, C.c_void_p(stream), C.byref(io), C.c_void_p(p), pitch,
                                       fraction, seed))

    def count(self) -> int:
        n = C.c_int32()
        check(self.lib.taa_mlp_record_count(self.handle, C.byref(n)))
        return n.value

    def records(self, first: int, count: int):
        import numpy as np
        buf = (MlpRecord * count)()
        check(self.lib.taa_mlp_records(self.handle, first, count, buf))
        raw = np.frombuffer(buf, dtype=np.uint8).reshape(count, C.sizeof(MlpRecord))
        f32 = raw.view(np.float32)
        return dict(features=raw[:, :64].copy().view(np.float16).astype(np.float64),
                    mean=f32[:, 16:19].astype(np.float64), sigma=f32[:, 19:22].astype(np.float64),
                    history=f32[:, 22:25].astype(np.float64), current=f32[:, 25:28].astype(np.float64),
                    truth=f32[:, 28:31].astype(np.float64), gamma=f32[:, 31].astype(np.float64),
                    alpha_fixed=f32[:, 32].astype(np.float64), flags=raw.view(np.uint32)[:, 33].copy(), key=raw.view(np.uint32)[:, 34:36].copy())

    def gradients(self, w: MlpWeights, first: int, count: int):
        g = MlpWeights()
        loss = C.c_float()
        check(self.lib.taa_mlp_gradients(self.handle, C.byref(w), first, count, C.byref(g), C.byref(loss)))
        return g, loss.value

    def train(self, w: MlpWeights, steps: int, batch: int, lr: float, seed: int = 1):
        lf, ll = C.c_float(), C.c_float()
        check(self.lib.taa_mlp_train(self.handle, C.byref(w), steps, batch, lr, seed, C.byref(lf), C.byref(ll)))
        return lf.value, ll.value


def synth_default_scene(w, h, seed) -> SynthScene:
    s = SynthScene()
    check(load().taa_synth_default_scene(C.byref(s), w, h, seed))
    return s


def synth_spheres(scene: SynthScene):
    import numpy as np
    buf = (C.c_float * (SYNTH_MAX_SPHERES * SYNTH_SPHERE_FLOATS))()
    check(load().taa_synth_spheres(C.byref(scene), buf, SYNTH_MAX_SPHERES))
    return np.frombuffer(buf, dtype=np.float32).reshape(SYNTH_MAX_SPHERES, SYNTH_SPHERE_FLOATS)[
        : scene.num_spheres].copy()


def synth_jitter(scene: SynthScene, frame: int):
    px = (C.c_float * 2)()
    ndc = (C.c_float * 2)()
    check(load().taa_synth_jitter(C.byref(scene), frame, px, ndc))
    return (px[0], px[1]), (ndc[0], ndc[1])


def synth_camera(scene: SynthScene, frame: int):
    import numpy as np
    p = (C.c_double * 16)()
    v = (C.c_double * 16)()
    check(load().taa_synth_camera(C.byref(scene), frame, p, v))
    return np.array(p[:]), np.array(v[:])


def compose_matrices(pc, vc, pp, vp):
    import numpy as np
    arr = [(C.c_double * 16)(*[float(x) for x in m]) for m in (pc, vc, pp, vp)]
    inv = (C.c_float * 16)()
    hist = (C.c_float * 16)()
    check(load().taa_compose_matrices(*arr, inv, hist))
    return np.array(inv[:], dtype=np.float32), np.array(hist[:], dtype=np.float32)


def synth_render(scene: SynthScene, frame: int, stream: int = 0, color=None, depth=None, motion=None, truth=None):
    f = SynthFrame()
    for name, t in (("color", color), ("depth", depth), ("motion", motion), ("truth", truth)):
        if t is not None:
            p, pitch = tensor_ptr_pitch(t)
            setattr(f, name, p)
            setattr(f, name + "_pitch", pitch)
    if motion is not None:
        f.motion_channels = int(motion.shape[-1])
    check(load().taa_synth_render(C.byref(scene), frame, C.c_void_p(stream), C.byref(f)))
