"""Generate the golden fixtures that pin the oracle to the reference's own code.

Runs where the reference tree is present: it builds oracle/_ref (the
reference's shaders/taa.comp and shaders/sharpen.comp compiled as C++ through
oracle/ref_shim, and CasSetup from shaders/ffx_cas.h with A_CPU) and records,
on small seeded inputs and for every parameter mode listed below, what the
reference code computes:

  taa_comp_golden.npz   inputs (colour, depth, velocity, history, previous
                        depth, material ids, uv/normals, previous segmask),
                        the 544-byte uniform block of each case, and the
                        reference outputs: FP64 history/screen/debug/segmask
                        and FP32 history/screen
  cas_setup_golden.json CasSetup const0/const1 for a set of sharpness values
  sharpen_golden.npz    shaders/sharpen.comp on one image (FP64 and FP32)
  cas_golden.npz        shaders/sharpen_cas.comp (FidelityFX CAS, FP32) on
                        seeded HDR images of several sizes (values up to 4,
                        so the filter's saturation is exercised) for several
                        sharpness values, with CasSetup's constants
  fxaa_golden.npz       shaders/antialias_fxaa_prepare.comp, then (through an
                        RGBA16F image, as source/taa.hpp:1063-1104 chains them)
                        shaders/antialias_fxaa.comp with Fxaa3_11_mod.h, on a
                        rendered frame with three segmentation masks (FP64 and
                        FP32)
  post_golden.npz       shaders/post_process.comp on a seeded RGBA16F image and
                        debug image for seven push-constant sets (split line,
                        debug on either side with and without its alpha shown,
                        zoom box and inset, the size-derived defaults of
                        source/taa.hpp:352-359) (FP64 and FP32)

Usage: python tests/golden/make_golden.py [taa] [cas] [casfilter] [sharpen] [fxaa] [post]   (default: all)
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (ROOT / "taa-star_gb300", ROOT / "oracle", ROOT / "tests"):
    sys.path.insert(0, str(p))

import oracle as O  # noqa: E402
import taa_abi as T  # noqa: E402
import workloads as WL  # noqa: E402

MODES = {
    "base": {},
    "c2_depth_reject": dict(mDepthCulling=1, mRejectOutside=1),
    "bilinear": dict(mInterpolationMode=0),
    "bspline": dict(mInterpolationMode=1),
    "clamp_rgb_minmax": dict(mColorClampingOrClipping=1, mUseYCoCg=0, mVarianceClipping=0),
    "no_clip": dict(mColorClampingOrClipping=0),
    "clip_slow_shaped": dict(mColorClampingOrClipping=3, mShapedNeighbourhood=1, mVarianceClipping=0),
    "clip_slow_variance": dict(mColorClampingOrClipping=3),
    "shrink_chroma": dict(mShrinkChromaAxis=1),
    "tonemap_lottes": dict(mToneMapLumaKaris=1, mLumaWeightingLottes=1),
    "near_clamp_velalpha": dict(mReduceBlendNearClamp=1, mVelBasedAlpha=1, mVelBasedAlphaFactor=40.0),
    "velocity_closest": dict(mVelocitySampleMode=2),
    "velocity_longest": dict(mVelocitySampleMode=1),
    "velocity_movers_only": dict(mUseVelocityVectors=1),
    "reprojection_only": dict(mUseVelocityVectors=0),
    "anti_ghosting": dict(mDynamicAntiGhosting=1),
    "noise": dict(mAddNoise=1),
    "unjitter": dict(mUnjitterNeighbourhood=1, mUnjitterCurrentSample=1),
    "gamma_1_5": dict(mVarClipGamma=1.5),
    "segmask_all_tests": dict(mRayTraceAugment=1, mRayTraceAugmentFlags=0x7F, mRayTraceHistoryCount=8),
    "segmask_no_history_count": dict(mRayTraceAugment=1, mRayTraceAugmentFlags=0x3F),
    "segmask_all": dict(mRayTraceAugment=1, mRayTraceAugmentFlags=0x80),
    "segmask_fixed_border": dict(mRayTraceAugment=1, mRayTraceAugmentFlags=0x100 | 0x3F),
}
for d in range(9):
    MODES[f"debug_{d}"] = dict(mDebugMode=d, mDebugScale=2.0, mDebugCenter=1 if d % 2 else 0)

UNIFORM_CASES = {
    "pass_through": dict(p0=dict(mPassThrough=1)),
    "bypass": dict(kw=dict(mBypassHistoryUpdate=1)),
    "reset": dict(kw=dict(mResetHistory=1)),
    "split_screen": dict(p1=dict(mInterpolationMode=0, mColorClampingOrClipping=1, mAlpha=0.3),
                         kw=dict(splitScreen=1, splitX=11)),
}


def scene_inputs(w, h, seed):
    wl = WL.small(w, h, frames=2, seed=seed)
    sc = wl.scene()
    sph = T.synth_spheres(sc)
    fr = [O.synth_frame(sc, sph, f) for f in range(2)]
    rng = np.random.default_rng(seed)
    col = fr[1]["color"].astype(np.float16).astype(np.float32)
    vel = fr[1]["motion"].astype(np.float16).astype(np.float32)
    mover = vel[..., 3] > 0.5
    mat = ((vel[..., 3].astype(np.uint32) % 7) + 1) | np.where(mover, np.uint32(0x80000000), np.uint32(0))
    pmat = np.roll(mat, 1, axis=1)
    ang = np.stack([rng.uniform(0, 6.28, (h, w)), rng.uniform(-1.5, 1.5, (h, w))], -1).astype(np.float32)
    uvnrm = np.concatenate([rng.uniform(0, 1, (h, w, 2)).astype(np.float32), ang], -1)
    pseg = (rng.integers(0, 4, (h, w)).astype(np.uint32) << 16) | rng.integers(0, 3, (h, w)).astype(np.uint32)
    return dict(color=col, depth=fr[1]["depth"].astype(np.float32), velocity=vel,
                history=fr[0]["color"].astype(np.float16).astype(np.float32),
                history_depth=fr[0]["depth"].astype(np.float32), material=mat.astype(np.uint32),
                prev_material=pmat.astype(np.uint32), uvnrm=uvnrm, prev_segmask=pseg,
                jitter=np.array(T.synth_jitter(sc, 1)[1], np.float32))


def main():
    import build_oracle
    libs = build_oracle.build_reference(force=True)
    if not libs:
        raise SystemExit("the reference tree is not present; nothing to generate")
    P = C.POINTER
    fp, dp, up = P(C.c_float), P(C.c_double), P(C.c_uint32)

    def load(name):
        lib = C.CDLL(str(libs[name]))
        lib.ref_taa_resolve.argtypes = [C.c_void_p] + [C.c_int] * 4 + [fp] * 5 + [up] * 3 + [fp] + [dp] * 3 + [up]
        lib.ref_sharpen.argtypes = [fp, C.c_int, C.c_int, C.c_float, dp]
        return lib

    ref = {32: load("libtaa_ref32.so"), 64: load("libtaa_ref64.so")}

    def f(a):
        return np.ascontiguousarray(a, np.float32).ctypes.data_as(fp)

    def u32(a):
        return np.ascontiguousarray(a, np.uint32).ctypes.data_as(up)

    which = set(sys.argv[1:]) or {"taa", "cas", "casfilter", "sharpen", "fxaa", "post"}
    if "taa" in which:
        make_taa(ref, f, u32, dp, up)
    if "cas" in which:
        make_cas(libs)
    if "casfilter" in which:
        make_cas_filter(libs, f, dp)
    if "sharpen" in which:
        make_sharpen(ref, f, dp)
    if "fxaa" in which:
        make_fxaa(libs, fp, dp, up)
    if "post" in which:
        make_post(libs, fp, dp)


def make_taa(ref, f, u32, dp, up):
    out = {}
    cases = []
    for scene_name, (w, h, ow, oh, seed) in {"s": (24, 16, 24, 16, 21), "up": (16, 10, 32, 20, 22)}.items():
        inp = scene_inputs(w, h, seed)
        hist = inp["history"] if (ow, oh) == (w, h) else np.repeat(np.repeat(inp["history"], 2, 0), 2, 1)
        pseg = inp["prev_segmask"] if (ow, oh) == (w, h) else np.repeat(np.repeat(inp["prev_segmask"], 2, 0), 2, 1)
        for k in ("color", "depth", "velocity", "history_depth", "material", "prev_material", "uvnrm", "jitter"):
            out[f"{scene_name}/{k}"] = inp[k]
        out[f"{scene_name}/history"] = np.ascontiguousarray(hist)
        out[f"{scene_name}/prev_segmask"] = np.ascontiguousarray(pseg)
        items = []
        if scene_name == "s":
            items += [(m, dict(p0=kw)) for m, kw in MODES.items()]
            items += list(UNIFORM_CASES.items())
        else:
            items += [("upsample", dict(kw=dict(mUpsampling=1))),
                      ("upsample_unjitter", dict(p0=dict(mUnjitterCurrentSample=1, mUnjitterNeighbourhood=1),
                                                 kw=dict(mUpsampling=1))),
                      ("upsample_bilinear", dict(p0=dict(mInterpolationMode=0), kw=dict(mUpsampling=1)))]
        for name, spec in items:
            p0 = WL.base_parameters(**spec.get("p0", {}))
            p1 = WL.base_parameters(**spec.get("p1", {})) if "p1" in spec else None
            kw = dict(spec.get("kw", {}))
            kw.setdefault("mSinTime", (C.c_float * 4)(0.3, 0.5, 0.7, 0.9))
            u = T.make_uniforms(p0, p1, jitter_ndc=tuple(inp["jitter"]), **kw)
            key = f"{scene_name}:{name}"
            res = {}
            for prec in (64, 32):
                oh_ = np.zeros((oh, ow, 4))
                os_ = np.zeros((oh, ow, 4))
                od = np.zeros((oh, ow, 4))
                sg = np.zeros((oh, ow), np.uint32)
                vel4 = np.ascontiguousarray(inp["velocity"], np.float32)
                ref[prec].ref_taa_resolve(C.addressof(u), w, h, ow, oh, f(inp["color"]), f(inp["depth"]), f(hist),
                                          f(inp["history_depth"]), f(vel4), u32(inp["material"]),
                                          u32(inp["prev_material"]), u32(pseg), f(inp["uvnrm"]),
                                          oh_.ctypes.data_as(dp), os_.ctypes.data_as(dp), od.ctypes.data_as(dp),
                                          sg.ctypes.data_as(up))
                res[prec] = (oh_, os_, od, sg)
            out[f"{key}/uniforms"] = np.frombuffer(bytes(u), np.uint8).copy()
            out[f"{key}/ref64_history"] = res[64][0]
            out[f"{key}/ref64_screen"] = res[64][1]
            out[f"{key}/ref64_debug"] = res[64][2]
            out[f"{key}/ref64_segmask"] = res[64][3]
            out[f"{key}/ref32_history"] = res[32][0].astype(np.float32)
            out[f"{key}/ref32_screen"] = res[32][1].astype(np.float32)
            cases.append(key)
    out["cases"] = np.array(cases)
    np.savez_compressed(HERE / "taa_comp_golden.npz", **out)
    print(f"{len(cases)} resolve cases written to {HERE}")


def make_cas(libs):
    cas = C.CDLL(str(libs["libcas_ref.so"]))
    rows = []
    for s in (0.0, 0.1, 0.25, 0.5, 0.75, 1.0, 1.5, -0.5):
        for dims in ((1920, 1080, 1920, 1080), (2560, 1440, 2560, 1440), (1280, 720, 1920, 1080)):
            c0 = (C.c_uint32 * 4)()
            c1 = (C.c_uint32 * 4)()
            cas.ref_cas_setup(C.c_float(s), *map(C.c_float, dims), c0, c1)
            rows.append(dict(sharpness=s, dims=dims, const0=list(c0), const1=list(c1)))
    (HERE / "cas_setup_golden.json").write_text(json.dumps(rows, indent=1) + "\n")
    print(f"{len(rows)} CasSetup rows written to {HERE}")


def make_cas_filter(libs, f, dp):
    setup = C.CDLL(str(libs["libcas_ref.so"]))
    filt = C.CDLL(str(libs["libcas_filter_ref.so"]))
    filt.ref_cas.argtypes = [C.POINTER(C.c_float), C.c_int, C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                             C.POINTER(C.c_double)]
    rng = np.random.default_rng(11)
    out = {}
    cases = []
    # sizes: a whole 16x16 work group, ragged edges, one row and one column
    for (w, h) in ((16, 16), (37, 23), (70, 41), (1, 9), (9, 1)):
        # RGBA16F values: mostly [0, 1.2] with 3 % of texels up to 4 (HDR, clipped by the filter)
        img = rng.uniform(0.0, 1.2, (h, w, 4))
        hot = rng.uniform(size=(h, w)) < 0.03
        img[hot, :3] = rng.uniform(1.0, 4.0, (int(hot.sum()), 3))
        img = img.astype(np.float16).astype(np.float32)
        for s_ in (0.0, 0.25, 0.5, 1.0):
            c0 = (C.c_uint32 * 4)()
            c1 = (C.c_uint32 * 4)()
            setup.ref_cas_setup(C.c_float(s_), *(C.c_float(v) for v in (w, h, w, h)), c0, c1)
            o = np.zeros((h, w, 4))
            filt.ref_cas(f(img), w, h, c0, c1, o.ctypes.data_as(dp))
            key = f"{w}x{h}_s{s_}"
            out[f"{key}/image"] = img
            out[f"{key}/const1"] = np.array(list(c1), np.uint32)
            out[f"{key}/ref32"] = o[..., :3].astype(np.float32)
            cases.append(key)
    out["cases"] = np.array(cases)
    np.savez_compressed(HERE / "cas_golden.npz", **out)
    print(f"{len(cases)} CAS filter cases written to {HERE}")


def make_sharpen(ref, f, dp):
    rng = np.random.default_rng(5)
    img = rng.uniform(0, 1.2, (13, 19, 4)).astype(np.float16).astype(np.float32)
    sh = {}
    for prec in (64, 32):
        o = np.zeros((13, 19, 4))
        ref[prec].ref_sharpen(f(img), 19, 13, C.c_float(0.6), o.ctypes.data_as(dp))
        sh[f"ref{prec}"] = o
    np.savez_compressed(HERE / "sharpen_golden.npz", image=img, factor=np.float32(0.6), **sh)
    print(f"sharpen fixture written to {HERE}")


def make_fxaa(libs, fp, dp, up):
    P = C.POINTER
    ref = {}
    for prec in (32, 64):
        lib = C.CDLL(str(libs[f"libfxaa_ref{prec}.so"]))
        lib.ref_fxaa_prepare.argtypes = [fp, C.c_int, C.c_int, dp]
        lib.ref_fxaa.argtypes = [fp, up, C.c_int, C.c_int] + [C.c_float] * 5 + [dp]
        ref[prec] = lib
    # a rendered frame of the synthetic scene (sphere silhouettes, checkerboard),
    # stored as the RGBA16F result image the FXAA passes read
    w, h = 72, 48
    wl = WL.small(w, h, frames=1, seed=31)
    sc = wl.scene()
    img = O.synth_frame(sc, T.synth_spheres(sc), 0)["color"].astype(np.float16).astype(np.float32)
    img = np.ascontiguousarray(img)
    rng = np.random.default_rng(7)
    masks = {
        "random": rng.integers(0, 1 << 20, (h, w)).astype(np.uint32),  # (mask & 3) == 1 on about a quarter
        "all": np.ones((h, w), np.uint32),
        "none": np.zeros((h, w), np.uint32),
    }
    params = (0.75, 0.116, 0.0833)  # source/taa.hpp:95-97
    rcp = np.float32(1.0) / np.array([w, h], np.float32)
    out = dict(image=img, params=np.array(params, np.float32), rcp=rcp)
    for name, m in masks.items():
        out[f"{name}/segmask"] = m
        for prec in (64, 32):
            prep = np.zeros((h, w, 4))
            ref[prec].ref_fxaa_prepare(img.ctypes.data_as(fp), w, h, prep.ctypes.data_as(dp))
            prep16 = np.ascontiguousarray(prep.astype(np.float16).astype(np.float32))  # the RGBA16F temp image
            res = np.zeros((h, w, 4))
            mm = np.ascontiguousarray(m)
            ref[prec].ref_fxaa(prep16.ctypes.data_as(fp), mm.ctypes.data_as(up), w, h, float(rcp[0]), float(rcp[1]),
                               *params, res.ctypes.data_as(dp))
            out[f"{name}/ref{prec}"] = res if prec == 64 else res.astype(np.float32)
    np.savez_compressed(HERE / "fxaa_golden.npz", **out)
    print(f"fxaa fixture written to {HERE}")


POST_CASES = {
    "defaults": dict(),
    "split_debug_left_alpha": dict(split_x=36, show_l=True, mask_l=(1.0, 1.0, 1.0, 1.0)),
    "split_debug_right": dict(split_x=20, show_r=True, mask_r=(0.0, 1.0, 0.0, 0.0)),
    "zoom_box": dict(zoom=True, zoom_src=(10, 8, 7, 5), zoom_dst=(40, 20, 25, 18)),
    "zoom_no_box_split": dict(zoom=True, show_zoom_box=False, zoom_src=(3, 4, 9, 9), zoom_dst=(50, 25, 16, 16),
                              split_x=30, show_l=True, mask_l=(1.0, 1.0, 1.0, 0.5)),
    "zoom_debug_both_sides": dict(zoom=True, zoom_src=(60, 30, 6, 6), zoom_dst=(2, 2, 30, 30), split_x=50,
                                  show_l=True, show_r=True, mask_r=(1.0, 1.0, 1.0, 1.0)),
    # source/taa.hpp:352-359 at 72 x 48: zoom source (35, 23, 1, 1), inset (65, 0, 7, 7) (72 / 9.6f < 7.5)
    "size_defaults_zoom": dict(zoom=True, zoom_src=(35, 23, 1, 1), zoom_dst=(65, 0, 7, 7)),
}


def make_post(libs, fp, dp):
    ip = C.POINTER(C.c_int)
    ref = {}
    for prec in (32, 64):
        lib = C.CDLL(str(libs[f"libpost_ref{prec}.so"]))
        lib.ref_post_process.argtypes = [fp, fp, C.c_int, C.c_int, ip, ip, fp, fp] + [C.c_int] * 5 + [dp]
        ref[prec] = lib
    w, h = 72, 48
    rng = np.random.default_rng(17)
    img = np.ascontiguousarray(rng.uniform(0.0, 4.0, (h, w, 4)).astype(np.float16).astype(np.float32))
    dbg = np.ascontiguousarray(rng.uniform(-1.0, 2.0, (h, w, 4)).astype(np.float16).astype(np.float32))
    out = dict(image=img, debug=dbg)
    for name, over in POST_CASES.items():
        pp = dict(O.POST_DEFAULTS)
        pp.update(over)
        out[f"{name}/params"] = np.array(json.dumps({k: list(v) if isinstance(v, tuple) else v for k, v in pp.items()}))
        iv = lambda v: (C.c_int * 4)(*v)
        fv = lambda v: np.ascontiguousarray(v, np.float32)
        ml, mr = fv(pp["mask_l"]), fv(pp["mask_r"])
        for prec in (64, 32):
            res = np.zeros((h, w, 4))
            ref[prec].ref_post_process(img.ctypes.data_as(fp), dbg.ctypes.data_as(fp), w, h, iv(pp["zoom_src"]),
                                       iv(pp["zoom_dst"]), ml.ctypes.data_as(fp), mr.ctypes.data_as(fp),
                                       int(pp["zoom"]), int(pp["show_zoom_box"]), int(pp["split_x"]),
                                       int(pp["show_l"]), int(pp["show_r"]), res.ctypes.data_as(dp))
            # every FP64 output here is a float32 value (copied half texels, 0/1, half + half)
            r32 = res.astype(np.float32)
            out[f"{name}/ref{prec}"] = r32 if np.array_equal(r32.astype(np.float64), res) else res
    np.savez_compressed(HERE / "post_golden.npz", **out)
    print(f"post-process fixture written to {HERE}")


if __name__ == "__main__":
    main()
