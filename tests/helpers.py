"""Shared helpers of the test suite: synthetic inputs, uploads, error metrics."""
from __future__ import annotations

import numpy as np

import oracle as O
import taa_abi as T
import workloads as WL


def cpu_frames(wl: WL.Workload, frames: range, motion_channels: int = 2):
    """Inputs of the given frames rendered by the FP64 scene evaluator and
    stored in the texel formats of the resolve (colour/motion FP16, depth FP32).
    Returns a list of dicts with float32 numpy arrays (the exact FP16 values)."""
    scene = wl.scene()
    sph = T.synth_spheres(scene)
    out = []
    for f in frames:
        r = O.synth_frame(scene, sph, f)
        color = r["color"].astype(np.float16)
        motion = r["motion"][..., :motion_channels].astype(np.float16)
        out.append(dict(frame=f, color=color, depth=r["depth"].astype(np.float32), motion=motion,
                        jitter=T.synth_jitter(scene, f)[1]))
    return out


def widen(a16):
    return np.asarray(a16, dtype=np.float32)


def max_rel(a, ref, floor=1e-3):
    """max |a - ref| / max(|ref|, floor) over all elements."""
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.max(np.abs(a - ref) / np.maximum(np.abs(ref), floor))) if a.size else 0.0


def rel_l2(a, ref):
    """Frame-level relative error ||a - ref||_2 / ||ref||_2."""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    n = float(np.linalg.norm(ref))
    return float(np.linalg.norm(a - ref)) / n if n else float(np.linalg.norm(a))


def half_ulp(x):
    """Spacing of binary16 at |x| (normal range), for comparisons after an FP16 store."""
    x = np.abs(np.asarray(x, dtype=np.float64))
    e = np.floor(np.log2(np.maximum(x, 2.0 ** -14)))
    return 2.0 ** (e - 10)


def psnr(a, ref, peak=None):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    mse = float(np.mean((a - ref) ** 2))
    peak = float(np.max(np.abs(ref))) if peak is None else peak
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)


def uniforms_for(wl: WL.Workload, frame_jitter_ndc, p0=None, **kw) -> T.Uniforms:
    return T.make_uniforms(p0 if p0 is not None else wl.parameters(), jitter_ndc=frame_jitter_ndc, **kw)


# ---------------------------------------------------------------- GPU side
def to_dev(a, dtype, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def gpu_resolve(ctx: T.Taa, dev, color, depth, motion, history, history_depth=None, history_fp16=False,
                want_result=True, want_sharpened=False, want_debug=False, stream=0):
    """Run one resolve on the GPU from numpy inputs; returns numpy outputs."""
    import torch
    H, W = color.shape[:2]
    oh, ow = ctx.desc.out_height, ctx.desc.out_width
    hist_dtype = torch.float16 if history_fp16 else torch.float32
    b = dict(
        color=to_dev(color, torch.float16, dev),
        depth=to_dev(depth, torch.float32, dev),
        velocity=to_dev(motion, torch.float16, dev),
        history=None if history is None else to_dev(history, hist_dtype, dev),
        history_depth=None if history_depth is None else to_dev(history_depth, torch.float32, dev),
        history_out=torch.full((oh, ow, 4), float("nan"), dtype=hist_dtype, device=dev),
        result=torch.full((oh, ow, 4), float("nan"), dtype=torch.float16, device=dev) if want_result else None,
        sharpened=torch.full((oh, ow, 4), float("nan"), dtype=torch.float16, device=dev) if want_sharpened else None,
        debug=torch.full((oh, ow, 4), float("nan"), dtype=torch.float16, device=dev) if want_debug else None,
    )
    ctx.resolve(stream=stream, **b)
    torch.cuda.synchronize()
    out = {k: b[k].float().cpu().numpy() for k in ("history_out", "result", "sharpened", "debug") if b[k] is not None}
    return out
