"""Training and evaluation of the learned rectifier on the synthetic renderer.

The workflow the C ABI supports (include/taa_gb300.h, taa_mlp_*), in Python:

* ``collect`` renders sequences of the seeded analytic scene on the GPU (with
  64-spp ground truth), resolves each frame with the plain variance clip and
  keeps a hashed sample of pixels as training records;
* ``train`` runs the library's tensor-core training kernels (Adam);
* ``evaluate`` resolves a sequence with a given form and reports the PSNR of
  every frame's result against the ground truth.

Everything runs on the device; the renderer, the resolve and the training are
the library's own kernels.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

import taa_abi as T
import workloads as WL


@dataclass
class Frames:
    color: list
    depth: list
    motion: list
    truth: list
    jitter: list


def render(wl: WL.Workload, frames: int, dev, truth: bool = True) -> Frames:
    import torch
    sc = wl.scene()
    H, W = wl.height, wl.width
    out = Frames([], [], [], [], [])
    for f in range(frames):
        c = torch.empty(H, W, 4, dtype=torch.float16, device=dev)
        d = torch.empty(H, W, dtype=torch.float32, device=dev)
        m = torch.empty(H, W, 2, dtype=torch.float16, device=dev)
        t = torch.empty(H, W, 4, dtype=torch.float32, device=dev) if truth else None
        T.synth_render(sc, f, color=c, depth=d, motion=m, truth=t)
        out.color.append(c)
        out.depth.append(d)
        out.motion.append(m)
        out.truth.append(t)
        out.jitter.append(T.synth_jitter(sc, f)[1])
    return out


def collect(trainer: T.MlpTrainer, wl: WL.Workload, frames: int, dev, fraction: float, skip: int = 4,
            seed: int = 0) -> int:
    """Resolves `frames` frames of the workload with the plain variance clip
    and records a `fraction` of the pixels of every frame after `skip`."""
    import torch
    fr = render(wl, frames, dev)
    H, W = wl.height, wl.width
    ctx = T.Taa(W, H, form=T.TAA_FORM_LEARNED)
    hist = [torch.zeros(H, W, 4, device=dev), torch.zeros(H, W, 4, device=dev)]
    for f in range(frames):
        ctx.set_uniforms(T.make_uniforms(wl.parameters(), jitter_ndc=fr.jitter[f], mResetHistory=1 if f == 0 else 0))
        b = dict(color=fr.color[f], depth=fr.depth[f], velocity=fr.motion[f], history=hist[f & 1],
                 history_depth=fr.depth[f - 1] if f else fr.depth[0], history_out=hist[(f + 1) & 1])
        trainer.collect(ctx, fr.truth[f], fraction if f >= skip else 0.0, seed * 1000 + f, **b)
    torch.cuda.synchronize()
    ctx.close()
    return trainer.count()


def train(trainer: T.MlpTrainer, seed: int = 1, steps: int = 3000, batch: int = 8192, lr: float = 2e-3,
          alpha0: float = 0.1):
    w = T.mlp_init_weights(seed, alpha0)
    first, last = trainer.train(w, steps, batch, lr, seed)
    return w, first, last


def psnr(a, ref) -> float:
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(ref, np.float64)) ** 2))
    peak = float(np.max(np.abs(ref)))
    return float("inf") if mse == 0 else 10.0 * math.log10(peak * peak / mse)


def evaluate(wl: WL.Workload, frames: int, dev, form: int, weights: T.MlpWeights | None = None,
             fr: Frames | None = None, skip: int = 8, flags: int = 0, stats: dict | None = None):
    """Per-frame PSNR (frames >= skip) of the resolved history against the
    ground truth, and the largest absolute error.  With `stats`, its "q9999"
    entry receives each frame's 99.99th percentile of the per-pixel error (the
    largest channel's absolute error)."""
    import torch
    fr = fr or render(wl, frames, dev)
    H, W = wl.height, wl.width
    ctx = T.Taa(W, H, form=form, flags=flags)
    if weights is not None:
        ctx.set_mlp(weights)
    hist = [torch.zeros(H, W, 4, device=dev), torch.zeros(H, W, 4, device=dev)]
    out, maxerr = [], 0.0
    for f in range(frames):
        ctx.set_uniforms(T.make_uniforms(wl.parameters(), jitter_ndc=fr.jitter[f], mResetHistory=1 if f == 0 else 0))
        ctx.resolve(color=fr.color[f], depth=fr.depth[f], velocity=fr.motion[f], history=hist[f & 1],
                    history_depth=fr.depth[f - 1] if f else fr.depth[0], history_out=hist[(f + 1) & 1])
        if f >= skip:
            res = hist[(f + 1) & 1][..., :3].cpu().numpy()
            ref = fr.truth[f][..., :3].cpu().numpy()
            out.append(psnr(res, ref))
            maxerr = max(maxerr, float(np.max(np.abs(res - ref))))
            if stats is not None:
                stats.setdefault("q9999", []).append(float(np.quantile(np.max(np.abs(res - ref), axis=-1), 0.9999)))
    ctx.close()
    return out, maxerr
