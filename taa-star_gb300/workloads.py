"""The five benchmark workloads and their parameter blocks.

C1  plain resolve, 1280x720, 16 frames, Catmull-Rom history, YCoCg variance
    clip (gamma 1), clip-fast, alpha 0.1, velocity for every pixel.
C2  the same generator at 3840x2160, 64 frames, pan accelerating to 40
    px/frame, 128 spheres, depth culling and out-of-screen rejection.
C3  resolve + CAS sharpen 0.5 fused, 2560x1440, 32 frames, spinning
    spheres, bilinear or Catmull-Rom history.
C4  48 independent views of log-uniform resolution 320x180 .. 3840x2160.
C5  1920x1080, 64 frames (learned rectification workload).

Scenes are seeded analytic renders (include/taa_synth.h); nothing is loaded
from disk.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import taa_abi as T


def base_parameters(**over) -> T.Parameters:
    """The shared mode of every workload (the reference defaults otherwise, source/taa.hpp:31-76)."""
    p = T.default_parameters()
    p.mInterpolationMode = 2
    p.mUseYCoCg = 1
    p.mVarianceClipping = 1
    p.mVarClipGamma = 1.0
    p.mColorClampingOrClipping = 2
    p.mAlpha = 0.1
    p.mUseVelocityVectors = 2
    p.mVelocitySampleMode = 0
    for k, v in over.items():
        setattr(p, k, v)
    return p


@dataclass
class Workload:
    name: str
    width: int
    height: int
    frames: int
    seed: int
    num_spheres: int
    cam_v0: tuple = (3.0, 0.0)
    cam_accel: tuple = (0.0, 0.0)
    spin_max: float = 0.0
    radius: tuple = (20.0, 120.0)
    params: dict = field(default_factory=dict)
    sharpener: int = T.TAA_SHARPEN_OFF
    sharpen_factor: float = 0.5
    jitter_phase: int = 0

    def scene(self) -> T.SynthScene:
        s = T.synth_default_scene(self.width, self.height, self.seed)
        s.num_spheres = self.num_spheres
        s.cam_v0[0], s.cam_v0[1] = self.cam_v0
        s.cam_accel[0], s.cam_accel[1] = self.cam_accel
        s.spin_max = self.spin_max
        s.radius_min, s.radius_max = self.radius
        s.jitter_phase = self.jitter_phase
        return s

    def parameters(self) -> T.Parameters:
        return base_parameters(**self.params)

    @property
    def pixels(self) -> int:
        return self.width * self.height

    def bytes_per_pixel(self, history_bytes: int = 16, motion_bytes: int = 4) -> int:
        """Algorithmic bytes per pixel: every input and output once (colour 8,
        depth 4, motion, history in and out, screen 8, previous depth 4 when
        depth culling is on)."""
        b = 8 + 4 + motion_bytes + 2 * history_bytes + 8
        if self.params.get("mDepthCulling"):
            b += 4
        return b


def c1() -> Workload:
    return Workload("C1 1280x720x16 plain", 1280, 720, 16, seed=1, num_spheres=32)


def c2() -> Workload:
    return Workload("C2 3840x2160x64 depth+velocity rejection", 3840, 2160, 64, seed=2, num_spheres=128,
                    cam_v0=(2.0, 0.0), cam_accel=(38.0 / 63.0, 0.0),
                    params=dict(mDepthCulling=1, mRejectOutside=1))


def c3(interp: int = 2) -> Workload:
    return Workload("C3 2560x1440x32 TAA+CAS", 2560, 1440, 32, seed=3, num_spheres=32, spin_max=0.05,
                    params=dict(mInterpolationMode=interp), sharpener=T.TAA_SHARPEN_CAS, sharpen_factor=0.5)


def c5() -> Workload:
    return Workload("C5 1920x1080x64", 1920, 1080, 64, seed=5, num_spheres=32)


def c4_views(n: int = 48, base_seed: int = 400, frames: int = 32) -> list[Workload]:
    """48 views, log-uniform resolution 320x180 .. 3840x2160 (16:9), own seed,
    jitter phase, pan speed U[0,30] px/frame and 16..128 spheres."""
    import numpy as np
    rng = np.random.default_rng(base_seed)
    views = []
    for i in range(n):
        s = math.exp(rng.uniform(math.log(1.0), math.log(12.0)))
        w = max(16, int(round(320 * s / 8)) * 8)
        h = max(9, int(round(w * 9 / 16)))
        speed = rng.uniform(0.0, 30.0)
        ang = rng.uniform(0, 2 * math.pi)
        views.append(Workload(f"C4 view {i} {w}x{h}", w, h, frames, seed=base_seed + i,
                              num_spheres=int(rng.integers(16, 129)),
                              cam_v0=(speed * math.cos(ang), speed * math.sin(ang)), jitter_phase=i % 8))
    return views


def small(width: int, height: int, frames: int = 4, seed: int = 11, **kw) -> Workload:
    """A scaled-down scene for parity tests (sphere radii scaled to the image)."""
    r = max(2.0, min(width, height) / 6.0)
    return Workload(f"small {width}x{height}", width, height, frames, seed=seed,
                    num_spheres=kw.pop("num_spheres", 8), radius=(r * 0.3, r), **kw)
