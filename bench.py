#!/usr/bin/env python3
"""Benchmark of the TAA resolve on the 4K workload (C2: 3840x2160, 64 frames).

A step is one pass of the resolve over the whole 64-frame sequence (64
launches with ping-pong history).  `value` is Mpx/s with every input already
resident in HBM; `e2e` is the same metric through the C ABI with host
buffers: each frame's colour, depth and motion go host->device from pinned
memory and its screen result comes back device->host inside the timed region.
Every frame's inputs (500 MB at 4K) are larger than the 129 MB L2, so no L2
flush is needed between launches.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  Multi-GPU runs are independent replicas: the
sequence has a frame-to-frame dependence and does not shard.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for p in (ROOT / "taa-star_gb300", ROOT / "oracle"):
    sys.path.insert(0, str(p))

METRIC = "4K TAA resolve Mpx/s & HBM GB/s, plain vs FP16/batched on 1 GB300 @ PSNR≥50dB"
UNIT = "Mpx/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--frames", type=int, default=64)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-fxaa", action="store_true")
    ap.add_argument("--no-modes", action="store_true")
    ap.add_argument("--no-c3", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--isa-rates", action="store_true",
                    help="build and run the FMA issue-rate measurement (taa-star_gb300/csrc/isa_rates.cu; no JSON "
                         "benchmark line)")
    ap.add_argument("--profile", choices=["fast", "tiled", "fp16", "plain", "batch48", "fxaa", "fused", "defaults",
                                          "learned", "learned_tc", "up"],
                    help="a small case for ncu: a few launches of one form on 4K frames (no JSON line)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float, world: int, device=None) -> float:
    """The largest of the ranks' values: the slowest replica's time, which sets
    the whole job's throughput.  One rank returns its own value."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Whole-job throughput of `world` replicas that each processed
    `units_per_rank` units, timed by the slowest of them."""
    return world * units_per_rank / seconds_max


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(form_name: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None, None
    d = json.loads(p.read_text())
    e = d.get(form_name)
    if not e:
        return None, None
    return e.get("bytes_per_launch_at_4k"), e.get("source")


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                vals = [v.strip() for v in out.stdout.strip().split(",")]
                if len(vals) == 7:
                    self.samples.append(vals)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        import statistics
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


class NvmlClockSampler:
    """The same record as ClockSampler from NVML itself (libnvidia-ml, read-only
    queries), every 10 ms: the GPU is found by the CUDA device's PCI bus id, so
    a short timed region still gets a dozen samples.  make() falls back to
    ClockSampler where NVML cannot be loaded."""

    SM = 1  # NVML_CLOCK_SM
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, nvml, handle):
        self.nvml, self.handle = nvml, handle
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    @classmethod
    def make(cls, device: int):
        import ctypes
        import ctypes.util
        try:
            nvml = ctypes.CDLL("libnvidia-ml.so.1")
            rt = ctypes.CDLL(ctypes.util.find_library("cudart") or "libcudart.so")
            bus = ctypes.create_string_buffer(64)
            if rt.cudaDeviceGetPCIBusId(bus, 64, device) != 0 or nvml.nvmlInit_v2() != 0:
                raise OSError("no bus id or NVML")
            handle = ctypes.c_void_p()
            if nvml.nvmlDeviceGetHandleByPciBusId_v2(bus, ctypes.byref(handle)) != 0:
                raise OSError("no NVML handle")
            return cls(nvml, handle)
        except (OSError, AttributeError):
            return ClockSampler(device)

    def _run(self):
        import ctypes
        sm, mx, reasons = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        get_reasons = getattr(self.nvml, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nvml.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self._stop.is_set():
            if (self.nvml.nvmlDeviceGetClockInfo(self.handle, self.SM, ctypes.byref(sm)) == 0 and
                    self.nvml.nvmlDeviceGetMaxClockInfo(self.handle, self.SM, ctypes.byref(mx)) == 0 and
                    get_reasons(self.handle, ctypes.byref(reasons)) == 0):
                self.samples.append((sm.value, mx.value, reasons.value))
            self._stop.wait(0.01)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["NVML returned no sample"]}
        import statistics
        reasons = sorted({name for _, _, r in self.samples for bit, name in self.REASONS.items() if r & bit})
        return {"sm_mhz": statistics.median(s[0] for s in self.samples), "sm_max_mhz": max(s[1] for s in self.samples),
                "reasons": reasons, "samples": len(self.samples), "source": "NVML, every 10 ms"}


# ------------------------------------------------------------------ reference arm
# The reference's path on the host cores is the oracle's FP32 restatement of
# taa.comp (the shader itself needs Vulkan).  This arm builds its inputs from
# the oracle alone - scene, sphere table, jitter, parameter and uniform blocks
# (oracle/oracle.py) - so the library is never loaded in it.
C2_SCENE = dict(width=3840, height=2160, seed=2, num_spheres=128, cam_v0=(2.0, 0.0), cam_accel=(38.0 / 63.0, 0.0))
C2_NAME = "C2 3840x2160x64 depth+velocity rejection"


def c2_config(world: int) -> dict:
    """The workload both arms run (the same dict on both lines)."""
    return {"workload": C2_NAME, "width": 3840, "height": 2160, "frames": 64,
            "mode": "Catmull-Rom, YCoCg variance clip gamma 1, clip-fast, alpha 0.1, depth culling, reject outside",
            "history": "RGBA32F", "motion": "RG16F", "bytes_per_px": 60,
            "l2": "no flush: each frame's inputs (500 MB) exceed the 129 MB L2",
            "parallelism": f"replicas x{world}"}


def reference_c2():
    """The C2 workload (workloads.c2()) from the oracle's helpers: its scene and
    parameter block (Catmull-Rom, YCoCg variance clip gamma 1, clip-fast,
    alpha 0.1, velocity for every pixel, depth culling, reject outside)."""
    import oracle as O
    c = dict(C2_SCENE)
    sc = O.synth_scene(c.pop("width"), c.pop("height"), c.pop("seed"), **c)
    p = O.default_parameters()
    for k, v in dict(mInterpolationMode=2, mUseYCoCg=1, mVarianceClipping=1, mVarClipGamma=1.0,
                     mColorClampingOrClipping=2, mAlpha=0.1, mUseVelocityVectors=2, mVelocitySampleMode=0,
                     mDepthCulling=1, mRejectOutside=1).items():
        setattr(p, k, v)
    return sc, p


def cpu_frames_for_reference(sc, n):
    """Inputs of the first n+1 frames, rendered on the host by the FP64 scene evaluator."""
    import numpy as np
    import oracle as O
    sph = O.synth_spheres(sc)
    out = []
    for f in range(n + 1):
        r = O.synth_frame(sc, sph, f)
        out.append(dict(color=r["color"].astype(np.float16).astype(np.float32), depth=r["depth"].astype(np.float32),
                        motion=r["motion"][..., :2].astype(np.float16).astype(np.float32),
                        jitter=O.synth_jitter(sc, f)))
    return out


def time_oracle(params, frames, nthreads, budget_s, min_frames=1):
    """Oracle FP32 resolve over consecutive frames until the time budget is spent."""
    import numpy as np
    import oracle as O
    hist = frames[0]["color"].copy()
    done, t_total = 0, 0.0
    i = 1
    while done < min_frames or t_total < budget_s:
        f = frames[1 + (i - 1) % (len(frames) - 1)]
        prev = frames[(i - 1) % (len(frames) - 1)]
        u = O.make_uniforms(params, jitter_ndc=f["jitter"])
        t0 = time.perf_counter()
        r = O.resolve(u, f["color"], f["depth"], f["motion"], history=hist, history_depth=prev["depth"],
                      nthreads=nthreads)
        t_total += time.perf_counter() - t0
        hist = r["history"].astype(np.float32)
        done += 1
        i += 1
        if done >= 10000:
            break
    return done, t_total


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sc, params = reference_c2()
    n = os.cpu_count() or 1
    frames = cpu_frames_for_reference(sc, 2)
    # warm-up frames, then `steps` timed frames (one 4K frame per step)
    time_oracle(params, frames, n, 0.0, min_frames=max(1, args.warmup))
    done, t = time_oracle(params, frames, n, 0.0, min_frames=args.steps)
    mpx = sc.width * sc.height * done / t / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": mpx, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t / done * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded analytic scene, rendered on the host)",
        "config": c2_config(world), "frames_per_step": 1,
        "timing": "wall clock over a bounded sample: one of the sequence's 4K frames per step",
        "cpu_baseline": {"value": mpx, "unit": UNIT, "cores": n, "kind": "port",
                         "sample": f"{done} consecutive 3840x2160 frames of the C2 scene, FP32 oracle restatement of taa.comp, {n} threads"},
        "e2e": {"value": mpx, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ our arm
def time_learned(T, WL, dev, stream, sid, args):
    """The C5 configuration of the learned rectifier: records from four other
    seeds of the renderer (about 2M pixels, resolved with the plain variance
    clip), Adam on the library's tensor-core training kernels, then the 64-frame
    seed-5 sequence resolved by the plain variance clip and by the learned form,
    each against the renderer's 64-spp ground truth; and the cost per 1080p
    frame of each over that sequence replayed from a CUDA graph (CUDA events,
    5 replays after 3), beside the cost of one frame resolved 20 times."""
    import numpy as np
    import torch
    import learned_pipeline as LP

    tr = T.MlpTrainer(2_200_000)
    for s in (501, 502, 503, 504):
        LP.collect(tr, WL.Workload(f"C5 training seed {s}", 1920, 1080, 24, seed=s, num_spheres=32), 24, dev, 0.0125,
                   skip=4, seed=s)
    records = tr.count()
    steps, batch = 2000, 8192
    w, loss_first, loss_last = LP.train(tr, seed=1, steps=steps, batch=batch, lr=3e-3)
    tr.close()
    wl = WL.c5()
    fr = LP.render(wl, wl.frames, dev)
    ps, ls = {}, {}
    plain, plain_max = LP.evaluate(wl, wl.frames, dev, T.TAA_FORM_TILED, fr=fr, stats=ps)
    learned, learned_max = LP.evaluate(wl, wl.frames, dev, T.TAA_FORM_LEARNED, weights=w, fr=fr, stats=ls)
    H, W = wl.height, wl.width
    # the cost of each form on the C5 sequence itself: the 64 frames (history chained, each
    # frame's inputs read once) captured in a CUDA graph, replayed as the 4K forms are; and on
    # one frame resolved 20 times in a row (its 124 MB of inputs stay in the 129 MB L2)
    cost, cost_one = {}, {}
    uni = [T.make_uniforms(wl.parameters(), jitter_ndc=fr.jitter[f], mResetHistory=1 if f == 0 else 0)
           for f in range(wl.frames)]
    for name, form in (("tiled", T.TAA_FORM_TILED), ("fast", T.TAA_FORM_FAST), ("learned", T.TAA_FORM_LEARNED)):
        ctx = T.Taa(W, H, form=form)
        if form == T.TAA_FORM_LEARNED:
            ctx.set_mlp(w)
        h = [torch.zeros(H, W, 4, device=dev) for _ in range(2)]
        gs = torch.cuda.Stream(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=gs):
            for f in range(wl.frames):
                ctx.set_uniforms(uni[f])
                ctx.resolve(stream=gs.cuda_stream, color=fr.color[f], depth=fr.depth[f], velocity=fr.motion[f],
                            history=h[f & 1], history_depth=fr.depth[f - 1] if f else fr.depth[0],
                            history_out=h[(f + 1) & 1])
        for _ in range(3):
            graph.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(5):
            graph.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        cost[name] = e0.elapsed_time(e1) * 1000 / (5 * wl.frames)
        del graph
        ctx.set_uniforms(uni[5])
        b = dict(color=fr.color[5], depth=fr.depth[5], velocity=fr.motion[5], history=h[0],
                 history_depth=fr.depth[4], history_out=h[1])
        for _ in range(3):
            ctx.resolve(stream=sid, **b)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(20):
            ctx.resolve(stream=sid, **b)
        e1.record(stream)
        torch.cuda.synchronize()
        cost_one[name] = e0.elapsed_time(e1) * 1000 / 20
        ctx.close()
    return {"mpx_s": W * H / cost["learned"], "us_per_frame_1080p": cost["learned"],
            "plain_variance_clip_us_per_frame_1080p": cost["tiled"], "cost_vs_plain": cost["learned"] / cost["tiled"],
            "fast_variance_clip_us_per_frame_1080p": cost["fast"], "cost_vs_fast": cost["learned"] / cost["fast"],
            "cost_timing": "the 64-frame C5 sequence from a CUDA graph (5 replays after 3)",
            "one_frame_us": cost_one, "one_frame_cost_vs_plain": cost_one["learned"] / cost_one["tiled"],
            "psnr_db_vs_64spp": float(np.mean(learned)), "plain_psnr_db_vs_64spp": float(np.mean(plain)),
            "gain_db": float(np.mean(learned) - np.mean(plain)), "max_abs_err": learned_max,
            "plain_max_abs_err": plain_max,
            "q9999_abs_err": float(np.median(ls["q9999"])), "plain_q9999_abs_err": float(np.median(ps["q9999"])),
            "frames_q9999_below_plain": int(np.sum(np.array(ls["q9999"]) < np.array(ps["q9999"]))),
            "training": {"records": records, "steps": steps, "batch": batch, "loss_first": loss_first,
                         "loss_last": loss_last, "seeds": [501, 502, 503, 504],
                         "deterministic": "records in key order, gradient sums added in CTA order"},
            "evaluation": f"{wl.name}, seed {wl.seed}, frames 8..{wl.frames - 1}, PSNR of the RGB history "
                          "against the 64-spp truth, peak = the frame's largest truth value"}


def time_fxaa(T, WL, dev, stream, sid, args, peak, col, dep, mot, uniforms):
    """The FXAA pass of the ray-trace-assist path at 4K: a plain-form resolve of
    C2 frame 2 with the segmentation mask (RT-augment tests OUT, DIS, NRM, DPT,
    MID, LUM and the FXAA flag) gives the result image and the mask; taa_fxaa
    then runs on them, on the mask and with every pixel marked (NULL mask).
    Four buffer sets rotate (660 MB), so no launch finds its inputs in the
    129 MB L2.  Algorithmic bytes: 8 (result) + 4 (mask) + 8 (output) per pixel,
    16 without a mask; the reference's prepare + FXAA dispatches move 36."""
    import numpy as np
    import torch
    import oracle as O

    H, W = col.shape[1], col.shape[2]
    u = T.Uniforms()
    ctypes_copy(u, uniforms[2])
    for i in range(2):
        u.param[i].mRayTraceAugment = 1
        u.param[i].mRayTraceAugmentFlags = 0x3F | 0x200
    ctx = T.Taa(W, H, form=T.TAA_FORM_PLAIN)
    ctx.set_uniforms(u)
    sets = 4
    res = [torch.empty(H, W, 4, dtype=torch.float16, device=dev) for _ in range(sets)]
    seg = [torch.empty(H, W, dtype=torch.int32, device=dev) for _ in range(sets)]
    out = [torch.empty(H, W, 4, dtype=torch.float16, device=dev) for _ in range(sets)]
    h0 = col[1].float()
    ctx.resolve(stream=sid, color=col[2], depth=dep[2], velocity=mot[2], history=h0, history_depth=dep[1],
                history_out=torch.empty(H, W, 4, device=dev), result=res[0], segmask=seg[0])
    for i in range(1, sets):
        res[i].copy_(res[0])
        seg[i].copy_(seg[0])
    torch.cuda.synchronize()
    ctx.close()
    marked = float(((seg[0] & 3) == 1).float().mean().item())
    result = {}
    k = max(8, args.steps * 4)
    fctx = T.Taa(W, H, form=T.TAA_FORM_PLAIN, flags=T.TAA_FLAG_FXAA)  # lends the pass its work list
    for name, use_mask, c in (("segmask", True, fctx), ("segmask_without_list", True, None),
                              ("all_pixels", False, None)):
        for i in range(3 * sets):
            T.fxaa(res[i % sets], out[i % sets], seg[i % sets] if use_mask else None, stream=sid, ctx=c)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(k):
            T.fxaa(res[i % sets], out[i % sets], seg[i % sets] if use_mask else None, stream=sid, ctx=c)
        e1.record(stream)
        torch.cuda.synchronize()
        us = e0.elapsed_time(e1) * 1000 / k
        bpp = 20 if use_mask else 16
        gbs = bpp * W * H / (us / 1e6) / 1e9
        result[name] = {"us_per_frame": us, "mpx_s": W * H / us, "bytes_per_px": bpp, "gb_s": gbs,
                        "frac_of_hbm": gbs / peak}
    result["marked_fraction"] = marked
    # the oracle on the same frame and mask (the checker, timed as the CPU reference)
    img = res[0].float().cpu().numpy()
    m = seg[0].cpu().numpy().view(np.uint32)
    nthr = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = O.fxaa(img, m, nthreads=nthr)
    t = time.perf_counter() - t0
    T.fxaa(res[0], out[0], seg[0], stream=sid, ctx=fctx)
    torch.cuda.synchronize()
    got = out[0].float().cpu().numpy()
    fctx.close()
    q = ref.astype(np.float32).astype(np.float16).astype(np.float32)
    result["cpu_oracle"] = {"mpx_s": W * H / t / 1e6, "threads": nthr}
    result["pixels_equal_to_oracle"] = float(np.mean(np.all(got == q, axis=-1)))
    return result


def time_modes(T, WL, dev, stream, sid, args, peak):
    """The resolve modes outside the benchmark mode: the ray-trace-assist
    classification writing the segmentation mask (every test, history count 8)
    TAAU upsampling (1920x1080 source, 3840x2160 target), a debug output
    (mode 2) and the reference's default parameter block, each in the form
    AUTO selects (recorded per entry: the fast form for TAAU and the default
    block, the tiled form for the others) and in the plain form (one thread
    per pixel).  Each on four rotating frames of the
    C2 scene (every frame's bindings exceed the L2), CUDA events over 12
    launches after 3.  Material ids and uv/normals are seeded synthetic blocks
    (48 px materials, 8 px normals).  Last the post-process pass at 4K (split,
    debug image on the left, zoom inset), 24 launches after 3."""
    import math
    import torch

    out = {}

    def frames(wl, n):
        sc = wl.scene()
        H, W = wl.height, wl.width
        col = [torch.empty(H, W, 4, dtype=torch.float16, device=dev) for _ in range(n)]
        dep = [torch.empty(H, W, dtype=torch.float32, device=dev) for _ in range(n)]
        mot = [torch.empty(H, W, 2, dtype=torch.float16, device=dev) for _ in range(n)]
        for f in range(n):
            T.synth_render(sc, f, stream=sid, color=col[f], depth=dep[f], motion=mot[f])
        return sc, col, dep, mot

    def run(name, ctx, ulist, binds, bpp, px):
        ctx.set_uniforms(ulist[0])
        form = {T.TAA_FORM_PLAIN: "plain", T.TAA_FORM_TILED: "tiled", T.TAA_FORM_FP16: "fp16",
                    T.TAA_FORM_FAST: "fast"}[ctx.selected_form()]
        for i in range(3):
            ctx.set_uniforms(ulist[i % len(ulist)])
            ctx.resolve(stream=sid, **binds(i))
        torch.cuda.synchronize()
        k = 12
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(k):
            ctx.set_uniforms(ulist[i % len(ulist)])
            ctx.resolve(stream=sid, **binds(i))
        e1.record(stream)
        torch.cuda.synchronize()
        us = e0.elapsed_time(e1) * 1000 / k
        gbs = bpp * px / (us / 1e6) / 1e9
        out[name] = {"us_per_frame": us, "mpx_s": px / us, "bytes_per_px": bpp, "gb_s": gbs, "frac_of_hbm": gbs / peak,
                     "form": form}

    n = 4
    wl = WL.c2()
    H, W = wl.height, wl.width
    sc, col, dep, mot = frames(wl, n + 1)
    hist = [torch.zeros(H, W, 4, device=dev) for _ in range(2)]
    res = torch.empty(H, W, 4, dtype=torch.float16, device=dev)
    yy = torch.arange(H, device=dev, dtype=torch.int32).view(H, 1)
    xx = torch.arange(W, device=dev, dtype=torch.int32).view(1, W)
    mat = ((yy // 48) * 977 + (xx // 48) * 131) % 61 + 1
    pmat = torch.roll(mat, 1, dims=1).contiguous()
    g = torch.Generator(device=dev).manual_seed(7)
    blk = torch.rand(H // 8 + 1, W // 8 + 1, 4, device=dev, generator=g)
    uvn = blk.repeat_interleave(8, 0).repeat_interleave(8, 1)[:H, :W].contiguous()
    uvn[..., 2] *= 2 * math.pi
    uvn[..., 3] = uvn[..., 3] * 3.0 - 1.5
    seg = [torch.zeros(H, W, dtype=torch.int32, device=dev) for _ in range(2)]

    def base(i):
        f = 1 + i % n
        return dict(color=col[f], depth=dep[f], velocity=mot[f], history=hist[i & 1], history_depth=dep[f - 1],
                    history_out=hist[(i + 1) & 1], result=res)

    def u_for(f, **over):
        p = wl.parameters()
        for k_, v_ in over.items():
            setattr(p, k_, v_)
        return T.make_uniforms(p, jitter_ndc=T.synth_jitter(sc, f)[1])

    rt = [u_for(1 + i, mRayTraceAugment=1, mRayTraceAugmentFlags=0x7F, mRayTraceHistoryCount=8) for i in range(n)]
    rt_binds = lambda i: dict(base(i), material=mat, prev_material=pmat, uvnrm=uvn, prev_segmask=seg[i & 1],
                              segmask=seg[(i + 1) & 1])
    rt_bpp = wl.bytes_per_pixel(16, 4) + 4 + 4 + 16 + 4 + 4
    ctx = T.Taa(W, H)
    run("rt_augment_segmask", ctx, rt, rt_binds, rt_bpp, W * H)
    ctx.close()
    ctx = T.Taa(W, H, form=T.TAA_FORM_PLAIN)
    run("rt_augment_segmask_plain", ctx, rt, rt_binds, rt_bpp, W * H)
    dbg = torch.empty(H, W, 4, dtype=torch.float16, device=dev)
    dm = [u_for(1 + i, mDebugMode=2, mDebugScale=1.0) for i in range(n)]
    run("debug_output_plain", ctx, dm, lambda i: dict(base(i), debug=dbg), wl.bytes_per_pixel(16, 4) + 8, W * H)
    ctx.close()
    # with a debug binding the default form runs the tiled FP32 form (taa_selected_form
    # answers for calls without one, so the form is recorded by hand)
    ctx = T.Taa(W, H)
    run("debug_output", ctx, dm, lambda i: dict(base(i), debug=dbg), wl.bytes_per_pixel(16, 4) + 8, W * H)
    out["debug_output"]["form"] = "tiled"
    ctx.close()
    # the reference's default parameter block (taa.hpp:31-76: min/max clamp, bilinear
    # history, velocity for movers only, no depth culling) on the same frames: AUTO runs
    # it in the tiled form's general path (no benchmark-mode specialisation)
    defaults = [T.make_uniforms(T.default_parameters(), jitter_ndc=T.synth_jitter(sc, 1 + i)[1]) for i in range(n)]
    ctx = T.Taa(W, H)
    run("reference_defaults", ctx, defaults, base, wl.bytes_per_pixel(16, 4) - 4, W * H)
    ctx.close()
    ctx = T.Taa(W, H, form=T.TAA_FORM_PLAIN)
    run("reference_defaults_plain", ctx, defaults, base, wl.bytes_per_pixel(16, 4) - 4, W * H)
    ctx.close()
    del col, dep, mot, seg, mat, pmat, uvn, dbg

    # TAAU: a 1920x1080 rendering of the same scene resolved into 3840x2160
    lo = WL.Workload("C2 scene at 1920x1080", 1920, 1080, n + 1, seed=wl.seed, num_spheres=wl.num_spheres,
                     cam_v0=(1.0, 0.0), cam_accel=(19.0 / 63.0, 0.0), radius=(10.0, 60.0), params=dict(wl.params))
    sc, col, dep, mot = frames(lo, n + 1)
    up = [T.make_uniforms(lo.parameters(), jitter_ndc=T.synth_jitter(sc, 1 + i)[1], mUpsampling=1) for i in range(n)]
    # per target pixel history in/out 16 + 16 and screen 8; per source pixel colour 8, depth 4, motion 4, previous depth 4
    up_bpp = 40 + 20 * (lo.width * lo.height) / (W * H)
    for name, form in (("upsample_2x", T.TAA_FORM_AUTO), ("upsample_2x_tiled", T.TAA_FORM_TILED),
                       ("upsample_2x_plain", T.TAA_FORM_PLAIN)):
        ctx = T.Taa(lo.width, lo.height, W, H, form=form)
        run(name, ctx, up, base, up_bpp, W * H)
        out[name]["source"] = [lo.width, lo.height]
        ctx.close()
    # the post-process pass at 4K: split at W / 2, the left side shows the debug
    # image with its alpha, the zoom inset drawn; 16 B/px (8 read from the input
    # or the debug image, 8 written); four rotating buffer sets (800 MB)
    pp = T.post_process_default_params(W, H)
    pp.zoom, pp.split_x, pp.debug_l_show = 1, W // 2, 1
    pp.debug_l_mask[3] = 1.0
    g2 = torch.Generator(device=dev).manual_seed(11)
    srcs = [torch.rand(H, W, 4, device=dev, generator=g2).half() for _ in range(n)]
    dbgs = [torch.rand(H, W, 4, device=dev, generator=g2).half() for _ in range(n)]
    outs = [torch.empty(H, W, 4, dtype=torch.float16, device=dev) for _ in range(n)]
    for i in range(3):
        T.post_process(srcs[i % n], outs[i % n], pp, debug=dbgs[i % n], stream=sid)
    torch.cuda.synchronize()
    k = 24
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(k):
        T.post_process(srcs[i % n], outs[i % n], pp, debug=dbgs[i % n], stream=sid)
    e1.record(stream)
    torch.cuda.synchronize()
    us = e0.elapsed_time(e1) * 1000 / k
    gbs = 16 * W * H / (us / 1e6) / 1e9
    out["post_process"] = {"us_per_frame": us, "mpx_s": W * H / us, "bytes_per_px": 16, "gb_s": gbs,
                           "frac_of_hbm": gbs / peak, "form": "post_process_kernel"}
    del srcs, dbgs, outs
    return out


def time_c3(T, WL, dev, stream, sid, args, peak):
    """The resolve with a CAS sharpener (strength 0.5) on the C3 sequence
    (2560x1440, 32 frames, spinning spheres), bilinear and Catmull-Rom history.
    Per history filter and form: the resolve followed by the sharpen pass on
    its RGBA16F result (the library's default, and the reference's structure
    of two dispatches, taa.hpp:1027 and 1111-1139) in the FP16, fast FP32,
    exact tiled FP32 and plain forms, and the fast and exact forms' single
    launch that resolves each tile with a 1-pixel ring and sharpens it from
    shared memory (TAA_FLAG_FUSED_SHARPEN); last the fast resolve alone
    (result image, no sharpener), which prices the sharpen pass.  A step is the 32-frame sequence; 1 warm-up
    step, 3 timed.  Bytes per pixel: 56 for one launch (colour 8, depth 4,
    motion 4, history 16 + 16, sharpened 8); two add the result image, written
    and read back (72)."""
    import torch

    out = {}
    for interp, iname in ((2, "catmull_rom"), (0, "bilinear")):
        wl = WL.c3(interp)
        H, W, F = wl.height, wl.width, wl.frames
        sc = wl.scene()
        col = torch.empty(F, H, W, 4, dtype=torch.float16, device=dev)
        dep = torch.empty(F, H, W, dtype=torch.float32, device=dev)
        mot = torch.empty(F, H, W, 2, dtype=torch.float16, device=dev)
        for f in range(F):
            T.synth_render(sc, f, stream=sid, color=col[f], depth=dep[f], motion=mot[f])
        ul = [T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(sc, f)[1],
                              mResetHistory=1 if f == 0 else 0) for f in range(F)]
        hist = [torch.zeros(H, W, 4, dtype=torch.float32, device=dev) for _ in range(2)]
        shp = torch.empty(H, W, 4, dtype=torch.float16, device=dev)
        torch.cuda.synchronize()

        def seq(ctx):
            sharp = ctx.desc.sharpener != T.TAA_SHARPEN_OFF
            for f in range(F):
                ctx.set_uniforms(ul[f])
                out_img = dict(sharpened=shp) if sharp else dict(result=shp)
                ctx.resolve(stream=sid, color=col[f], depth=dep[f], velocity=mot[f], history=hist[f & 1],
                            history_depth=dep[f - 1] if f else dep[0], history_out=hist[(f + 1) & 1], **out_img)

        cas = dict(sharpener=T.TAA_SHARPEN_CAS, sharpen_factor=0.5)
        fused = T.TAA_FLAG_FUSED_SHARPEN
        variants = (("fp16_then_cas", dict(form=T.TAA_FORM_FP16, **cas), 72),
                    ("fast_then_cas", dict(form=T.TAA_FORM_AUTO, **cas), 72),
                    ("fast_fused_cas", dict(form=T.TAA_FORM_AUTO, flags=fused, **cas), 56),
                    ("tiled_exact_then_cas", dict(form=T.TAA_FORM_TILED, **cas), 72),
                    ("tiled_exact_fused_cas", dict(form=T.TAA_FORM_TILED, flags=fused, **cas), 56),
                    ("plain_then_cas", dict(form=T.TAA_FORM_PLAIN, **cas), 72),
                    ("fast_no_sharpener", dict(form=T.TAA_FORM_AUTO), 56))
        res_i = {}
        for name, kw, bpp in variants:
            ctx = T.Taa(W, H, **kw)
            ctx.set_uniforms(ul[1])
            form = {T.TAA_FORM_PLAIN: "plain", T.TAA_FORM_TILED: "tiled", T.TAA_FORM_FP16: "fp16",
                    T.TAA_FORM_FAST: "fast"}[ctx.selected_form()]
            seq(ctx)
            torch.cuda.synchronize()
            k = 3
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(k):
                seq(ctx)
            e1.record(stream)
            torch.cuda.synchronize()
            us = e0.elapsed_time(e1) * 1000 / (k * F)
            gbs = bpp * W * H / (us / 1e6) / 1e9
            res_i[name] = {"us_per_frame": us, "mpx_s": W * H / us, "bytes_per_px": bpp, "gb_s": gbs,
                           "frac_of_hbm": gbs / peak, "resolve_form": form}
            ctx.close()
        out[iname] = res_i
        del col, dep, mot, hist, shp
    out["workload"] = "C3 2560x1440, 32 frames, CAS 0.5"
    return out


def ctypes_copy(dst, src):
    import ctypes as C
    C.memmove(C.addressof(dst), C.addressof(src), C.sizeof(dst))


def time_batch(T, WL, dev, stream, sid, world, args, peak, single_mpx):
    """48 views of the C4 sizes resolved by one batched launch per step; the
    batch is autotuned first (tile shape, job order, grid).  Returns its Mpx/s,
    GB/s and the per-pixel ratio to the single-4K number."""
    import torch
    import torch.distributed as dist

    views = WL.c4_views()
    npx = sum(v.width * v.height for v in views)
    bufs = []
    for v in views:
        sc, w, h = v.scene(), v.width, v.height
        col = [torch.empty(h, w, 4, dtype=torch.float16, device=dev) for _ in range(2)]
        dep = [torch.empty(h, w, dtype=torch.float32, device=dev) for _ in range(2)]
        mot = [torch.empty(h, w, 2, dtype=torch.float16, device=dev) for _ in range(2)]
        for f in range(2):
            T.synth_render(sc, f, stream=sid, color=col[f], depth=dep[f], motion=mot[f])
        u = T.make_uniforms(v.parameters(), jitter_ndc=T.synth_jitter(sc, 1)[1])
        bufs.append(dict(u=u, b=dict(color=col[1], depth=dep[1], velocity=mot[1], history=col[0].float(),
                                     history_depth=dep[0], history_out=torch.empty(h, w, 4, device=dev),
                                     result=torch.empty(h, w, 4, dtype=torch.float16, device=dev))))
    torch.cuda.synchronize()
    batch = T.Batch([(v.width, v.height) for v in views])
    for i, b in enumerate(bufs):
        batch.set_uniforms(i, b["u"])
    batch.prepare(0, [b["b"] for b in bufs], stream=sid)
    best = batch.autotune(0, reps=3, stream=sid)
    # the launch captured in a CUDA graph and replayed, as the configuration specifies
    gs = torch.cuda.Stream(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=gs):
        batch.launch(0, stream=torch.cuda.current_stream(dev).cuda_stream)
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    k = max(3, args.steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(k):
        graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
    batch.close()
    mpx = job_throughput(npx * k, world, ms / 1e3) / 1e6
    gbs = views[0].bytes_per_pixel(history_bytes=16, motion_bytes=4) * npx / (ms / 1e3 / k) / 1e9
    return {"mpx_s": mpx, "gb_s": gbs, "frac_of_hbm": gbs / peak, "views": len(views), "pixels": npx,
            "per_pixel_vs_single_4k": (mpx / world) / single_mpx,
            "tuning": {"tile": [best.tile_w, best.tile_h], "schedule": best.schedule,
                       "body": "fast strips" if best.form == T.TAA_FORM_FAST else "exact tiles",
                       "grid": "one CTA per tile" if best.ctas_per_sm == T.TAA_BATCH_CTA_PER_TILE else "persistent"},
            "launches_per_step": 1, "timed": "CUDA graph replay"}


def summarize(form_name, mpx, frac, forms, e2e, cpu):
    """The numbers behind every target in a few flat keys, printed last so that
    a truncated tail of the line still carries them."""
    f = forms or {}
    g = lambda k, field="mpx_s": (f.get(k) or {}).get(field)
    tiled = g("tiled") if form_name != "tiled" else mpx
    out = {"form": form_name, "mpx_s": mpx, "frac_of_hbm": frac, "tiled_exact_mpx_s": tiled,
           "plain_mpx_s": g("plain"), "fp16_mpx_s": g("fp16"), "fp16_guarded_mpx_s": g("fp16_guarded")}
    if tiled:
        out["value_vs_tiled"] = mpx / tiled
        for k in ("fp16", "fp16_guarded"):
            if g(k):
                out[f"{k}_vs_tiled"] = g(k) / tiled
    if g("plain"):
        out["value_vs_plain"] = mpx / g("plain")
    if g("fast_rgba16f_history"):
        out["fast_rgba16f_history_mpx_s"] = g("fast_rgba16f_history")
    m = (f.get("modes") or {}).get("reference_defaults")
    if m:
        out["reference_defaults_us"] = m["us_per_frame"]
        out["reference_defaults_form"] = m["form"]
    b = f.get("batch48")
    if b:
        out["batch48_mpx_s"] = b["mpx_s"]
        out["batch48_per_pixel_vs_single"] = b["per_pixel_vs_single_4k"]
    ln = f.get("learned")
    if ln:
        out.update(learned_cost_vs_plain=ln["cost_vs_plain"], learned_cost_vs_fast=ln.get("cost_vs_fast"),
                   learned_gain_db=ln["gain_db"],
                   learned_max_abs_err=ln["max_abs_err"], plain_max_abs_err=ln["plain_max_abs_err"],
                   learned_q9999_abs_err=ln.get("q9999_abs_err"), plain_q9999_abs_err=ln.get("plain_q9999_abs_err"))
    c3 = f.get("c3_cas")
    if c3:
        for interp, entries in c3.items():
            if isinstance(entries, dict):
                us = {k: v["us_per_frame"] for k, v in entries.items() if isinstance(v, dict) and "us_per_frame" in v}
                if us:
                    out[f"c3_{interp}_us"] = us
    if e2e:
        out["e2e_mpx_s"] = e2e["value"]
    if cpu:
        out["cpu_mpx_s"] = cpu["value"]
    return out


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    if rank == 0 or world == 1:
        from importlib import util
        spec = util.spec_from_file_location("taa_lib_build", ROOT / "taa-star_gb300" / "build.py")
        m = util.module_from_spec(spec)
        spec.loader.exec_module(m)
        m.build_library()
    if world > 1:
        dist.barrier()

    import taa_abi as T
    import workloads as WL

    wl = WL.c2()
    F = args.frames
    H, W = wl.height, wl.width
    sc = wl.scene()
    stream = torch.cuda.current_stream(dev)
    sid = stream.cuda_stream

    # inputs of the whole sequence, resident in HBM
    col = torch.empty(F, H, W, 4, dtype=torch.float16, device=dev)
    dep = torch.empty(F, H, W, dtype=torch.float32, device=dev)
    mot = torch.empty(F, H, W, 2, dtype=torch.float16, device=dev)
    for f in range(F):
        T.synth_render(sc, f, stream=sid, color=col[f], depth=dep[f], motion=mot[f])
    uniforms = []
    for f in range(F):
        uniforms.append(T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(sc, f)[1],
                                        mResetHistory=1 if f == 0 else 0))
    hist = [torch.zeros(H, W, 4, dtype=torch.float32, device=dev) for _ in range(2)]
    res = torch.empty(H, W, 4, dtype=torch.float16, device=dev)
    torch.cuda.synchronize()
    # the end-to-end run's pinned host images, taken while the process is young
    if not args.no_e2e:
        h_col = col.cpu().pin_memory()
        h_dep = dep.cpu().pin_memory()
        h_mot = mot.cpu().pin_memory()
        h_out = torch.empty(F, H, W, 4, dtype=torch.float16).pin_memory()

    def make_ctx(form, flags=0):
        c = T.Taa(W, H, form=form, flags=flags)
        c.set_uniforms(uniforms[1])
        return c

    def sequence(ctx, s=sid):
        for f in range(F):
            ctx.set_uniforms(uniforms[f])
            ctx.resolve(stream=s, color=col[f], depth=dep[f], velocity=mot[f], history=hist[f & 1],
                        history_depth=dep[f - 1] if f else dep[0], history_out=hist[(f + 1) & 1], result=res)

    def timed(ctx, steps, warmup, sampler=None):
        """A step is the 64-frame sequence, captured once in a CUDA graph and
        replayed (the launches a renderer would record per frame, without the
        host's per-launch cost)."""
        gs = torch.cuda.Stream(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=gs):
            sequence(ctx, gs.cuda_stream)
        for _ in range(warmup):
            graph.replay()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if sampler:
            sampler.__enter__()
        e0.record(stream)
        for _ in range(steps):
            graph.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        if sampler:
            sampler.__exit__(None, None, None)
        del graph
        ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
        if world > 1:
            dist.barrier()
        return ms

    bpp = wl.bytes_per_pixel(history_bytes=16, motion_bytes=4)
    launch_bytes = bpp * W * H
    peak, peak_kind = load_peaks()

    ctx = make_ctx(T.TAA_FORM_AUTO)
    form_used = ctx.selected_form()
    form_name = {1: "plain", 2: "tiled", 3: "fp16", 5: "fast"}[form_used]
    sampler = NvmlClockSampler.make(local)
    ms = timed(ctx, args.steps, args.warmup, sampler)
    launches = args.steps * F
    mpx = job_throughput(W * H * F * args.steps, world, ms / 1e3) / 1e6
    avg_launch_s = ms / 1e3 / launches
    achieved = launch_bytes / avg_launch_s / 1e9
    traffic, traffic_src = load_traffic(form_name)

    # end to end right after the headline (the rest of the run allocates much more: placed
    # after it, the same measurement gave 5 Gpx/s; here 11.2-12.4, the host link's rate)
    e2e = None
    if not args.no_e2e:
        nbuf = 3
        d_col = [torch.empty(H, W, 4, dtype=torch.float16, device=dev) for _ in range(nbuf)]
        d_dep = [torch.empty(H, W, dtype=torch.float32, device=dev) for _ in range(nbuf)]
        d_mot = [torch.empty(H, W, 2, dtype=torch.float16, device=dev) for _ in range(nbuf)]
        s_in = torch.cuda.Stream(dev)
        ectx = make_ctx(T.TAA_FORM_AUTO)
        in_ready = [torch.cuda.Event() for _ in range(nbuf)]
        done_ev = [torch.cuda.Event() for _ in range(nbuf)]

        def e2e_sequence():
            for f in range(F):
                b = f % nbuf
                with torch.cuda.stream(s_in):
                    # slot b last held frame f-3's inputs and was frame f-2's history depth
                    s_in.wait_event(done_ev[(f - 2) % nbuf])
                    d_col[b].copy_(h_col[f], non_blocking=True)
                    d_dep[b].copy_(h_dep[f], non_blocking=True)
                    d_mot[b].copy_(h_mot[f], non_blocking=True)
                    in_ready[b].record(s_in)
                stream.wait_event(in_ready[b])
                ectx.set_uniforms(uniforms[f])
                pb = (f - 1) % nbuf
                # the result binding is the frame's pinned host image: the resolve's
                # stores cross the host link themselves (no device image, no copy)
                ectx.resolve(stream=sid, color=d_col[b], depth=d_dep[b], velocity=d_mot[b], history=hist[f & 1],
                             history_depth=d_dep[pb] if f else d_dep[b], history_out=hist[(f + 1) & 1],
                             result=h_out[f])
                done_ev[b].record(stream)

        for ev in done_ev:
            ev.record(stream)
        e2e_sequence()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        # the host link is shared with the machine's other GPUs: five timed runs, the median reported
        k = max(2, args.steps // 4)
        runs = []
        for _ in range(5):
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(s_in)
            s_in.wait_stream(stream)
            for _ in range(k):
                e2e_sequence()
            stream.wait_stream(s_in)
            t1.record(stream)
            torch.cuda.synchronize()
            ms_e = max_over_ranks(t0.elapsed_time(t1), world, dev)
            runs.append(job_throughput(W * H * F * k, world, ms_e / 1e3) / 1e6)
        e2e = {"value": sorted(runs)[len(runs) // 2], "unit": UNIT,
               "h2d_bytes_per_step": F * H * W * (8 + 4 + 4), "d2h_bytes_per_step": F * H * W * 8,
               "runs": runs,
               "note": f"median of {len(runs)} runs of {k} steps; pinned host buffers; inputs copied 3 slots ahead on a "
                       "copy stream; the resolve stores its RGBA16F result straight into the frame's pinned "
                       "host image"}
        # the last frame's result against the same frame resolved into device memory
        ref = torch.empty(H, W, 4, dtype=torch.float16, device=dev)
        ectx.set_uniforms(uniforms[F - 1])
        hist_chk = hist[F & 1].clone()
        ectx.resolve(stream=sid, color=d_col[(F - 1) % nbuf], depth=d_dep[(F - 1) % nbuf],
                     velocity=d_mot[(F - 1) % nbuf], history=hist[(F - 1) & 1], history_depth=d_dep[(F - 2) % nbuf],
                     history_out=hist_chk, result=ref)
        torch.cuda.synchronize()
        e2e["result_matches_device_resolve"] = bool(torch.equal(ref.cpu(), h_out[F - 1]))
        ectx.close()


    forms = {form_name: {"mpx_s": mpx, "gb_s": achieved, "frac_of_hbm": achieved / peak}}
    if not args.no_forms:
        for fid, name, fl in ((T.TAA_FORM_TILED, "tiled", 0), (T.TAA_FORM_PLAIN, "plain", 0),
                              (T.TAA_FORM_FP16, "fp16", 0), (T.TAA_FORM_FP16, "fp16_guarded", T.TAA_FLAG_FP16_GUARD)):
            if name in forms:
                continue
            c2 = make_ctx(fid, fl)
            k = max(2, args.steps // 4)
            m2 = timed(c2, k, 1)
            v = job_throughput(W * H * F * k, world, m2 / 1e3) / 1e6
            g = launch_bytes / (m2 / 1e3 / (k * F)) / 1e9
            forms[name] = {"mpx_s": v, "gb_s": g, "frac_of_hbm": g / peak}
            c2.close()
        # RGBA16F history (the reference's storage format) in the fast form: 44 B/px
        hist16 = [torch.zeros(H, W, 4, dtype=torch.float16, device=dev) for _ in range(2)]
        c2 = T.Taa(W, H, form=T.TAA_FORM_AUTO, history_format=T.TAA_HISTORY_RGBA16F)
        gs = torch.cuda.Stream(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=gs):
            for f in range(F):
                c2.set_uniforms(uniforms[f])
                c2.resolve(stream=gs.cuda_stream, color=col[f], depth=dep[f], velocity=mot[f], history=hist16[f & 1],
                           history_depth=dep[f - 1] if f else dep[0], history_out=hist16[(f + 1) & 1], result=res)
        graph.replay()
        torch.cuda.synchronize()
        k = max(2, args.steps // 4)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            graph.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        m2 = max_over_ranks(e0.elapsed_time(e1), world, dev)
        b16 = bpp - 16
        v = job_throughput(W * H * F * k, world, m2 / 1e3) / 1e6
        g = b16 * W * H / (m2 / 1e3 / (k * F)) / 1e9
        forms["fast_rgba16f_history"] = {"mpx_s": v, "gb_s": g, "frac_of_hbm": g / peak, "bytes_per_px": b16,
                                         "form": {5: "fast", 2: "tiled"}.get(c2.selected_form(), "other")}
        c2.close()
        del graph, hist16

    # the 48-view batch (C4 sizes, log-uniform 320x180 .. 3840x2160): one launch per step
    if not args.no_batch:
        forms["batch48"] = time_batch(T, WL, dev, stream, sid, world, args, peak, mpx / world)

    # the ray-trace-assist classification (tiled and plain), TAAU and debug output (plain form), post-process
    if not args.no_modes and rank == 0:
        forms["modes"] = time_modes(T, WL, dev, stream, sid, args, peak)

    # the resolve with the CAS sharpener (C3: 2560x1440), one pass against two dispatches
    if not args.no_c3 and rank == 0:
        forms["c3_cas"] = time_c3(T, WL, dev, stream, sid, args, peak)

    # the FXAA pass on the segmentation mask (ray-trace-assist path) at 4K
    if not args.no_fxaa and rank == 0:
        forms["fxaa"] = time_fxaa(T, WL, dev, stream, sid, args, peak, col, dep, mot, uniforms)

    # the learned rectifier (C5: 1920x1080): trained here, judged against the 64-spp truth
    if not args.no_learned and rank == 0:
        forms["learned"] = time_learned(T, WL, dev, stream, sid, args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        import oracle as O  # the checker; timed here as the CPU baseline only
        O.load()
        nthr = os.cpu_count() or 1
        frames = []
        for f in range(3):
            frames.append(dict(color=col[f].float().cpu().numpy(), depth=dep[f].cpu().numpy(),
                               motion=mot[f].float().cpu().numpy(), jitter=T.synth_jitter(sc, f)[1]))
        params = O.Parameters.from_buffer_copy(bytes(wl.parameters()))
        done, t = time_oracle(params, frames, nthr, args.cpu_seconds)
        cpu = {"value": wl.pixels * done / t / 1e6, "unit": UNIT, "cores": nthr, "kind": "port",
               "sample": f"{done} consecutive 3840x2160 frames of the C2 workload through the FP32 oracle "
                         f"restatement of taa.comp ({t:.1f} s, {nthr} threads)"}
        # the same restatement on one core: one 3840x2160 frame at least
        done1, t1 = time_oracle(params, frames, 1, min(3.0, args.cpu_seconds))
        cpu["single_core"] = {"value": wl.pixels * done1 / t1 / 1e6, "unit": UNIT, "cores": 1,
                              "sample": f"{done1} 3840x2160 frame(s) ({t1:.1f} s, 1 thread)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": mpx, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded analytic scene rendered on the GPU)",
            "config": c2_config(world), "frames_per_step": F, "form": form_name,
            "timing": "CUDA events around a CUDA graph of the 64-frame sequence, replayed once per step",
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "note": f"peak: {peak_kind}; achieved = {bpp} B/px x {W}x{H} / avg launch"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": sampler.summary(),
            "forms": forms,
            "summary": summarize(form_name, mpx, achieved / peak, forms, e2e, cpu),
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_profile_case(args):
    """A few launches of one form on 3 frames of the 4K workload (or one batch
    of the C4 views), for an ncu capture: about 1 GB on the device."""
    import torch
    import taa_abi as T
    import workloads as WL
    from importlib import util
    spec = util.spec_from_file_location("taa_lib_build", ROOT / "taa-star_gb300" / "build.py")
    m = util.module_from_spec(spec)
    spec.loader.exec_module(m)
    m.build_library()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    sid = stream.cuda_stream
    if args.profile == "batch48":
        args.steps, args.warmup = 3, 1
        print(json.dumps(time_batch(T, WL, dev, stream, sid, 1, args, 1.0, 1.0)))
        return 0
    wl = WL.c2()
    H, W, F = wl.height, wl.width, 3
    sc = wl.scene()
    col = torch.empty(F, H, W, 4, dtype=torch.float16, device=dev)
    dep = torch.empty(F, H, W, dtype=torch.float32, device=dev)
    mot = torch.empty(F, H, W, 2, dtype=torch.float16, device=dev)
    for f in range(F):
        T.synth_render(sc, f, stream=sid, color=col[f], depth=dep[f], motion=mot[f])
    hist = [torch.zeros(H, W, 4, dtype=torch.float32, device=dev) for _ in range(2)]
    res = torch.empty(H, W, 4, dtype=torch.float16, device=dev)
    if args.profile == "fxaa":
        # one resolve with the segmentation mask, then the FXAA pass: 3 launches on the mask, 1 on every pixel
        u = T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(sc, 2)[1])
        for i in range(2):
            u.param[i].mRayTraceAugment = 1
            u.param[i].mRayTraceAugmentFlags = 0x3F | 0x200
        ctx = T.Taa(W, H, form=T.TAA_FORM_PLAIN)
        ctx.set_uniforms(u)
        seg = torch.empty(H, W, dtype=torch.int32, device=dev)
        ctx.resolve(stream=sid, color=col[2], depth=dep[2], velocity=mot[2], history=col[1].float(),
                    history_depth=dep[1], history_out=hist[0], result=res, segmask=seg)
        out = torch.empty_like(res)
        fctx = T.Taa(W, H, form=T.TAA_FORM_PLAIN, flags=T.TAA_FLAG_FXAA)
        for i in range(4):
            T.fxaa(res, out, seg if i < 3 else None, stream=sid, ctx=fctx)
        fctx.close()
        torch.cuda.synchronize()
        ctx.close()
        return 0
    if args.profile == "up":  # TAAU 1920x1080 -> 3840x2160 in the fast form, two resolves
        lo = WL.Workload("C2 scene at 1920x1080", 1920, 1080, F, seed=wl.seed, num_spheres=wl.num_spheres,
                         cam_v0=(1.0, 0.0), cam_accel=(19.0 / 63.0, 0.0), radius=(10.0, 60.0), params=dict(wl.params))
        lsc = lo.scene()
        lc = torch.empty(F, 1080, 1920, 4, dtype=torch.float16, device=dev)
        ld = torch.empty(F, 1080, 1920, dtype=torch.float32, device=dev)
        lm = torch.empty(F, 1080, 1920, 2, dtype=torch.float16, device=dev)
        for f in range(F):
            T.synth_render(lsc, f, stream=sid, color=lc[f], depth=ld[f], motion=lm[f])
        ctx = T.Taa(1920, 1080, W, H)
        for f in range(1, F):
            ctx.set_uniforms(T.make_uniforms(lo.parameters(), jitter_ndc=T.synth_jitter(lsc, f)[1], mUpsampling=1))
            ctx.resolve(stream=sid, color=lc[f], depth=ld[f], velocity=lm[f], history=hist[f & 1],
                        history_depth=ld[f - 1], history_out=hist[(f + 1) & 1], result=res)
        torch.cuda.synchronize()
        ctx.close()
        return 0
    params = wl.parameters()
    kw, bind = {}, {}
    if args.profile == "fused":  # the fast form's one-launch resolve + CAS 0.5
        kw = dict(sharpener=T.TAA_SHARPEN_CAS, sharpen_factor=0.5, flags=T.TAA_FLAG_FUSED_SHARPEN)
        bind = dict(sharpened=torch.empty(H, W, 4, dtype=torch.float16, device=dev))
    elif args.profile == "defaults":  # the reference's default parameter block in the fast form
        params = T.default_parameters()
    elif args.profile == "learned":  # the learned form's strip kernel (random weights)
        kw = dict(form=T.TAA_FORM_LEARNED)
    elif args.profile == "learned_tc":  # the same on tcgen05, activations in tensor memory
        kw = dict(form=T.TAA_FORM_LEARNED, flags=T.TAA_FLAG_LEARNED_TCGEN05)
    form = {"fast": T.TAA_FORM_FAST, "tiled": T.TAA_FORM_TILED, "fp16": T.TAA_FORM_FP16, "plain": T.TAA_FORM_PLAIN,
            "fused": T.TAA_FORM_FAST, "defaults": T.TAA_FORM_FAST, "learned": T.TAA_FORM_LEARNED,
            "learned_tc": T.TAA_FORM_LEARNED}[args.profile]
    kw.setdefault("form", form)
    ctx = T.Taa(W, H, **kw)
    if args.profile in ("learned", "learned_tc"):
        ctx.set_mlp(T.mlp_init_weights(1, 0.1))
    for f in range(1, F):
        ctx.set_uniforms(T.make_uniforms(params, jitter_ndc=T.synth_jitter(sc, f)[1]))
        ctx.resolve(stream=sid, color=col[f], depth=dep[f], velocity=mot[f], history=hist[f & 1],
                    history_depth=dep[f - 1], history_out=hist[(f + 1) & 1], result=res, **bind)
    torch.cuda.synchronize()
    ctx.close()
    return 0


def run_isa_rates():
    """Packed FP32, packed FP16 and scalar FP32 FMA issue rates on this GPU: the
    stand-alone program in taa-star_gb300/csrc/isa_rates.cu, built with nvcc."""
    sys.path.insert(0, str(ROOT / "taa-star_gb300"))
    import build as B
    B.OUT.mkdir(exist_ok=True)
    exe = B.OUT / "isa_rates"
    subprocess.run([B.nvcc(), *B.ARCH, "-O3", "-o", str(exe), str(B.CSRC / "isa_rates.cu")], check=True)
    return subprocess.run([str(exe)]).returncode


def main():
    args = parse()
    if args.isa_rates:
        return run_isa_rates()
    if args.profile:
        return run_profile_case(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
