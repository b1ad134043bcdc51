"""Build recipe for libtaa_gb300.so (sm_103a), in-tree, without cmake.

Every translation unit is compiled by nvcc in parallel and linked into
``taa-star_gb300/_build/libtaa_gb300.so``.  The FP32 resolve units are
compiled with ``-fmad=false`` so that they round operation for operation like
the FP32 oracle (their sources place explicit FMAs where the oracle has them);
the FP16 form's and the reassociating FP32 form's units may contract to FMA.

Usage: ``python taa-star_gb300/build.py`` or ``build_library()`` from Python.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libtaa_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"),
          "--expt-relaxed-constexpr"]

# unit -> extra flags
UNITS = {
    "resolve_plain.cu": ["-fmad=false"],
    "resolve_fast.cu": ["-fmad=false"],
    "resolve_tiled.cu": ["-fmad=false"],
    "resolve_fast32.cu": [],
    "resolve_up32.cu": [],
    "resolve_gen32.cu": [],
    "resolve_learned_strips.cu": [],
    "resolve_half.cu": [],
    "resolve_half_guard.cu": [],
    "batch_tiled.cu": ["-fmad=false"],
    "learned.cu": ["-fmad=false"],
    "fxaa.cu": ["-fmad=false"],
    "post_process.cu": ["-fmad=false"],
    "synth.cu": [],
    "static_scratch.cu": [],
    "device_state.cu": [],
    "capi.cpp": [],
    "batch_api.cpp": [],
    "learned_api.cpp": [],
    "post_api.cpp": [],
    "settings.cpp": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compile and link the CUDA library; returns the path of the .so."""
    OUT.mkdir(exist_ok=True)
    cc = nvcc()
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    for unit, extra in UNITS.items():
        src = CSRC / unit
        obj = OUT / (unit.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers, Path(__file__)]):
            flags = list(extra)
            if ptxas_info and unit.endswith(".cu"):
                flags += ["-Xptxas", "-v"]
            lang = ["-x", "cu"]  # capi.cpp includes the device headers too
            jobs.append([cc, *ARCH, *COMMON, *flags, *lang, "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
        list(ex.map(_run, jobs))
    if force or jobs or not LIB.exists():
        _run([cc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart_static", "-lrt", "-ldl", "-lpthread",
              "-Xlinker", "--no-undefined"])
    return LIB


if __name__ == "__main__":
    p = build_library(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(p)
