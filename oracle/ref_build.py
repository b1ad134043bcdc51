"""Builds oracle/_ref: the reference's own code for the resolve path, compiled here.

Test infrastructure: these libraries pin the oracle's restatement; nothing in
the product loads them, and they exist only where the reference tree is
present (they are not built on the GPU machine).

  * libtaa_ref32.so / libtaa_ref64.so - shaders/taa.comp and
    shaders/sharpen.comp compiled as C++ through oracle/ref_shim/glsl_shim.hpp
    with REAL = float / double.  The shader text is copied into oracle/_ref
    with three mechanical rewrites only: the `#version` and `#extension` lines
    are dropped (C++ has no such directives) and `out T name` / `inout T name`
    parameters become `T &name` (C++ spells out-parameters as references).
  * libcas_ref.so - CasSetup from shaders/ffx_cas.h with ffx_a.h's CPU path
    (A_CPU), exactly as source/taa.hpp:15-19 compiles it.
  * libcas_filter_ref.so - shaders/sharpen_cas.comp (CasFilter of
    shaders/ffx_cas.h on the GLSL half of shaders/ffx_a.h, A_GPU + A_GLSL)
    through oracle/ref_shim/ffx_glsl.hpp, FP32; ffx_a.h and ffx_cas.h get the
    same rewrites (plus `#define outAF2 out AF2` -> `#define outAF2 AF2 &`)
    and are written beside the shader so that its includes find them.

The reference tree is read from $TAA_REFERENCE_ROOT, by default
/root/reference.
  * libfxaa_ref32.so / libfxaa_ref64.so - shaders/antialias_fxaa_prepare.comp
    and shaders/antialias_fxaa.comp (which includes shaders/Fxaa3_11_mod.h
    from the reference tree as it lies) through the same shim, with the
    sampler snapping within 1/512 texel of a texel centre.
  * libpost_ref32.so / libpost_ref64.so - shaders/post_process.comp (which
    includes shaders/shader_cpu_common.h) through the same shim.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REF = Path(os.environ.get("TAA_REFERENCE_ROOT", "/root/reference"))
SHADERS = REF / "shaders"
OUT = HERE / "_ref"
SHIM = HERE / "ref_shim"


def available() -> bool:
    return (SHADERS / "taa.comp").exists() and (SHADERS / "ffx_cas.h").exists()


def rewrite(src: Path, dst: Path) -> None:
    text = src.read_text()
    lines = [ln for ln in text.splitlines() if not re.match(r"\s*#\s*(version|extension)\b", ln)]
    text = "\n".join(lines) + "\n"
    text = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)\b", r"\1 &\2", text)
    # the same qualifier inside a macro that names a parameter type (ffx_a.h:1720-1731)
    text = re.sub(r"^(\s*#\s*define\s+\w+\s+)(?:inout|out)\s+(\w+)\s*$", r"\1\2 &", text, flags=re.M)
    dst.write_text(text)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)


def build(force: bool = False):
    if not available():
        return None
    OUT.mkdir(exist_ok=True)
    taa = OUT / "taa_comp.glsl.inc"
    sharpen = OUT / "sharpen_comp.glsl.inc"
    rewrite(SHADERS / "taa.comp", taa)
    rewrite(SHADERS / "sharpen.comp", sharpen)
    cxx = shutil.which("g++") or "c++"
    common = [cxx, "-O1", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
              "-Wno-pedantic", "-I", str(SHIM), "-I", str(SHADERS), "-I", str(ROOT / "include"),
              f'-DTAA_COMP_SOURCE="{taa}"', f'-DSHARPEN_SOURCE="{sharpen}"', str(SHIM / "taa_ref_main.cpp")]
    libs = {}
    for name, flags in (("libtaa_ref32.so", ["-DREAL=float", "-fsingle-precision-constant"]),
                        ("libtaa_ref64.so", ["-DREAL=double"])):
        lib = OUT / name
        if force or not lib.exists() or lib.stat().st_mtime < max(p.stat().st_mtime for p in SHIM.iterdir()):
            _run([*common, *flags, "-o", str(lib)])
        libs[name] = lib
    prep = OUT / "fxaa_prepare_comp.glsl.inc"
    fx = OUT / "fxaa_comp.glsl.inc"
    rewrite(SHADERS / "antialias_fxaa_prepare.comp", prep)
    rewrite(SHADERS / "antialias_fxaa.comp", fx)
    fxaa_common = [cxx, "-O1", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                   "-Wno-pedantic", "-I", str(SHIM), "-I", str(SHADERS), "-DGLSL_SNAP=(1.0/512.0)",
                   f'-DFXAA_PREPARE_SOURCE="{prep}"', f'-DFXAA_SOURCE="{fx}"', str(SHIM / "fxaa_ref_main.cpp")]
    for name, flags in (("libfxaa_ref32.so", ["-DREAL=float", "-fsingle-precision-constant"]),
                        ("libfxaa_ref64.so", ["-DREAL=double"])):
        lib = OUT / name
        if force or not lib.exists() or lib.stat().st_mtime < max(p.stat().st_mtime for p in SHIM.iterdir()):
            _run([*fxaa_common, *flags, "-o", str(lib)])
        libs[name] = lib
    post = OUT / "post_process_comp.glsl.inc"
    rewrite(SHADERS / "post_process.comp", post)
    post_common = [cxx, "-O1", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                   "-Wno-pedantic", "-I", str(SHIM), "-I", str(SHADERS), f'-DPOST_SOURCE="{post}"',
                   str(SHIM / "post_ref_main.cpp")]
    for name, flags in (("libpost_ref32.so", ["-DREAL=float", "-fsingle-precision-constant"]),
                        ("libpost_ref64.so", ["-DREAL=double"])):
        lib = OUT / name
        if force or not lib.exists() or lib.stat().st_mtime < max(p.stat().st_mtime for p in SHIM.iterdir()):
            _run([*post_common, *flags, "-o", str(lib)])
        libs[name] = lib
    cas = OUT / "libcas_ref.so"
    if force or not cas.exists():
        _run([cxx, "-O1", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", str(SHADERS),
              str(SHIM / "cas_setup_ref.cpp"), "-o", str(cas)])
    libs["libcas_ref.so"] = cas
    # sharpen_cas.comp includes ffx_a.h and ffx_cas.h; the rewritten copies sit
    # beside it, so the compiler's search from the including file finds them first
    rewrite(SHADERS / "sharpen_cas.comp", OUT / "sharpen_cas_comp.glsl.inc")
    rewrite(SHADERS / "ffx_a.h", OUT / "ffx_a.h")
    rewrite(SHADERS / "ffx_cas.h", OUT / "ffx_cas.h")
    casf = OUT / "libcas_filter_ref.so"
    if force or not casf.exists() or casf.stat().st_mtime < max(p.stat().st_mtime for p in SHIM.iterdir()):
        _run([cxx, "-O1", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
              "-fsingle-precision-constant", "-Wno-pedantic", "-I", str(SHIM), "-I", str(SHADERS),
              f'-DCAS_SOURCE="{OUT / "sharpen_cas_comp.glsl.inc"}"', str(SHIM / "cas_ref_main.cpp"), "-o", str(casf)])
    libs["libcas_filter_ref.so"] = casf
    return libs


if __name__ == "__main__":
    print(build(force=True))
