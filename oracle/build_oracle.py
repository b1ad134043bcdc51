"""Build recipe for the oracle (test infrastructure, the checker).

``build_oracle()`` compiles the CPU restatement of the reference resolve into
``oracle/_build/liboracle.so`` with g++.  It is built with
``-ffp-contract=off`` so that its FP32 instance rounds every operation as
written, and without any machine-specific flag so it gives the same bits on
x86-64 and aarch64.

``build_reference()`` (only where the reference tree is present) builds
``oracle/_ref/``: the reference's own source files compiled as they lie, used
to pin the restatement (see ``oracle/ref_build.py``).
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"

SOURCES = [HERE / "taa_oracle.cpp", HERE / "oracle_capi.cpp"]
HEADERS = [HERE / "taa_oracle.hpp", ROOT / "include" / "taa_params.h", ROOT / "include" / "taa_synth.h",
           ROOT / "taa-star_gb300" / "csrc" / "synth_scene.h"]


def cxx() -> str:
    for cand in ("g++", "c++"):
        p = shutil.which(cand)
        if p:
            return p
    raise RuntimeError("no C++ compiler found")


def build_oracle(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    deps = SOURCES + HEADERS + [Path(__file__)]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    cmd = [cxx(), "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread",
           "-I", str(ROOT / "include"), *map(str, SOURCES), "-o", str(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


def build_reference(force: bool = False):
    """Build oracle/_ref from the reference sources when they are present."""
    from importlib import util

    spec = util.spec_from_file_location("ref_build", HERE / "ref_build.py")
    if spec is None or not (HERE / "ref_build.py").exists():
        return None
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
