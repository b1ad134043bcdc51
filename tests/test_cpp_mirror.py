"""The C++ mirror of taa<CF> (taa-star_gb300/taa.hpp): it compiles against the
C ABI (CPU) and drives a short synthetic sequence on the GPU (-m gpu)."""
import subprocess
from pathlib import Path

import pytest

import build as lib_build

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "taa-star_gb300" / "examples" / "sequence.cpp"


def compile_example(tmp_path):
    lib = lib_build.build_library()
    exe = tmp_path / "sequence"
    cmd = [lib_build.nvcc(), "-std=c++17", "-O2", "-x", "cu", str(SRC), "-o", str(exe), "-L", str(lib.parent),
           "-ltaa_gb300", f"-Xlinker=-rpath,{lib.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_mirror_compiles(built, tmp_path):
    assert compile_example(tmp_path).exists()


@pytest.mark.gpu
def test_mirror_runs_a_sequence(cuda, tmp_path):
    exe = compile_example(tmp_path)
    r = subprocess.run([str(exe), "160", "96", "6"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("frame")]
    assert len(lines) == 6
    means = [float(l.split()[-1]) for l in lines]
    assert all(0.0 < m < 64.0 for m in means), r.stdout


@pytest.mark.gpu
def test_mirror_runs_the_fxaa_chain(cuda, tmp_path):
    # resolve with the segmentation mask -> FXAA on the marked pixels -> CAS
    exe = compile_example(tmp_path)
    r = subprocess.run([str(exe), "160", "96", "6", "fxaa"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l.split() for l in r.stdout.splitlines() if l.startswith("frame")]
    assert len(lines) == 6
    marked = [int(l[l.index("marked") + 1]) for l in lines]
    assert all(m > 0 for m in marked[1:]), r.stdout
    assert all(0.0 < float(l[-1]) < 64.0 for l in lines), r.stdout


@pytest.mark.gpu
def test_mirror_runs_the_post_process_pass(cuda, tmp_path):
    # split screen, debug image on the left, zoom inset: the split column is black
    exe = compile_example(tmp_path)
    r = subprocess.run([str(exe), "160", "96", "4", "post"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l.split() for l in r.stdout.splitlines() if l.startswith("frame")]
    assert len(lines) == 4
    black = [int(l[l.index("split_black") + 1]) for l in lines]
    assert all(b == 96 for b in black[1:]), r.stdout  # every row of column W / 2 (frame 0 is the source copy)
