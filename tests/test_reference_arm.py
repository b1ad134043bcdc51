"""The benchmark's reference arm builds its inputs from the oracle alone (CPU).

`bench.py --impl reference` times the oracle's FP32 restatement of taa.comp
on the host cores.  It must not load the library (the arm measures the
reference's path, not this library), so its scene, sphere table, jitter,
parameter block and uniform block come from oracle/oracle.py.  These tests
hold those inputs to the workload the library's own arm runs (C2), byte for
byte, and check in a child process that the arm's imports leave the library
unloaded.
"""
import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

import oracle as O
import taa_abi as T
import workloads as WL

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def test_reference_inputs_equal_the_c2_workload(built):
    import bench
    sc, params = bench.reference_c2()
    wl = WL.c2()
    assert bytes(sc) == bytes(wl.scene())
    assert bytes(params) == bytes(wl.parameters())
    assert bench.C2_NAME == wl.name
    cfg = bench.c2_config(1)
    assert (cfg["width"], cfg["height"], cfg["frames"]) == (wl.width, wl.height, wl.frames)
    assert cfg["bytes_per_px"] == wl.bytes_per_pixel(history_bytes=16, motion_bytes=4)
    np.testing.assert_array_equal(O.synth_spheres(sc)[:sc.num_spheres],
                                  np.asarray(T.synth_spheres(wl.scene()))[:sc.num_spheres])
    for f in (0, 3, 7, 63):
        assert O.synth_jitter(sc, f) == T.synth_jitter(wl.scene(), f)[1]
    u_o = O.make_uniforms(params, jitter_ndc=O.synth_jitter(sc, 5), mResetHistory=1)
    u_t = T.make_uniforms(wl.parameters(), jitter_ndc=T.synth_jitter(wl.scene(), 5)[1], mResetHistory=1)
    assert bytes(u_o) == bytes(u_t)
    assert bytes(O.default_parameters()) == bytes(T.default_parameters())


def test_reference_arm_does_not_load_the_library(built):
    code = (f"import sys; sys.path[:0] = [{str(ROOT)!r}, {str(ROOT / 'oracle')!r}]\n"
            "import bench\n"
            "sc, p = bench.reference_c2()\n"
            "fr = bench.cpu_frames_for_reference(bench.reference_c2()[0].__class__.from_buffer_copy(bytes(sc)), 0)\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('LIB' if 'libtaa_gb300' in maps else 'NOLIB', 'ORACLE' if 'liboracle' in maps else '')\n")
    # a small scene keeps the host render short
    code = code.replace("bench.reference_c2()[0].__class__.from_buffer_copy(bytes(sc))",
                        "__import__('oracle').synth_scene(64, 36, 2)")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "NOLIB" in r.stdout and "ORACLE" in r.stdout, r.stdout
