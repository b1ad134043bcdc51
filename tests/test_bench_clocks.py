"""The benchmark's clock record on CPU: the NVML sampler's summary of its
samples (median SM clock, the largest maximum clock, the throttle reasons by
NVML's bit, none left out) and its fallback to nvidia-smi where NVML cannot
be loaded.  No GPU."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def test_nvml_summary_names_every_throttle_reason():
    s = bench.NvmlClockSampler(None, None)
    s.samples = [(2070, 2070, 0x0), (1950, 2070, 0x4), (2070, 2070, 0x8 | 0x40), (2070, 2070, 0x20), (2010, 2070, 0x1)]
    r = s.summary()
    assert r["sm_mhz"] == 2070 and r["sm_max_mhz"] == 2070 and r["samples"] == 5
    assert r["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap", "sw_thermal_slowdown"]


def test_nvml_summary_without_samples_says_so():
    r = bench.NvmlClockSampler(None, None).summary()
    assert r["sm_mhz"] is None and r["reasons"]


def test_sampler_falls_back_without_nvml(monkeypatch):
    import ctypes

    def no_library(*a, **k):
        raise OSError("not here")

    monkeypatch.setattr(ctypes, "CDLL", no_library)
    assert isinstance(bench.NvmlClockSampler.make(0), bench.ClockSampler)
