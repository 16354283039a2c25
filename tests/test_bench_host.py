"""Host-side logic of bench.py, CPU only: the nvidia-smi clock record (samples
kept by timestamp inside the timed region, throttle reasons collected) and
the measured-peak lookup."""
import importlib.util
import os
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _line(t, sm, reasons=("Not Active",) * 4):
    ts = time.strftime("%Y/%m/%d %H:%M:%S", time.localtime(int(t))) + ".%03d" % int((t % 1) * 1000)
    return "%s, 0, %d, 2070, 900.0, 0x0, %s\n" % (ts, sm, ", ".join(reasons))


def test_clock_samples_inside_the_window(bench):
    c = bench.Clocks(0)
    c.proc = True        # summary() only checks that a sampler ran
    t = float(int(time.time())) + 0.1
    c.out = (_line(t, 1200) + _line(t + 0.2, 2070) + _line(t + 0.4, 2050)
             + _line(t + 0.6, 2070, ("Not Active", "Not Active", "Not Active", "Active")) + _line(t + 0.9, 900)
             + "garbage line\n")
    s = c.summary(t + 0.15, t + 0.65)
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    everything = c.summary()
    assert everything["samples"] == 5


def test_clock_reasons_detected(bench):
    c = bench.Clocks(0)
    c.proc = True
    t = float(int(time.time())) + 0.1
    c.out = _line(t, 1500, ("Active", "Not Active", "Active", "Not Active"))
    s = c.summary(t - 1, t + 1)
    assert s["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]


def test_no_sampler(bench):
    c = bench.Clocks(0)
    c.proc = None
    s = c.summary(0.0, 1.0)
    assert s["sm_mhz"] is None and s["reasons"] == ["nvidia-smi unavailable"]


def test_measured_peaks(bench):
    peak, kind = bench.measured_peaks()
    assert peak > 0 and kind in ("measured", "fallback")
