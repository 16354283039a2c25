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


def test_serving_phases(bench):
    """The serving stream's per-request phase split: means by lattice size and
    channel, failed requests left out, shares of the admitted time."""
    class Wav:
        def __init__(self, L, channel):
            self.L, self.channel = L, channel

    def req(L, ch):
        return (0.0, {"wav": Wav(L, ch)})

    def res(sub, adm, sta, wal, don, steps, status=0):
        return {"status": status, "t_submit": sub, "t_admit": adm, "t_started": sta, "t_walked": wal,
                "t_done": don, "steps": steps}

    reqs = [req(8, "groundstate"), req(8, "groundstate"), req(16, "trans"), req(16, "trans")]
    out = [res(0.0, 1.0, 2.0, 5.0, 6.0, 300), res(1.0, 1.0, 3.0, 4.0, 6.0, 100),
           res(0.0, 0.5, 1.0, 3.0, 4.0, 400), res(0.0, 0.0, 0.0, 0.0, 0.0, 0, status=6)]
    phases, share = bench.serving_phases(reqs, out)
    assert set(phases) == {"L8_gs", "L16_trans"}
    gs = phases["L8_gs"]
    assert gs["jobs"] == 2 and gs["queue_s"] == 0.5 and gs["start_s"] == 1.5 and gs["walk_s"] == 2.0
    assert gs["retire_s"] == 1.5 and gs["steps_per_job"] == 200 and gs["walk_steps_per_s"] == 100.0
    tr = phases["L16_trans"]
    assert tr["jobs"] == 1 and tr["walk_s"] == 2.0 and tr["walk_steps_per_s"] == 200.0
    # admitted time: start 3 + 0.5, walk 4 + 2, retire 3 + 1
    assert abs(share["start_s"] - 3.5 / 13.5) < 1e-12 and abs(share["walk_s"] - 6.0 / 13.5) < 1e-12
    assert abs(sum(share.values()) - 1.0) < 1e-12
