"""bench.py's nvidia-smi samplers, fed synthetic samples (no GPU): the clock
summary that decides whether a timed run is kept (median SM clock, the
throttle reasons seen) and the memory peaks, overall and inside a time
window, that the large-configuration line reports per phase."""

import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_clock_summary_median_and_reasons():
    b = _bench()
    c = b.ClockSampler(0)
    row = lambda sm, pc: ["%d" % sm, "2070", "900", "Not Active", "Not Active", "Not Active", pc]
    c.samples = [(0.0, row(2070, "Not Active")), (0.2, row(1965, "Active")), (0.4, row(2070, "Not Active")),
                 (0.6, ["[N/A]", "2070"])]  # a short or unreadable line is skipped
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    c.samples = [(0.0, ["1400", "2070", "900", "Active", "Not Active", "Active", "Not Active"])]
    assert c.summary()["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]


def test_memory_peak_overall_and_by_window():
    b = _bench()
    m = b.MemSampler(0)
    m.samples = [(1.0, ["700"]), (2.0, ["48000"]), (3.0, ["30000"]), (4.0, ["bad"])]
    mib = 1048576 / 1e9
    assert m.peak_gb() == round(48000 * mib, 2)
    assert m.peak_gb(2.5, 3.5) == round(30000 * mib, 2)
    assert m.peak_gb(5.0, 6.0) is None


def test_samplers_without_nvidia_smi():
    b = _bench()
    with b.ClockSampler(0) as c, b.MemSampler(0) as m:
        pass
    # on a host without the tool the samplers record nothing and report empty summaries
    if c.proc is None:
        assert c.summary()["samples"] == 0 and m.peak_gb() is None
