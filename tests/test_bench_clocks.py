"""Host logic of bench.py's clock record (no GPU): samples taken during the
timed region are summarised; a region shorter than the sampling interval is
bracketed by the samples just before and after it."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _sampler():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.ClockSampler(0)


IDLE = "2070, 2070, Not Active, Not Active, Not Active, Not Active"
CAPPED = "1980, 2070, Not Active, Not Active, Not Active, Active"
HOT = "1500, 2070, Not Active, Not Active, Active, Not Active"


def test_samples_inside_the_timed_region():
    c = _sampler()
    c.lines = [HOT, IDLE, IDLE, CAPPED, HOT]
    c.skip, c.n_inside = 1, 3  # the first sample predates the region, the last follows it
    out = c.summary()
    assert out["samples"] == 3 and out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]
    assert "bracketing" not in out


def test_short_region_is_bracketed():
    c = _sampler()
    c.lines = [IDLE, IDLE, HOT]
    c.skip, c.n_inside = 2, 0
    out = c.summary()
    assert out["samples"] == 2 and out["reasons"] == ["sw_thermal_slowdown"]
    assert "bracketing" in out


def test_no_samples_at_all():
    c = _sampler()
    out = c.summary()
    assert out["samples"] == 0 and out["sm_mhz"] is None
