"""Host logic of bench.py's measurement harness, without a GPU: the clock
record keeps only the samples taken inside the timed region and reports the
median SM clock under load and every throttle reason seen there."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _line(sm, smax=2070, power=900.0, hw="Not Active", thermal="Not Active",
          sw_thermal="Not Active", power_cap="Not Active"):
    return f"0, {sm}, {smax}, {power}, 0x0, {hw}, {thermal}, {sw_thermal}, {power_cap}"


class _Done:
    """Stands in for the finished nvidia-smi process."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _sampler(samples, t0=None, t1=None):
    c = bench.ClockSampler(0)
    c.proc = _Done()
    c.lines = list(samples)
    c.t0, c.t1 = t0, t1
    return c


def test_only_samples_inside_the_region_count():
    samples = [(0.0, _line(900)), (1.0, _line(2070)), (1.1, _line(2070)),
               (1.2, _line(2055)), (3.0, _line(600, thermal="Active"))]
    rec = _sampler(samples, 0.5, 2.0).stop()
    assert rec["samples"] == 3
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == []  # the thermal sample lies after the region


def test_reasons_seen_in_the_region_are_reported():
    samples = [(1.0, _line(1980, power_cap="Active")), (1.1, _line(1500, hw="Active"))]
    rec = _sampler(samples, 0.5, 2.0).stop()
    assert rec["reasons"] == ["hw_slowdown", "sw_power_cap"]


def test_all_samples_count_when_none_fell_inside():
    samples = [(0.0, _line(2070)), (5.0, _line(2070))]
    rec = _sampler(samples, 1.0, 2.0).stop()
    assert rec["samples"] == 2


def test_malformed_lines_are_skipped():
    samples = [(1.0, "garbage"), (1.1, _line("[N/A]")), (1.2, _line(2040))]
    rec = _sampler(samples, 0.5, 2.0).stop()
    assert rec["samples"] == 1 and rec["sm_mhz"] == 2040.0


def test_unavailable_sampler_says_so():
    c = bench.ClockSampler(0)
    c.proc = None
    assert c.stop()["reasons"] == ["nvidia-smi unavailable"]
