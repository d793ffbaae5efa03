"""Host logic of bench.py's measurement harness, without a GPU: the clock
record keeps only the samples taken inside the timed region and reports the
median SM clock under load and every throttle reason seen there; the
reference arm (``--impl reference``, the CPU oracle timed on a bounded row
sample) prints one line with the contract's keys on rank 0 and nothing on
the other ranks."""
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


def _reference_arm(env_extra=None):
    import json
    import subprocess

    env = dict(os.environ)
    env.update(env_extra or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "wf32768", "--steps", "2", "--warmup", "1",
                        "--cpu-sample-s", "0.2"],
                       capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_prints_one_contract_line():
    (line,) = _reference_arm()
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC
    assert line["unit"] == "s" and line["higher_is_better"] is False
    assert line["steps"] == 2 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert line["value"] > 0 and abs(line["ms_per_step"] - 1e3 * line["value"]) < 1e-6 * 1e3 * line["value"]
    assert line["config"]["workload"] == "wf-32768px-grf"
    base = line["cpu_baseline"]
    assert base["kind"] == "port" and base["cores"] >= 1 and base["value"] == line["value"]
    assert "rows" in base["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["vs_baseline"] is None


def test_reference_arm_other_ranks_do_no_work():
    assert _reference_arm({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []
