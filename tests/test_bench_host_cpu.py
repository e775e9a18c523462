"""Host-side measurement logic of bench.py on the CPU (no GPU, no nvidia-smi).

- ClockSampler keeps only the nvidia-smi samples whose timestamps fall inside the timed
  region, reports their median SM clock and the throttle reasons seen active there, and falls
  back to the sample nearest to a region shorter than the sampling period;
- the algorithmic bytes of one rank-kernel launch follow the roofline's unit count: 4 B value
  + 4 B row id per stored entry, 8 B per column pointer, 4 B per cell's group id and 16 B per
  test (U1 and P), i.e. 1.238 GB for the 200,000 x 8,000 x 500 screen;
- the per-launch ncu figures bench.py reads come from the committed summary of the rank kernel.
"""
import os
import sys
import tempfile
import types

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


class _DoneProcess:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _sampler(lines):
    s = bench.ClockSampler.__new__(bench.ClockSampler)
    s.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
    s.f.write("\n".join(lines) + "\n")
    s.f.flush()
    s.p = _DoneProcess()
    return s


def _line(sec, sm, reasons=("Not Active",) * 4):
    # timestamp, index, clocks.sm, clocks.max.sm, power.draw, reasons.active,
    # hw_slowdown, hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap
    return f"2026/12/03 10:00:{sec:06.3f}, 0, {sm}, 2070, 900.5, 0x0, " + ", ".join(reasons)


def _t(sec):
    return bench.ClockSampler._parse(_line(sec, 0))[0]


def test_clock_sampler_keeps_the_timed_region_only():
    lines = [_line(1.0, 1200), _line(2.0, 2070), _line(2.05, 2055),
             _line(2.10, 2070, ("Not Active", "Not Active", "Not Active", "Active")),
             _line(3.0, 900, ("Active", "Not Active", "Not Active", "Not Active"))]
    out = _sampler(lines).stop(_t(1.99), _t(2.11))
    assert out["samples"] == 3 and out["where"] == "inside the timed region"
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]  # the hw_slowdown outside the region is not kept


def test_clock_sampler_nearest_sample_for_a_short_region():
    lines = [_line(1.0, 1500), _line(1.05, 2070), _line(1.10, 1800)]
    out = _sampler(lines).stop(_t(1.051), _t(1.052))
    assert out["samples"] == 1 and out["where"] == "nearest to the timed region"
    assert out["sm_mhz"] == 2070.0


def test_clock_sampler_without_samples_or_nvidia_smi():
    assert _sampler(["garbage"]).stop(0.0, 1.0)["reasons"] == ["no samples"]
    s = bench.ClockSampler.__new__(bench.ClockSampler)
    s.p = None
    assert s.stop()["reasons"] == ["nvidia-smi unavailable"]


def test_algorithmic_bytes_of_the_screen():
    w = types.SimpleNamespace(nnz=146_628_899, n_cols=8_000, n_targets=500, n_rows=200_000)
    b = bench.algorithmic_bytes(w)
    assert b == 146_628_899 * 8 + 8 * 8_001 + 4 * 200_000 + 16 * 8_000 * 500
    assert abs(b / 1e9 - 1.238) < 0.001


def test_profile_figures_come_from_the_committed_summary():
    path = os.path.join(ROOT, "profiles", "mwu_rank_kernel_perturb_screen.txt")
    if not os.path.exists(path):
        pytest.skip("no committed rank-kernel summary")
    traffic = bench.traffic_from_profile()
    insts = bench.profile_figure("warp_instructions_per_launch_full_workload")
    assert traffic is not None and traffic > 1e9
    assert insts is not None and insts > 1e9
    assert bench.profile_figure("no_such_figure") is None
