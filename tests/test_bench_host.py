"""Host-side parts of bench.py that need no GPU: the clock-record parser
that decides whether a timed run was throttled, and the seeded synthetic
workloads every arm runs."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class _Done:
    """Stands in for the finished nvidia-smi process."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _parse(tmp_path, lines):
    path = tmp_path / "clocks.csv"
    path.write_text("".join(l + "\n" for l in lines))
    s = bench.ClockSampler(0)
    s.proc, s.path = _Done(), str(path)
    return s.stop()


def test_clock_record_median_and_no_reasons(tmp_path):
    rows = ["0, %d, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active" % mhz
            for mhz in (2070, 2055, 2070, 1980, 2070)]
    c = _parse(tmp_path, rows)
    assert c == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 5}
    assert not os.path.exists(tmp_path / "clocks.csv")  # the record is removed after parsing


def test_clock_record_reports_throttle_reasons(tmp_path):
    rows = ["0, 1800, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
            "0, 1700, 2070, 1395.0, 0x40, Not Active, Active, Not Active, Not Active",
            "bad line",
            "0, n/a, 2070, 1.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    c = _parse(tmp_path, rows)
    assert c["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert c["samples"] == 2 and c["sm_mhz"] == 1750.0


def test_clock_record_empty_is_none(tmp_path):
    assert _parse(tmp_path, []) is None


def test_workload_is_seeded_and_inside_the_box():
    pos_a, p_a = bench.workload(32, 16)
    pos_b, p_b = bench.workload(32, 16)
    pos_r1, _ = bench.workload(32, 16, seed_offset=1)
    assert pos_a.shape == (32 ** 3, 3) and pos_a.dtype == np.float64
    assert np.array_equal(pos_a, pos_b) and p_a == p_b
    assert not np.array_equal(pos_a, pos_r1)  # each replica rank gets its own box
    L = p_a["boxsize"]
    assert L == pytest.approx(500.0 * 32 / 256)
    assert pos_a.min() >= 0.0 and pos_a.max() < L
    assert p_a["maxleaf"] == 16 and p_a["theta"] == 0.5


@pytest.mark.parametrize("name", ["nfw128", "zeldovich512"])
def test_named_workloads_scale_at_fixed_density(name):
    pos, p = bench.workload(24, 64, name=name)
    assert pos.shape == (24 ** 3, 3)
    assert pos.min() >= 0.0 and pos.max() < p["boxsize"]
    assert p["maxleaf"] == 64


def test_defaults_and_the_cpu_legs_leaf(monkeypatch):
    # with no flags: one GPU, the 256^3 workload, leaf size from the autotuner
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    args = bench.parse()
    assert (args.gpus, args.impl, args.workload, args.nside, args.maxleaf) == (1, "ours", "zeldovich256", 256, 0)
    assert args.warmup >= 3
    # the CPU baseline and the reference arm run the leaf the autotuner picks
    # for that workload, not a faster but less accurate one
    assert bench.CHOSEN_LEAF["zeldovich256"] == 64
