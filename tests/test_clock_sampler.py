"""bench.py's clock record, against a stand-in nvidia-smi on PATH that
prints the query's CSV rows every 50 ms: the sampler waits for its first
row, keeps the rows taken while it runs, and reads the throttle reasons."""
import os
import stat
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

FAKE = """#!/bin/sh
# stand-in: idle row first, then rows under load
echo "345, 2070, 120.00, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
while true; do
  echo "2032, 2070, 1100.00, 0x0000000000000004, Not Active, Not Active, Not Active, %s"
  sleep 0.05
done
"""


@pytest.fixture
def bench_with_fake_smi(tmp_path, monkeypatch, request):
    exe = tmp_path / "nvidia-smi"
    exe.write_text(FAKE % request.param)
    exe.chmod(exe.stat().st_mode | stat.S_IXUSR)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ["PATH"])
    sys.path.insert(0, ROOT)
    import bench
    yield bench
    sys.path.remove(ROOT)


@pytest.mark.parametrize("bench_with_fake_smi", ["Active"], indirect=True)
def test_power_cap_is_reported_and_idle_row_dropped(bench_with_fake_smi):
    cs = bench_with_fake_smi.ClockSampler(0)
    cs.start()
    assert cs.lines, "start() returns after the first row"
    time.sleep(0.4)
    rec = cs.stop()
    assert rec["samples"] >= 3
    assert rec["sm_mhz"] == 2032.0 and rec["sm_max_mhz"] == 2070.0   # the idle 345 MHz row is not kept
    assert rec["reasons"] == ["sw_power_cap"]


@pytest.mark.parametrize("bench_with_fake_smi", ["Not Active"], indirect=True)
def test_short_region_keeps_one_row(bench_with_fake_smi):
    cs = bench_with_fake_smi.ClockSampler(0)
    cs.start()
    rec = cs.stop()                       # a region shorter than one interval
    assert rec is not None and rec["samples"] >= 1 and rec["reasons"] == []
