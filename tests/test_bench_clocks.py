"""bench.py's clock sampler against a stand-in nvidia-smi on PATH: it waits
for the first sample before the timed region starts, keeps only what it saw
during the region, and reports the median SM clock, the maximum and the
throttle reasons that were active."""
import os
import stat
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402

SCRIPT = """#!/bin/sh
sleep 0.2
echo "0, 1200, 2070, 300.0, 0x1, Not Active, Not Active, Not Active, Not Active"
while true; do
  echo "0, {mhz}, 2070, 1100.5, 0x4, Not Active, Not Active, Not Active, {cap}"
  sleep 0.05
done
"""


def _fake(tmp_path, monkeypatch, mhz=2070, cap="Not Active"):
    exe = tmp_path / "nvidia-smi"
    exe.write_text(SCRIPT.format(mhz=mhz, cap=cap))
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ.get("PATH", ""))


def test_samples_cover_the_timed_region_only(tmp_path, monkeypatch):
    _fake(tmp_path, monkeypatch, mhz=1980)
    with bench.ClockSampler(0) as c:
        time.sleep(0.2)
    s = c.summary()
    # the idle first line (1200 MHz) came before the region and is dropped
    assert s["sm_mhz"] == 1980.0 and s["sm_max_mhz"] == 2070.0
    assert s["samples"] >= 2 and s["reasons"] == []


def test_active_reasons_are_reported(tmp_path, monkeypatch):
    _fake(tmp_path, monkeypatch, cap="Active")
    with bench.ClockSampler(0) as c:
        time.sleep(0.15)
    assert c.summary()["reasons"] == ["sw_power_cap"]


def test_no_sampler_reads_as_unsampled(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))  # no nvidia-smi anywhere
    with bench.ClockSampler(0) as c:
        pass
    assert c.summary()["reasons"] == ["unsampled"]
