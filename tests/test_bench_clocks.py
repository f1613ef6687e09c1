"""bench.py samples the SM clocks and throttle reasons during the timed region
with nvidia-smi: the sampler waits for its first sample before the timed
region starts (a timed region is a fraction of a second), reports the median
SM clock and every throttle reason seen, and gives None where nvidia-smi is
absent (CPU; nvidia-smi is faked by a script on PATH)."""

import os
import stat
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402

FAKE = """#!{python}
import sys, time
time.sleep({delay})
rows = {rows!r}
k = 0
while True:
    sys.stdout.write(rows[k % len(rows)] + "\\n")
    sys.stdout.flush()
    k += 1
    time.sleep(0.05)
"""

ROWS = ["0, 2070 MHz, 2070 MHz, 812.40 W, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1980 MHz, 2070 MHz, 1391.00 W, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070 MHz, 2070 MHz, 1020.10 W, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"]


def _fake_smi(tmp_path, monkeypatch, delay):
    path = tmp_path / "nvidia-smi"
    path.write_text(FAKE.format(python=sys.executable, delay=delay, rows=ROWS))
    path.chmod(path.stat().st_mode | stat.S_IXUSR)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ.get('PATH', '')}")


def test_sampler_waits_for_first_sample_and_summarises(tmp_path, monkeypatch):
    _fake_smi(tmp_path, monkeypatch, delay=0.4)
    s = bench.ClockSampler(0)
    t0 = time.monotonic()
    s.start()
    assert time.monotonic() - t0 >= 0.3
    assert os.path.getsize(s.path) > 0
    time.sleep(0.3)
    out = s.stop()
    assert out["samples"] >= 3
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_sampler_wait_is_bounded(tmp_path, monkeypatch):
    _fake_smi(tmp_path, monkeypatch, delay=30)
    s = bench.ClockSampler(0)
    t0 = time.monotonic()
    s.start(first_sample_s=0.5)
    assert time.monotonic() - t0 < 5
    assert s.stop() is None


def test_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))
    s = bench.ClockSampler(0)
    s.start()
    assert s.stop() is None
