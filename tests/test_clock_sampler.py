"""bench.py's clock record: the nvidia-smi sampler keeps the samples of the timed window, falls
back to a 200 ms interval without the timestamp field when nvidia-smi refuses the first form,
and reports throttle reasons only from the samples it keeps.  A fake nvidia-smi stands in for
the real one; no GPU is needed."""
import os
import stat
import sys
import textwrap
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

FAKE = """\
#!{python}
import datetime, sys, time
args = " ".join(sys.argv[1:])
if {refuse_timestamp} and "timestamp" in args:
    sys.exit(2)
period = int(sys.argv[sys.argv.index("-lms") + 1]) / 1000.0
t_start = time.time()
while True:
    now = time.time()
    # sw_thermal_slowdown for the first {hot_ms} ms, none afterwards
    hot = "Active" if (now - t_start) * 1000 < {hot_ms} else "Not Active"
    row = ["0", "2070", "2070", "900.0", "0x0", "Not Active", "Not Active", hot, "Not Active"]
    if "timestamp" in args:
        row.append(datetime.datetime.fromtimestamp(now).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3])
    print(", ".join(row), flush=True)
    time.sleep(period)
"""


def _fake(tmp_path, refuse_timestamp=False, hot_ms=0):
    p = tmp_path / "nvidia-smi"
    p.write_text(textwrap.dedent(FAKE.format(python=sys.executable, refuse_timestamp=refuse_timestamp,
                                             hot_ms=hot_ms)))
    p.chmod(p.stat().st_mode | stat.S_IEXEC)
    return str(p)


def test_samples_of_the_timed_window(tmp_path):
    s = bench.ClockSampler(0, period_ms=10, exe=_fake(tmp_path, hot_ms=150))
    s.start()
    assert s.lines, "start() returns once the first sample is in"
    time.sleep(0.4)                        # the throttled samples are before the window
    t0 = time.time()
    time.sleep(0.2)
    t1 = time.time()
    c = s.stop(t0, t1)
    assert c["window"] == "timed" and c["samples"] >= 3
    assert c["sm_mhz"] == 2070.0 and c["sm_max_mhz"] == 2070.0
    assert c["reasons"] == [], "a reason seen only before the window is not reported"
    assert c["period_ms"] == 10


def test_reasons_inside_the_window_are_reported(tmp_path):
    s = bench.ClockSampler(0, period_ms=10, exe=_fake(tmp_path, hot_ms=10_000))
    s.start()
    t0 = time.time()
    time.sleep(0.1)
    c = s.stop(t0, time.time())
    assert c["window"] == "timed" and c["reasons"] == ["sw_thermal_slowdown"]


def test_short_window_takes_the_nearest_sample(tmp_path):
    s = bench.ClockSampler(0, period_ms=300, exe=_fake(tmp_path))
    s.start()
    time.sleep(0.05)
    t0 = time.time()
    t1 = t0 + 1e-4                          # shorter than the interval: no sample inside
    c = s.stop(t0, t1)
    assert c["samples"] == 1 and c["window"] in ("nearest", "timed")


def test_falls_back_when_the_first_form_is_refused(tmp_path):
    s = bench.ClockSampler(0, period_ms=25, exe=_fake(tmp_path, refuse_timestamp=True))
    s.start()
    assert s.period_ms == 200 and "timestamp" not in s.fields
    time.sleep(0.5)
    c = s.stop()
    assert c["window"] == "all" and c["samples"] >= 1 and c["sm_mhz"] == 2070.0


def test_missing_nvidia_smi(tmp_path):
    s = bench.ClockSampler(0, exe=str(tmp_path / "no-such-tool"))
    s.start()
    c = s.stop(time.time(), time.time())
    assert c["sm_mhz"] is None and c["reasons"] == ["nvidia-smi unavailable"]


@pytest.mark.parametrize("text", ["2026/12/04 07:42:00.123", "garbage"])
def test_timestamp_parse(text):
    t = bench.ClockSampler._stamp(text, fallback=-1.0)
    assert (t == -1.0) == (text == "garbage")
