"""Host-side pieces of bench.py on CPU: the clock record keeps only the nvidia-smi samples stamped
inside the timed region, and flags throttle reasons seen there."""
import os
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Done:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _stamp(t):
    return time.strftime("%Y/%m/%d %H:%M:%S", time.localtime(t)) + ".%03d" % int((t % 1) * 1000)


def _clocks_with(rows, t0, t1):
    c = bench.Clocks(0)
    fd, c.path = tempfile.mkstemp(suffix=".csv")
    os.close(fd)
    with open(c.path, "w") as f:
        for t, mhz, reason in rows:
            act = ["Not Active"] * 4
            if reason is not None:
                act[reason] = "Active"
            f.write(f"{_stamp(t)}, 0, {mhz}, 2070, 900.0, 0x0, {act[0]}, {act[1]}, {act[2]}, {act[3]}\n")
    c.f = open(os.devnull, "w")
    c.proc = _Done()
    c.t0, c.t1 = t0, t1
    return c


def test_clock_samples_outside_the_region_are_dropped(monkeypatch):
    monkeypatch.setattr(bench.time, "sleep", lambda s: None)
    base = time.time() - 100.0
    rows = [(base + 0.00, 1000.0, 1), (base + 0.50, 2070.0, None), (base + 0.55, 2060.0, 3),
            (base + 0.60, 2070.0, None), (base + 1.50, 900.0, 2)]
    rec = _clocks_with(rows, base + 0.45, base + 0.65).stop()
    assert rec["samples"] == 3 and rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["sw_power_cap"] and rec["where"] == "inside the timed region"


def test_short_region_takes_the_nearest_samples(monkeypatch):
    monkeypatch.setattr(bench.time, "sleep", lambda s: None)
    base = time.time() - 100.0
    rows = [(base + 0.00, 1500.0, None), (base + 0.05, 2070.0, None), (base + 0.10, 2065.0, None),
            (base + 0.90, 800.0, 1)]
    rec = _clocks_with(rows, base + 0.06, base + 0.07).stop()
    assert rec["samples"] == 2 and rec["where"] == "nearest to the timed region"
    assert rec["sm_mhz"] == (2070.0 + 2065.0) / 2 and rec["reasons"] == []
