"""The bench's clock record on CPU: rows written before the timed region are left out,
throttle reasons are read from the samples, and a missing nvidia-smi is reported."""
from conftest import ROOT  # noqa: F401  (puts the repository root on sys.path)
import bench


class _Proc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def poll(self):
        return None


def _row(sm, hw="Not Active", pc="Not Active"):
    return f"0, {sm}, 2070, 900.00, 0x0, {hw}, Not Active, Not Active, {pc}\n"


def test_rows_before_the_mark_are_left_out():
    c = bench.ClockSampler(0)
    c.proc = _Proc()
    c.skip = 0
    with open(c.out.name, "w") as f:
        f.write(_row(345) + _row(345))
    c.mark()
    with open(c.out.name, "a") as f:
        f.write(_row(2070) + _row(2070, pc="Active") + _row(2070))
    r = c.stop()
    assert r["samples"] == 3 and r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0
    assert r["reasons"] == ["sw_power_cap"]


def test_no_rows_in_the_region_keeps_the_earlier_ones():
    c = bench.ClockSampler(0)
    c.proc = _Proc()
    c.skip = 0
    with open(c.out.name, "w") as f:
        f.write(_row(2070, hw="Active"))
    c.mark()
    r = c.stop()
    assert r["samples"] == 1 and r["reasons"] == ["hw_slowdown"]


def test_missing_nvidia_smi():
    c = bench.ClockSampler(0)
    c.proc = None
    c.skip = 0
    assert c.stop()["reasons"] == ["nvidia-smi unavailable"]
