"""The bench line's host logic on CPU: the clock record (rows written before the timed region
are left out, throttle reasons are read from the samples, a missing nvidia-smi is reported) and
the roofline arithmetic of the per-kernel CUDA-event figures."""
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


def test_roofline_arithmetic():
    """The bench line's roofline objects from per-kernel CUDA-event stats: achieved = the
    algorithmic work per launch over the average launch time, frac = achieved / peak."""
    pairs = 4.45e6 * 4096  # algorithmic point pairs of one launch
    stats = {"cubature": {"count": 2, "ms": 90.0, "flops": 2 * 1e12},
             "cubature_far": {"count": 2, "ms": 80.0, "flops": 2 * pairs},
             "fisher": {"count": 2, "ms": 2.0, "flops": 0.0}}
    r = bench.roofline(stats, {"sm_mhz": 2070.0}, 6783.8, 1928.8, "measured", 41)
    avg_s = 0.040
    assert r["bound"] == "issue" and r["launches"] == 2
    assert abs(r["achieved"] - pairs / avg_s / 1e9) < 1e-6 * r["achieved"]
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert abs(r["peak"] - 128.0 * 152 * 2070e6 / bench.FAR_OPS_PER_PAIR / 1e9) < 1e-6 * r["peak"]
    h = r["roofline_hbm"]
    assert abs(h["algorithmic_bytes_per_launch"] - 8.0 * 41 * 4.45e6) < 1.0
    assert abs(h["frac"] - h["achieved"] / 6783.8) < 1e-12
    t = bench.tensor_roofline({"count": 1, "ms": 42.0, "flops": 1.76e13}, 1928.8, "measured")
    assert abs(t["achieved"] - 3 * 1.76e13 / 0.042 / 1e12) < 1e-6 * t["achieved"]
    assert abs(t["algorithmic_tflops_per_s"] - t["achieved"] / 3) < 1e-9 * t["achieved"]
    assert bench.tensor_roofline({"count": 0, "ms": 0.0, "flops": 0.0}, 1928.8, "measured") is None
