"""CPU checks of bench.py's host logic: the clock-sample parsing that decides whether a timed
run is kept (throttle reasons, median SM clock) and the roofline arithmetic."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("h3d_bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Done:
    """A finished sampler process."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def test_clock_samples_give_median_clock_and_active_reasons():
    B = _bench()
    c = B.ClockSampler(0)
    c.proc = _Done()
    c.lines = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 1965, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1200.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    r = c.stop()
    assert r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0 and r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]
    c2 = B.ClockSampler(0)
    c2.proc = _Done()
    c2.lines = ["0, 1200, 2070, 700, 0x40, Not Active, Active, Not Active, Not Active"]
    assert c2.stop()["reasons"] == ["hw_thermal_slowdown"]
    c3 = B.ClockSampler(0)
    assert c3.stop()["reasons"] == ["nvidia-smi unavailable"]


def test_roofline_arithmetic():
    B = _bench()
    peak, kind = B._peaks()
    r = B._roofline(sweep_bytes=15 * 2 * 1e9, sweep_seconds=2e-3, samples=2, launches_per_ds=15, kernel="k",
                    traffic=1.0)
    assert abs(r["achieved"] - 15000.0) < 1e-9 and abs(r["frac"] - 15000.0 / peak) < 1e-12
    assert abs(r["alg_bytes_per_launch"] - 1e9) < 1e-3 and abs(r["avg_launch_us"] - 1e6 * 2e-3 / 30) < 1e-9
    assert r["peak_source"] == kind and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert B._roofline(1.0, 0.0, 0, 15, "k") is None
