"""Host-side pieces of bench.py on the CPU: the clock sampler keeps the samples of the
timed window only (injected samples and a fake sampler command stand in for
nvidia-smi), and the grouped contraction's algorithmic bytes follow from the library's
counters."""
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402


def _row(mhz, power_cap=False):
    return [str(mhz), "2070", "900.0", "Not Active", "Not Active", "Not Active",
            "Active" if power_cap else "Not Active"]


def test_summary_keeps_the_timed_window():
    clk = bench.ClockSampler(0)
    clk.rows = [(1.0, _row(1500)), (2.0, _row(2070)), (2.5, _row(2070, True)), (3.0, _row(2055)),
                (4.0, _row(1500))]
    clk.t0, clk.t1 = 1.5, 3.5
    s = clk.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}


def test_sampler_collects_rows_from_its_command():
    fake = [sys.executable, "-u", "-c",
            "import time\n"
            "for i in range(20):\n"
            "    print('2070, 2070, 900.0, Not Active, Not Active, Not Active, Not Active', flush=True)\n"
            "    time.sleep(0.01)\n"]
    clk = bench.ClockSampler(0, cmd=fake).start()
    deadline = time.time() + 10
    while len(clk.rows) < 20 and time.time() < deadline:
        time.sleep(0.02)
    clk.stop()
    s = clk.summary()  # no window set: every sample
    assert s["samples"] == 20 and s["sm_mhz"] == 2070.0 and s["reasons"] == []


def test_summary_without_a_sampler_says_so():
    clk = bench.ClockSampler(0, cmd=["/nonexistent/sampler"]).start()
    clk.begin()
    clk.end()
    clk.stop()
    s = clk.summary()
    assert s["samples"] == 0 and s["reasons"] == ["unavailable"]


def test_grouped_algorithmic_bytes():
    # 64 particles x 625 origins against 900 listed rows each, K = 12,736, two launches
    g = {"gemm_launches": 2, "kpad": 12736, "gemm_flops": 2 * (64 * 2.0 * 625 * 900 * 12736)}
    want = (64 * 625 + 64 * 900) * 12736 * 2.0
    assert abs(bench.grouped_algorithmic_bytes(g, 625) - want) < 1e-6 * want
    assert bench.grouped_algorithmic_bytes({"gemm_launches": 0, "kpad": 0, "gemm_flops": 0.0}, 625) is None
