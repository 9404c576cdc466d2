"""Host logic of bench.py that the JSON line rests on: the clock record read
from nvidia-smi samples, the DRAM traffic per launch read from the committed
ncu summary, and the CPU baseline's energy sample."""
import json
import os

import numpy as np

import bench


class _FakeProc:
    def terminate(self):
        pass

    def wait(self):
        return 0


def _sampler_with(tmp_path, lines):
    cs = bench.ClockSampler()
    cs.path = str(tmp_path / "clocks.csv")
    with open(cs.path, "w") as f:
        f.write("\n".join(lines) + "\n")
    cs.f = open(cs.path)
    cs.proc = _FakeProc()
    return cs


def test_clock_record_median_max_and_reasons(tmp_path):
    # index, sm, sm max, power, active mask, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
    lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
             "0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
             "0, 2070, 2070, 1200.5, 0x0, Not Active, Not Active, Not Active, Not Active",
             "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
             "garbage"]
    rec = _sampler_with(tmp_path, lines).stop()
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["sw_power_cap"]
    assert rec["samples"] == 3


def test_clock_record_reports_thermal_slowdown(tmp_path):
    lines = ["0, 1500, 2070, 1000, 0x40, Not Active, Active, Not Active, Not Active",
             "0, 1600, 2070, 1000, 0x0, Not Active, Not Active, Not Active, Not Active"]
    rec = _sampler_with(tmp_path, lines).stop()
    assert rec["reasons"] == ["hw_thermal_slowdown"]
    assert rec["sm_mhz"] == 1550.0


def test_clock_record_without_nvidia_smi():
    cs = bench.ClockSampler()
    cs.proc = None
    assert cs.stop()["reasons"] == ["nvidia-smi unavailable"]


def test_traffic_reads_the_committed_summary():
    """roofline.traffic is the per-launch capture scaled by the problems a
    benchmark launch processes, as each entry states ("x a/b")."""
    with open(os.path.join(bench.HERE, "profiles", "traffic.json")) as f:
        t = json.load(f)
    kernels = [k for k in t if not k.startswith("_")]
    assert "k_oz_mma" in kernels
    for kernel in kernels:
        v = t[kernel]
        assert bench._traffic(kernel) == v["bytes"] > 0
        a, b = v["scale"].split()[1].split("/")
        assert abs(v["bytes"] - v["measured_bytes_per_launch"] * float(a) / float(b)) < 1e-6 * v["bytes"]
    assert bench._traffic("no such kernel") is None


def test_cpu_energy_sample_covers_the_grid():
    grid = np.round(np.arange(401) * bench.E_STEP + bench.E_MIN, 10)
    s0 = bench.cpu_energy_sample(16, 0)
    assert len(s0) == 16 and len(set(s0)) == 16
    assert set(s0) <= set(grid)
    assert s0[0] == bench.E_MIN and s0[-1] == bench.E_MAX
    s1 = bench.cpu_energy_sample(16, 1)
    # successive steps take other energies (the last index wraps onto the first)
    assert len(set(s0) & set(s1)) <= 1
    assert set(bench.cpu_energy_sample(16, 401)) == set(s0)
