"""Host logic of bench.py that needs no GPU: the clock record (median SM
clock, maximum, throttle reasons) from NVML samples and from nvidia-smi
lines."""
import bench


def test_clock_summary_from_nvml_samples():
    c = bench.Clocks(0)
    c.source, c.max_mhz = "nvml", 2070.0
    # clock-event reason bits: 0x4 sw power cap, 0x8 hw slowdown, 0x40 hw thermal
    c.samples = [(2070.0, 0), (2070.0, 0x8), (1500.0, 0x40 | 0x4)]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap"]


def test_clock_summary_from_nvidia_smi_lines():
    c = bench.Clocks(0)
    c.source = "nvidia-smi"
    c.lines = ["0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
               "0, 1980, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
               "garbage"]
    s = c.summary()
    assert s["sm_mhz"] == 2025.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 2
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_summary_without_samples():
    s = bench.Clocks(0).summary()
    assert s["sm_mhz"] is None and s["reasons"] == ["no clock samples"]
