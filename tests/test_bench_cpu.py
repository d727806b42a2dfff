"""Host logic of bench.py: the clock record that decides whether a run is
kept (throttle reasons seen during the timed region, median SM clock) and
the mixed form's algorithmic bytes per cell-step behind its roofline."""
import bench


def row(idx, sm, mx, hw="Not Active", hwt="Not Active", swt="Not Active", pcap="Not Active"):
    return f"{idx}, {sm}, {mx}, 950.00, 0x0000000000000000, {hw}, {hwt}, {swt}, {pcap}"


def test_clean_run():
    text = "\n".join(row(0, 2070, 2070) for _ in range(5))
    c = bench.parse_clocks(text, 0)
    assert c == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 5}


def test_throttle_reasons_and_median():
    text = "\n".join([row(0, 2070, 2070), row(0, 1900, 2070, pcap="Active"), row(0, 1500, 2070, hwt="Active"),
                      row(0, 2070, 2070)])
    c = bench.parse_clocks(text, 0)
    assert c["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert c["sm_mhz"] == 1985.0 and c["sm_max_mhz"] == 2070.0 and c["samples"] == 4


def test_other_gpus_ignored():
    text = "\n".join([row(0, 2070, 2070), row(3, 900, 2070, hw="Active"), row(0, 2070, 2070)])
    c = bench.parse_clocks(text, 0)
    assert c["reasons"] == [] and c["sm_mhz"] == 2070.0 and c["samples"] == 2


def test_unparsable_samples():
    c = bench.parse_clocks("garbage\n\n", 0)
    assert c["sm_mhz"] is None and c["samples"] == 0


def test_mixed_bytes_per_cell_step():
    # Two refinement passes and seven V-cycles per projection at 256^3.
    assert round(bench.mixed_bytes_per_cell_step(2, 7)) == 1736
