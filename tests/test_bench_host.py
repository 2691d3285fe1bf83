"""Host-side pieces of bench.py (no GPU): the clock summary that accepts or flags a timed run,
and the byte model of the fused V-cycle phases that the live roofline divides by."""
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)


def test_clock_summary_median_max_and_reasons():
    import bench

    text = "\n".join([
        "0, 2070, 2070, 812.4, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1390.2, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 1980, 2070, 1399.9, 0x0000000000000008, Active, Not Active, Not Active, Active",
        "garbage line",
        "0, [N/A], 2070, 0, 0, Not Active, Not Active, Not Active, Not Active",
    ])
    out = bench.clock_summary(text)
    assert out["samples"] == 3
    assert out["sm_mhz"] == 2055.0
    assert out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["hw_slowdown", "sw_power_cap"]


def test_clock_summary_empty():
    import bench

    out = bench.clock_summary("")
    assert out == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_phase_bytes_of_the_served_union():
    """The L0 post-smooth of the served config-2 batch: FP32 f in and u out plus the corrections'
    face reads, the figure the live roofline uses (201,097,216 bytes)."""
    import bench
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB

    levels, _, _ = PB.config2()
    bl, _ = M.union_hierarchy([levels] * 16)
    assert bench._phase_bytes("L0 post-smooth", bl, 4) == pytest.approx(201097216.0)
    pre = bench._phase_bytes("L0 pre-smooth", bl, 4)
    assert pre == pytest.approx(2 * 4 * bl[0].num_cells)
