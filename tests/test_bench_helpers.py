"""Host-side pieces of bench.py: the clock record, the figures read from the
committed ncu summaries, the replica arithmetic and the workload generators."""

from __future__ import annotations

import numpy as np

import bench


def test_clock_summary_flags_throttling():
    s = bench.ClockSampler(0)
    s.lines = [
        "0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2070, 2070, 1100.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 1800, 2070, 1200.0, 0x8, Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    out = s.summary()
    assert out["samples"] == 3
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["hw_slowdown", "sw_power_cap"]


def test_committed_profile_figures_are_readable():
    # the bench line's traffic and issue roofline come from these summaries
    assert bench.ncu_traffic("c2") > 1e6
    inst = bench.ncu_figure("c2", "warp_instructions_per_launch")
    assert inst is not None and inst > 1e8
    assert bench.ncu_traffic("no-such-workload") is None


def test_replica_value_and_single_rank_max():
    assert bench.replica_value(1e9, 2.0, 4) == 4 * 1e9 / 2e-3
    assert bench.max_over_ranks([1.0, 3.0]) == [1.0, 3.0]


def test_workloads_have_the_stated_shapes():
    wl = bench.make_workload("c1")
    assert wl["configs_i"].shape == (400, 2) and wl["n_terms"] == wl["site"].shape[0]
    # unique, sorted determinants with 3 alpha and 3 beta electrons
    rows = wl["configs_i"]
    assert np.unique(rows, axis=0).shape[0] == rows.shape[0]
    bits = np.unpackbits(rows, axis=1, bitorder="little")[:, :12]
    assert np.all(bits[:, 0::2].sum(axis=1) == 3) and np.all(bits[:, 1::2].sum(axis=1) == 3)
    for name, spec in bench.WORKLOADS.items():
        assert "description" in spec and spec["n_i"] > 0, name
