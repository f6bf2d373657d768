"""Host-side pieces of bench.py: the clock record, the figures read from the
committed ncu summaries (used only on the kernel sources they were taken
on), the reference arm's timing, the replica arithmetic and the workload
generators."""

from __future__ import annotations

import argparse
import glob
import json
import os
import time

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


def test_committed_profile_figures_are_keyed_to_the_kernel_sources(tmp_path, monkeypatch):
    # a figure is used only when taken on the current kernel sources
    sha = bench.kernel_sources_sha()
    assert len(sha) == 16
    prof = tmp_path / "profiles"
    prof.mkdir()
    (prof / "fresh.json").write_text(json.dumps({"kernel_sources_sha": sha, "warp_instructions_per_launch": 5e8}))
    (prof / "stale.json").write_text(json.dumps({"kernel_sources_sha": "0" * 16, "warp_instructions_per_launch": 5e8}))
    for rel in bench.KERNEL_SOURCES:
        (tmp_path / rel).parent.mkdir(parents=True, exist_ok=True)
        (tmp_path / rel).write_bytes(open(os.path.join(bench.REPO, rel), "rb").read())
    monkeypatch.setattr(bench, "REPO", str(tmp_path))
    assert bench.ncu_figures("fresh")["warp_instructions_per_launch"] == 5e8
    assert bench.ncu_figures("stale") is None
    assert bench.ncu_figures("absent") is None
    # a figure that names its kernel's sources is keyed to those alone
    (prof / "apply.json").write_text(json.dumps({"kernel_sources_sha": bench.kernel_sources_sha(bench.APPLY_SOURCES),
                                                 "sources": list(bench.APPLY_SOURCES)}))
    assert bench.ncu_figures("apply") is not None
    (tmp_path / "qmb-public_gb300/csrc/relative.cu").write_bytes(b"// changed")
    assert bench.ncu_figures("apply") is not None
    assert bench.ncu_figures("fresh") is None
    (tmp_path / "qmb-public_gb300/csrc/apply.cu").write_bytes(b"// changed")
    assert bench.ncu_figures("apply") is None


def test_committed_profile_json_files_parse():
    for path in glob.glob(os.path.join(bench.REPO, "profiles", "*.json")):
        figs = json.load(open(path))
        assert len(figs["kernel_sources_sha"]) == 16 and "command" in figs, path


def test_both_arms_report_the_same_config():
    wl = bench.make_workload("c1")
    args = argparse.Namespace(workload="c1", gpus=1)
    assert bench.workload_config(args, wl) == bench.workload_config(args, wl)
    assert bench.workload_config(args, wl)["n_i"] == 400


def test_reference_arm_times_what_it_reports():
    # a tiny fraction of C1 on two processes: the line's steps and times are the ones it ran
    wl = bench.make_workload("c1")
    args = argparse.Namespace(workload="c1", gpus=1, steps=3, warmup=1, ref_fraction=0.1)
    t0 = time.perf_counter()
    line = bench.run_reference(args, wl)
    wall = time.perf_counter() - t0
    assert line["impl"] == "reference" and line["steps"] == 3
    assert line["ms_per_step"] * line["steps"] / 1e3 <= wall
    assert line["value"] > 0 and line["cpu_baseline"]["one_core"]["cores"] == 1
    assert line["config"] == bench.workload_config(args, wl)


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
