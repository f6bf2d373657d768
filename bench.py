"""Benchmark of the Hamiltonian engine's hot path on one GB300.

Default workload (``--workload c2``): a synthetic ab-initio Hamiltonian on 28
spin orbitals (14 spatial, n_qubytes 4; 55,371 normal-ordered terms from
seeded integrals), configs_i = 20,000 and configs_j = 200,000 unique random
determinants with 5 alpha + 5 beta electrons, complex N(0,1) amplitudes.

One step is the FP32-compensated apply_within forward (configs_i ->
configs_j) followed by its adjoint (configs_j -> configs_i), i.e. the work of
one energy-gradient evaluation, run as it is in training: through
apply_within's autograd function, whose forward walk records its hits and
whose backward replays them.  The metric is term applications per second
counted as the reference counts them: T * (N_i + N_j) per step (the
reference's thread grid is T * N_i for a forward application, T * N_j for
the same kernel run on the daggered table from configs_j).  The engine
visits fewer pairs (one walk over the 20,000 configs_i rows);
``walked_pairs_per_s`` reports that count.  The same
line reports the FP64 path, the reference's own CUDA apply_within run from
its cubin (``ref_cuda_fp64``), find_relative (top 50,000 excluding
configs_i), the energy error of the FP32 path, the end-to-end rate through
the public API with host buffers, the rooflines of the term walk, and the
CPU oracle's rate on the host cores.

``--impl reference`` times the reference's CPU algorithm (the oracle port in
oracle/, bit-identical to the reference's _hamiltonian_cpu.cpp and within 16 %
of its speed on one core where both run) on a bounded sample of every step:
the forward over a slice of configs_i and the adjoint, as the reference
would compute it (its apply_within on the daggered table from configs_j
onto configs_i), over a slice of configs_j, on every host core.

``--workload c1|c3|c4|c5|lanczos|pt2|sampler`` runs the other shapes (one JSON line
each, clocked, L2 flushed before every timed step, with a roofline).
"""

from __future__ import annotations

import argparse
import importlib
import json
import math
import multiprocessing as mp
import os
import re
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOADS = {
    "c3": dict(n_orbit=26, n_alpha=7, n_beta=7, n_i=65536, n_j=65536, count_selected=0, seed=2025,
               description="ab-initio 52 spin orbitals (n_qubytes 7), 7a+7b, 65536 configs, MLP 4x512 wave function, "
                           "energy forward + backward"),
    "c4": dict(hubbard=(8, 8, 1.0, 4.0), n_orbit=64, n_alpha=32, n_beta=32, n_i=1000000, n_j=1000000,
               count_selected=0, seed=2026,
               description="Fermi-Hubbard 8x8 open, t=1, U=4, 128 spin orbitals (n_qubytes 16), 32a+32b, "
                           "1,000,000 configs, complex64 amplitudes"),
    "c5": dict(n_orbit=38, n_alpha=10, n_beta=10, n_i=8192, n_j=8192, count_selected=1000000, seed=2027,
               description="ab-initio 76 spin orbitals (n_qubytes 10), 10a+10b, 8192 seeds, find_relative top "
                           "1,000,000"),
    "c2": dict(n_orbit=14, n_alpha=5, n_beta=5, n_i=20000, n_j=200000, count_selected=50000, seed=2024,
               description="ab-initio 28 spin orbitals (n_qubytes 4), 5a+5b, N_i 20000, N_j 200000, K 50000"),
    "c1": dict(n_orbit=6, n_alpha=3, n_beta=3, n_i=400, n_j=400, count_selected=100, seed=2024,
               description="ab-initio 12 spin orbitals (n_qubytes 2), 3a+3b, all 400 determinants"),
    "lanczos": dict(n_orbit=26, n_alpha=7, n_beta=7, n_i=65536, n_j=65536, count_selected=0, seed=2025,
                    lanczos_steps=20,
                    description="ab-initio 52 spin orbitals (n_qubytes 7), 7a+7b, 65536-determinant basis, "
                                "20 Lanczos iterations (H materialised once; through_walks_ms: every iteration "
                                "walks the terms)"),
    "sampler": dict(n_orbit=26, n_alpha=7, n_beta=7, n_i=65536, n_j=65536, count_selected=0, seed=2028,
                    hidden=(512, 512),
                    description="autoregressive MLP wave function (qmb/mlp.py WaveFunctionElectronUpDown) on 26 sites "
                                "(52 spin orbitals), 7a+7b, hidden (512, 512): generate_unique of 65,536 configurations"),
    "pt2": dict(n_orbit=38, n_alpha=10, n_beta=10, n_i=8192, n_j=8192, count_selected=1000000, seed=2027,
                description="ab-initio 76 spin orbitals (n_qubytes 10), 10a+10b, 8192 variational determinants, "
                            "Epstein-Nesbet PT2 over the top 1,000,000 connection records"),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------


def make_workload(name: str):
    import numpy as np

    qmb = importlib.import_module("qmb-public_gb300")
    terms = qmb.terms
    w = WORKLOADS[name]
    if "hubbard" in w:
        site, kind, coef = terms.sort_terms(*terms.prepare(terms.hubbard_dict(*w["hubbard"])))
    else:
        site, kind, coef = terms.integral_hamiltonian_tables(w["n_orbit"], seed=w["seed"])
    if w["n_i"] == w["n_j"] and name == "c1":
        ci = terms.all_determinants(w["n_orbit"], w["n_alpha"], w["n_beta"])
        cj = ci
    elif w["n_i"] == w["n_j"]:
        ci = terms.random_determinants(w["n_orbit"], w["n_alpha"], w["n_beta"], w["n_i"], seed=w["seed"] + 1)
        cj = ci
    else:
        ci = terms.random_determinants(w["n_orbit"], w["n_alpha"], w["n_beta"], w["n_i"], seed=w["seed"] + 1)
        cj = terms.random_determinants(w["n_orbit"], w["n_alpha"], w["n_beta"], w["n_j"], seed=w["seed"] + 2)
    psi = terms.random_psi(ci.shape[0], seed=w["seed"] + 3)
    return dict(site=site.numpy(), kind=kind.numpy(), coef=coef.numpy(), configs_i=ci, configs_j=cj, psi=psi,
                n_terms=int(site.shape[0]), nq=int(ci.shape[1]), spec=w)


# ---------------------------------------------------------------------------
# CPU timing of the reference's algorithm (the oracle port): reference arm and
# cpu_baseline
# ---------------------------------------------------------------------------

_CPU = {}


def _cpu_init(site, kind, coef, ci, psi, cj, g):
    """Worker set-up: both directions' tables, rows and amplitudes, targets sorted once.

    The reference sorts configs_j once per apply_within call (thrust /
    std::sort) and then walks T * N_i pairs; a sample that calls the oracle
    once per slice would re-sort per slice, so the sort is done here, once,
    and the timed jobs run the loop alone.
    """
    sys.path.insert(0, REPO)
    import numpy as np

    import oracle
    from oracle import ref_cuda

    oracle.build()
    dsite, dkind, dcoef = ref_cuda.daggered(site, kind, coef)
    c = lambda a, t: np.ascontiguousarray(a, dtype=t)
    _CPU.update(
        fwd=(c(site, np.int16), c(kind, np.uint8), c(coef, np.float64), c(ci, np.uint8),
             c(np.asarray(psi).view(np.float64).reshape(-1, 2), np.float64), c(cj, np.uint8)),
        adj=(c(dsite, np.int16), c(dkind, np.uint8), c(dcoef, np.float64), c(cj, np.uint8),
             c(np.asarray(g).view(np.float64).reshape(-1, 2), np.float64), c(ci, np.uint8)))
    _CPU["idx_fwd"] = oracle.sort_rows(_CPU["fwd"][5])
    _CPU["idx_adj"] = oracle.sort_rows(_CPU["adj"][5])
    _CPU["acc_fwd"] = np.zeros((cj.shape[0], 2))
    _CPU["acc_adj"] = np.zeros((ci.shape[0], 2))


def _cpu_job(job):
    """One slice of one direction: (direction, first row, end row) -> (pairs walked, seconds)."""
    import oracle

    direction, a, b = job
    site, kind, coef, src, psi, dst = _CPU[direction]
    t0 = time.perf_counter()
    oracle.apply_within_sorted(site, kind, coef, src, psi, dst, _CPU["idx_" + direction], _CPU["acc_" + direction],
                               (a, b))
    return site.shape[0] * (b - a), time.perf_counter() - t0


class CpuReference:
    """The reference's CPU apply_within (oracle port) on `cores` processes, forward and adjoint slices per step."""

    def __init__(self, wl, cores: int):
        import concurrent.futures

        import numpy as np

        rng = np.random.default_rng(7)
        g = rng.standard_normal(wl["configs_j"].shape[0]) + 1j * rng.standard_normal(wl["configs_j"].shape[0])
        self.cores = cores
        self.n_i, self.n_j = wl["configs_i"].shape[0], wl["configs_j"].shape[0]
        self.T = wl["n_terms"]
        self.pool = concurrent.futures.ProcessPoolExecutor(
            cores, mp_context=mp.get_context("spawn"), initializer=_cpu_init,
            initargs=(wl["site"], wl["kind"], wl["coef"], wl["configs_i"], wl["psi"], wl["configs_j"], g))
        self.cursor = 0

    def step(self, fraction: float) -> tuple[float, float]:
        """One sampled step: `fraction` of the forward rows and of the adjoint rows; returns (pairs, wall seconds)."""
        n_f = max(1, int(round(fraction * self.n_i)))
        n_a = max(1, int(round(fraction * self.n_j)))
        jobs = []
        for direction, n, total in (("fwd", n_f, self.n_i), ("adj", n_a, self.n_j)):
            a0 = (self.cursor * n) % max(total - n + 1, 1)
            per = -(-n // self.cores)
            for a in range(a0, a0 + n, per):
                jobs.append((direction, a, min(a + per, a0 + n)))
        self.cursor += 1
        t0 = time.perf_counter()
        done = list(self.pool.map(_cpu_job, jobs))
        wall = time.perf_counter() - t0
        return float(sum(d[0] for d in done)), wall

    def close(self):
        self.pool.shutdown()


def cpu_reference_rate(wl, budget_s: float, cores: int | None = None, fraction: float | None = None) -> dict:
    """Term applications per second of the reference's CPU algorithm over about budget_s of sampled steps."""
    cores = cores or os.cpu_count() or 1
    ref = CpuReference(wl, cores)
    try:
        frac = fraction or 0.02 * min(1.0, cores / 16)
        ref.step(frac / 4)  # starts the workers (spawn + set-up) outside the timing
        pairs = secs = 0.0
        steps = 0
        while secs < budget_s or steps == 0:
            p, w = ref.step(frac)
            pairs += p
            secs += w
            steps += 1
    finally:
        ref.close()
    return {"value": pairs / secs, "unit": "term-applications/s", "cores": cores, "kind": "port",
            "sample": f"{steps} steps of apply_within forward over {frac:.2%} of the {wl['configs_i'].shape[0]} "
                      f"configs_i rows (targets: all {wl['configs_j'].shape[0]} configs_j) and adjoint over "
                      f"{frac:.2%} of the configs_j rows (daggered table, targets: configs_i), {cores} processes, "
                      f"{secs:.1f} s, targets sorted once per process"}


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------


def max_over_ranks(values: list[float], device=None) -> list[float]:
    """Element-wise maximum of per-rank timings (the slowest rank sets the step time)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(values)
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def replica_value(units_per_rank: float, ms_per_step: float, world: int) -> float:
    """Whole-job throughput of `world` replicas that each process units_per_rank per step."""
    return world * units_per_rank / (ms_per_step * 1e-3)


def measured_peaks() -> tuple[float, str]:
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# Sources whose change invalidates a committed ncu figure of the engine's kernels.
KERNEL_SOURCES = ("qmb-public_gb300/csrc/device.cuh", "qmb-public_gb300/csrc/apply.cu",
                  "qmb-public_gb300/csrc/keys.cu", "qmb-public_gb300/csrc/relative.cu",
                  "qmb-public_gb300/csrc/format.h", "qmb-public_gb300/csrc/table.cpp")
# the sources of the apply_within walks (profiles of grouped_kernel / enumerate_kernel under apply_within)
APPLY_SOURCES = ("qmb-public_gb300/csrc/device.cuh", "qmb-public_gb300/csrc/apply.cu",
                 "qmb-public_gb300/csrc/keys.cu", "qmb-public_gb300/csrc/format.h",
                 "qmb-public_gb300/csrc/table.cpp")
# the sources of find_relative's walks
RELATIVE_SOURCES = ("qmb-public_gb300/csrc/device.cuh", "qmb-public_gb300/csrc/relative.cu",
                    "qmb-public_gb300/csrc/keys.cu", "qmb-public_gb300/csrc/format.h",
                    "qmb-public_gb300/csrc/table.cpp")


def kernel_sources_sha(sources=KERNEL_SOURCES) -> str:
    """First 16 hex digits of the SHA-256 over kernel source files (paths relative to the repo)."""
    import hashlib

    h = hashlib.sha256()
    for rel in sources:
        with open(os.path.join(REPO, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


# the committed ncu summary (profiles/<name>.json) of each workload's dominant walk kernel
WALK_FIGURES = {"c2": "term_walk_c2", "c4": "tiled_walk_c4", "c5": "pivot_walk_c5", "c3": "pivot_walk_c3"}


def ncu_figures(name: str) -> dict | None:
    """Per-launch ncu figures committed as profiles/<name>.json, or None when absent or
    taken on kernel sources other than the current ones (a stale figure is never used).
    The file names the sources its kernel is built from ("sources") and their hash at the
    capture ("kernel_sources_sha"); without a list, every file of KERNEL_SOURCES counts."""
    path = os.path.join(REPO, "profiles", f"{name}.json")
    try:
        with open(path) as f:
            figs = json.load(f)
    except (OSError, ValueError):
        return None
    try:
        current = kernel_sources_sha(tuple(figs.get("sources") or KERNEL_SOURCES))
    except OSError:
        return None
    if figs.get("kernel_sources_sha") != current:
        return None
    return figs


def issue_roofline(figs: dict | None, launch_ms: float, device, clocks: dict):
    """The walk's binding resource: warp instructions issued per second against the SMs' issue slots.

    The walk is sparse integer work (bit tests, hashing, L2 lookups), so its
    HBM fraction is small by construction; this second roofline divides the
    warp instructions of one launch (ncu, committed with the hash of the
    kernel sources it was taken on) by the live launch time, against 4 issue
    slots per SM per clock at the sampled clock.
    """
    import torch

    inst = (figs or {}).get("warp_instructions_per_launch")
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if inst is None or not mhz or launch_ms <= 0:
        return None
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    achieved = inst / (launch_ms * 1e-3)
    peak = sms * 4 * mhz * 1e6
    return {"achieved": achieved, "peak": peak, "unit": "warp-inst/s", "frac": achieved / peak,
            "warp_instructions_per_launch": inst, "sms": sms, "sm_mhz": mhz,
            "source": f"profiles/{figs.get('name', '')}.json (kernel sources {figs.get('kernel_sources_sha')})"}


def hbm_roofline(alg_bytes: float, launch_ms: float, kernel: str, figs: dict | None = None, **extra) -> dict:
    """The contract's roofline: algorithmic bytes per launch over the live launch time, against measured HBM."""
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9 if launch_ms > 0 else 0.0
    line = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": (figs or {}).get("traffic_bytes_per_launch"), "kernel": kernel,
            "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": launch_ms,
            "peak_source": f"{peak_kind} hbm_gbs"}
    line.update(extra)
    return line


def workload_config(args, wl) -> dict:
    """The config both arms report (identical dicts, so the two lines compare)."""
    return {"workload": f"{args.workload}: {wl['spec']['description']}", "n_terms": wl["n_terms"],
            "n_i": int(wl["configs_i"].shape[0]), "n_j": int(wl["configs_j"].shape[0]), "n_qubytes": wl["nq"],
            "parallelism": f"replicas x{args.gpus}", "l2": "flushed (256 MB write) before every timed step"}


def time_reference_cuda(wl, device, reps: int = 3) -> dict:
    """The reference's own CUDA apply_within (its cubin, oracle/_ref) on the same workload, forward and adjoint.

    The adjoint is what a user of the reference would run for H^dagger g: its
    apply_within on the daggered table from configs_j onto configs_i.
    """
    import numpy as np
    import torch

    from oracle import ref_cuda

    nq = wl["nq"]
    if not ref_cuda.available(nq, 1):
        return {"unavailable": f"no reference cubin for n_qubytes {nq} in oracle/_ref (built from the reference's "
                               "sources by oracle/ref_build.py where they are present)"}
    ref = ref_cuda.ReferenceCuda(nq, 1, device)
    fwd = ref.table(wl["site"], wl["kind"], wl["coef"])
    adj = ref.table(*ref_cuda.daggered(wl["site"], wl["kind"], wl["coef"]))
    ci = torch.from_numpy(wl["configs_i"]).to(device)
    cj = torch.from_numpy(wl["configs_j"]).to(device)
    psi = torch.from_numpy(wl["psi"]).to(device)
    stream = torch.cuda.current_stream(device)

    def timed(fn):
        fn()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            out = fn()
            b.record(stream)
            ts.append((a, b))
        torch.cuda.synchronize(device)
        return out, sum(a.elapsed_time(b) for a, b in ts) / reps

    y, ms_fwd = timed(lambda: ref.apply_within(fwd, ci, psi, cj))
    x, ms_adj = timed(lambda: ref.apply_within(adj, cj, y, ci))
    # kernel alone, targets presorted
    perm = ref.sort_rows(cj)
    sorted_j = cj[perm].contiguous()
    acc = torch.zeros((cj.shape[0], 2), dtype=torch.float64, device=device)
    psi_f = torch.view_as_real(psi).contiguous()

    def kernel_only():
        acc.zero_()
        ref.launch(fwd, ci, psi_f, sorted_j, acc, stream.cuda_stream)

    _, ms_kernel = timed(kernel_only)
    T = wl["n_terms"]
    units = T * (ci.shape[0] + cj.shape[0])
    return {"fwd_ms": ms_fwd, "adj_ms": ms_adj, "step_ms": ms_fwd + ms_adj, "fwd_kernel_ms": ms_kernel,
            "value": units / ((ms_fwd + ms_adj) * 1e-3), "unit": "term-applications/s",
            "y": y, "x": x,
            "what": "qmb/_hamiltonian_cuda.cu apply_within_kernel_interface from the reference's own sources "
                    "(oracle/ref_build.py), host side replayed with torch (targets sorted by a stable byte-wise "
                    "LSD sort in place of thrust::sort_by_key); adjoint = the same kernel on the daggered table "
                    "from configs_j onto configs_i"}


def run_ours(args, wl, rank: int, world: int) -> dict | None:
    import numpy as np
    import torch
    import torch.distributed as dist

    qmb = importlib.import_module("qmb-public_gb300")
    native = importlib.import_module("qmb-public_gb300._native")
    device = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(device)
    ham = qmb.Hamiltonian((torch.from_numpy(wl["site"]), torch.from_numpy(wl["kind"]), torch.from_numpy(wl["coef"])),
                          kind="fermi")
    ci = torch.from_numpy(wl["configs_i"]).to(device)
    cj = torch.from_numpy(wl["configs_j"]).to(device)
    psi64 = torch.from_numpy(wl["psi"]).to(device)
    psi32 = psi64.to(torch.complex64)
    n_i, n_j, T, nq = ci.shape[0], cj.shape[0], wl["n_terms"], wl["nq"]
    units = T * (n_i + n_j)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)  # > 129 MB of L2
    stream = torch.cuda.current_stream(device)

    # a step is apply_within and its backward (the adjoint applied to the
    # output, as in an energy-gradient step) through the autograd function:
    # the forward walk records its hits and the backward replays them.
    # FP32 pipeline: complex64 in and out, compensated accumulation inside
    def fwd_adj(psi):
        p = psi.detach().requires_grad_(True)
        y = ham.apply_within(ci, p, cj)
        return torch.autograd.grad(y, p, grad_outputs=y)[0]

    def step32():
        return fwd_adj(psi32)

    def step64():
        return fwd_adj(psi64)

    def barrier():
        if world > 1:
            dist.barrier()

    def timed(fn, steps):
        times = []
        for _ in range(steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            times.append((a, b))
        torch.cuda.synchronize(device)
        return sum(a.elapsed_time(b) for a, b in times)

    for _ in range(args.warmup):
        step32()
        step64()
    torch.cuda.synchronize(device)

    # the clock sampler runs across every timed region below (headline, FP64, end to end)
    clocks = ClockSampler(device.index)
    clocks.__enter__()

    # headline: FP32-compensated forward + adjoint; the launch counter is
    # always on, per-kernel timing is off here (its events would add to the step)
    launches0 = native.profile_read()["launches"]
    barrier()
    torch.cuda.synchronize(device)
    ms32 = timed(step32, args.steps)
    barrier()
    torch.cuda.synchronize(device)
    launches = native.profile_read()["launches"] - launches0

    ms64 = timed(step64, args.steps)

    # find_relative (top K excluding configs_i); it synchronises, so it is timed on its own
    K = wl["spec"]["count_selected"]
    ham.find_relative(ci, psi64, K)
    reps = max(1, min(args.steps, 5))
    ms_rel = timed(lambda: ham.find_relative(ci, psi64, K), reps) / reps
    rel = ham.find_relative(ci, psi64, K)

    # energy error of the FP32 path on the configs_i block
    e64 = float(qmb.variational_energy(ham, ci, psi32.to(torch.complex128)))
    e32 = float(qmb.variational_energy(ham, ci, psi32))

    # end to end through the public API with host buffers
    ci_h = torch.from_numpy(wl["configs_i"]).pin_memory()
    cj_h = torch.from_numpy(wl["configs_j"]).pin_memory()
    psi_h = torch.from_numpy(wl["psi"]).to(torch.complex64).pin_memory()
    y_h = torch.empty(n_j, dtype=torch.complex64).pin_memory()
    x_h = torch.empty(n_i, dtype=torch.complex64).pin_memory()

    def step_e2e():
        a_i = ci_h.to(device, non_blocking=True)
        a_j = cj_h.to(device, non_blocking=True)
        p = psi_h.to(device, non_blocking=True).requires_grad_(True)
        y = ham.apply_within(a_i, p, a_j)
        (x,) = torch.autograd.grad(y, p, grad_outputs=y)
        y_h.copy_(y.detach(), non_blocking=True)
        x_h.copy_(x, non_blocking=True)

    step_e2e()
    ms_e2e = timed(step_e2e, args.steps)
    clocks.__exit__(None, None, None)
    h2d = ci_h.numel() + cj_h.numel() + psi_h.numel() * 8
    d2h = y_h.numel() * 8 + x_h.numel() * 8
    ms32, ms64, ms_e2e = max_over_ranks([ms32, ms64, ms_e2e], device)

    # per-kernel-group device time, in separate profiled passes of the same step and of find_relative
    native.profile_enable(True)
    timed(step32, args.steps)
    torch.cuda.synchronize(device)
    prof = native.profile_read()
    native.profile_enable(True)
    timed(lambda: ham.find_relative(ci, psi64, K), reps)
    prof_rel = native.profile_read()
    stats_rel = native.find_relative_stats()
    native.profile_enable(False)
    n_enum, ms_enum = prof["groups"]["enumerate"]
    walks_per_step = n_enum / args.steps
    n_replay, ms_replay = prof["groups"]["spmv"]
    # hits of one forward walk (the records the backward replays)
    y_rec, record = ham._apply(ci, psi32, cj, adjoint=False, log=True)
    ham._adjoint_from_log(record, y_rec)
    hits = record.hits or 0

    if rank != 0:
        return None
    cpu = cpu_reference_rate(wl, budget_s=args.cpu_seconds) if world == 1 else None
    try:
        ref_cuda = time_reference_cuda(wl, device)
        if "y" in ref_cuda:
            y_ref, x_ref = ref_cuda.pop("y"), ref_cuda.pop("x")
            y_our = ham.apply_within(ci, psi64, cj)
            x_our = ham.apply_within_adjoint(ci, y_ref, cj)
            ref_cuda["max_abs_diff_vs_engine_fp64"] = max((y_our - y_ref).abs().max().item(),
                                                         (x_our - x_ref).abs().max().item())
            ref_cuda["engine_fp64_speedup"] = ref_cuda["step_ms"] / (ms64 / args.steps)
            ref_cuda["engine_fp32c_speedup"] = ref_cuda["step_ms"] / (ms32 / args.steps)
    except (RuntimeError, OSError) as exc:  # a missing driver entry point or cubin load failure
        ref_cuda = {"unavailable": f"{type(exc).__name__}: {exc}"}

    # roofline of the term walk: algorithmic bytes per launch
    # forward: targets N_j (key + FP64 result), sources N_i (key + FP32 amplitude), terms T (28 B)
    # adjoint: the same with the two sets swapped
    # (a step walks once, the forward, when its backward replays the hit log; twice without it)
    alg_fwd = n_j * (nq + 16) + n_i * (nq + 8) + T * 28
    alg_adj = n_i * (nq + 16) + n_j * (nq + 8) + T * 28
    alg = alg_fwd if walks_per_step < 1.5 else (alg_fwd + alg_adj) / 2
    per_launch_ms = ms_enum / max(n_enum, 1)
    figs = ncu_figures(WALK_FIGURES.get(args.workload, f"term_walk_{args.workload}"))
    ms_step32 = ms32 / args.steps
    value = replica_value(units, ms_step32, world)
    # the radix sorts of find_relative: passes x 2 x records x record bytes over their device time
    n_sort, ms_sort = prof_rel["groups"]["sort"]
    sort_bytes = stats_rel["sort_bytes"]  # per call; ms_sort covers `reps` calls
    line = {
        "metric": "apply_within term-applications/s (FP32-compensated forward + adjoint)",
        "value": value,
        "unit": "term-applications/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step32,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(args, wl),
        "roofline": hbm_roofline(alg, per_launch_ms, "term walk (grouped_kernel)", figs),
        "issue_roofline": issue_roofline(figs, per_launch_ms, device, clocks.summary()),
        "cpu_baseline": cpu,
        "e2e": {"value": world * units / (ms_e2e / args.steps * 1e-3), "unit": "term-applications/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e / args.steps},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "hit_log": {"hits_per_step": hits, "record_bytes_per_step": 16 * hits,
                    # per hit: its 16-byte record, the FP32 hi/lo coefficient (16) and g (8) it gathers;
                    # per configs_i row: the result (16, FP64 atomics) and its first row (4)
                    # (both replay kernels of a step timed together)
                    "replay_roofline": hbm_roofline(hits * 40 + n_i * 20, ms_replay / args.steps,
                                                    "hit-log replay (log_adjoint_kernel + diagonal records)",
                                                    launches_per_step=n_replay / args.steps)},
        "walked_pairs_per_s": {"value": world * walks_per_step * T * n_i / (ms_step32 * 1e-3),
                               "walks_per_step": walks_per_step,
                               "what": "(term, row) pairs the term walks visit: each walk covers configs_i's "
                                       f"{n_i} rows (T * N_i = {T * n_i:.3e}); the forward walk records its hits "
                                       "and the adjoint replays them"},
        "fp64": {"value": world * units / (ms64 / args.steps * 1e-3), "ms_per_step": ms64 / args.steps},
        "speedup_fp32c_vs_fp64": ms64 / ms32,
        "ref_cuda_fp64": ref_cuda,
        "find_relative": {"ms": ms_rel, "count_selected": K, "rows_out": int(rel.shape[0]),
                          "kernel_groups_ms": {g: prof_rel["groups"][g][1] / reps for g in prof_rel["groups"]},
                          "stats": stats_rel,
                          "sort_roofline": hbm_roofline(sort_bytes, ms_sort / reps,
                                                        "radix sort of the selected rows (radix_hist/scatter + scans)",
                                                        None, launches_per_call=n_sort / reps) if ms_sort > 0 else None},
        "energy": {"fp64": e64, "fp32c": e32, "abs_error_ha": abs(e32 - e64)},
        "kernel_groups_ms_per_step": {g: prof["groups"][g][1] / args.steps for g in prof["groups"]},
        "clock_window": "nvidia-smi every 50 ms across the FP32c, FP64, find_relative and end-to-end timed loops",
    }
    return line


class _Mlp:
    """Plain MLP wave function: unpacked bits -> 4 hidden layers of 512 (SiLU) -> (log|psi|, phase), FP32."""

    def __init__(self, n_sites: int, device, seed: int):
        import torch

        gen = torch.Generator().manual_seed(seed)
        layers = []
        width = n_sites
        for _ in range(4):
            lin = torch.nn.Linear(width, 512)
            torch.nn.init.normal_(lin.weight, std=1.0 / math.sqrt(width), generator=gen)
            torch.nn.init.zeros_(lin.bias)
            layers += [lin, torch.nn.SiLU()]
            width = 512
        head = torch.nn.Linear(512, 2)
        torch.nn.init.normal_(head.weight, std=0.01, generator=gen)
        torch.nn.init.zeros_(head.bias)
        layers.append(head)
        self.net = torch.nn.Sequential(*layers).to(device)
        self.n_sites = n_sites

    def __call__(self, configs):
        import torch

        bitspack = importlib.import_module("qmb-public_gb300.bitspack")
        bits = bitspack.unpack_int(configs, 1, self.n_sites).to(torch.float32)
        out = self.net(bits)
        return torch.polar(torch.exp(out[:, 0]), out[:, 1])


def _timed_loop(fn, steps, device, flush=None):
    """Mean milliseconds of fn over `steps` runs: CUDA events on the current stream, L2 flushed before each run."""
    import torch

    stream = torch.cuda.current_stream(device)
    pairs = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        pairs.append((a, b))
    torch.cuda.synchronize(device)
    return sum(a.elapsed_time(b) for a, b in pairs) / steps


def _profiled(native, fn, device):
    """Per-group (launches, ms) of one run of fn."""
    import torch

    native.profile_enable(True)
    fn()
    torch.cuda.synchronize(device)
    prof = native.profile_read()
    native.profile_enable(False)
    return prof


def run_extra(args, wl) -> dict:
    """The other benchmark shapes: c1 (all 400 determinants of 12 spin orbitals), c3 (energy + gradient through
    an MLP), c4 (Hubbard 1M), c5 (find_relative 1M), and the engine's callers: lanczos (20 iterations on the c3
    basis) and pt2 (one PT2 step on the c5 shape).  Every line is clocked (nvidia-smi across the timed loops),
    flushes L2 before every timed step and carries the roofline of its dominant kernel group."""
    import torch

    qmb = importlib.import_module("qmb-public_gb300")
    native = importlib.import_module("qmb-public_gb300._native")
    device = torch.device("cuda", 0)
    ham = qmb.Hamiltonian((torch.from_numpy(wl["site"]), torch.from_numpy(wl["kind"]), torch.from_numpy(wl["coef"])),
                          kind="fermi")
    ci = torch.from_numpy(wl["configs_i"]).to(device)
    cj = torch.from_numpy(wl["configs_j"]).to(device)
    T, nq, n = wl["n_terms"], wl["nq"], ci.shape[0]
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)
    line = {"config": workload_config(args, wl), "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "data": "synthetic", "vs_baseline": None, "scaling": "weak"}
    clocks = ClockSampler(device.index)
    walk_alg = lambda n_walk, n_look, amp: n_walk * (nq + 16) + n_look * (nq + amp) + T * 28

    def walk_roofline(prof, n_walk, n_look, amp, kernel):
        cnt, ms = prof["groups"]["enumerate"]
        return hbm_roofline(walk_alg(n_walk, n_look, amp), ms / max(cnt, 1), kernel,
                            ncu_figures(WALK_FIGURES.get(args.workload, f"term_walk_{args.workload}")), launches=cnt)

    if args.workload == "c3":
        mlp = _Mlp(8 * nq, device, seed=wl["spec"]["seed"])

        def step(dtype, shortcut=True, hit_log=True):
            for p in mlp.net.parameters():
                p.grad = None
            psi = mlp(ci)
            ham.hit_log = hit_log
            try:
                e = qmb.variational_energy(ham, ci, psi if dtype == torch.complex64 else psi.to(torch.complex128),
                                           hermitian_shortcut=shortcut)
                e.backward()
            finally:
                ham.hit_log = True
            return e

        # three backwards: the Hermitian shortcut (default), the forward walk's hit log replayed,
        # and the adjoint kernel's own walk
        for _ in range(args.warmup):
            step(torch.complex64)
            step(torch.complex128)
            step(torch.complex64, False)
            step(torch.complex64, False, False)
        with clocks:
            ms32 = _timed_loop(lambda: step(torch.complex64), args.steps, device, flush)
            ms64 = _timed_loop(lambda: step(torch.complex128), args.steps, device, flush)
            ms32_log = _timed_loop(lambda: step(torch.complex64, False), args.steps, device, flush)
            ms32_adj = _timed_loop(lambda: step(torch.complex64, False, False), args.steps, device, flush)
            ms64_adj = _timed_loop(lambda: step(torch.complex128, False, False), args.steps, device, flush)
        prof = _profiled(native, lambda: step(torch.complex64), device)
        prof_log = _profiled(native, lambda: step(torch.complex64, False), device)
        prof_adj = _profiled(native, lambda: step(torch.complex64, False, False), device)
        e32 = float(step(torch.complex64).detach())
        e64 = float(step(torch.complex128).detach())
        line.update({"metric": "energy forward + backward step (FP32-compensated)", "value": ms32, "unit": "ms",
                     "ms_per_step": ms32, "higher_is_better": False, "dtype": "f32", "fp64_ms": ms64,
                     "speedup_fp32c_vs_fp64": ms64 / ms32,
                     "through_hit_log": {"fp32c_ms": ms32_log,
                                         "walks_per_step": prof_log["groups"]["enumerate"][0],
                                         "kernel_groups_ms": {g: v[1] for g, v in prof_log["groups"].items()}},
                     "through_adjoint_kernel": {"fp32c_ms": ms32_adj, "fp64_ms": ms64_adj,
                                                "speedup_fp32c_vs_fp64": ms64_adj / ms32_adj,
                                                "walks_per_step": prof_adj["groups"]["enumerate"][0],
                                                "kernel_groups_ms": {g: v[1] for g, v in prof_adj["groups"].items()}},
                     "energy_fp64": e64, "energy_fp32c": e32, "energy_abs_error_ha": abs(e32 - e64),
                     "hermitian": ham._table(device, nq).hermitian,
                     "walks_per_step": prof["groups"]["enumerate"][0],
                     "roofline": walk_roofline(prof, n, n, 8, "term walk (pivot_kernel)"),
                     "kernel_groups_ms_per_step": {g: v[1] for g, v in prof["groups"].items()}})
    elif args.workload in ("c1", "c4"):
        psi32 = torch.from_numpy(wl["psi"]).to(torch.complex64).to(device)
        psi64 = psi32.to(torch.complex128)

        # forward + adjoint as in the headline workload: apply_within's autograd function, whose
        # backward replays the forward walk's hits
        def fwd_adj(psi):
            p = psi.detach().requires_grad_(True)
            y = ham.apply_within(ci, p, cj)
            return torch.autograd.grad(y, p, grad_outputs=y)[0]

        step32 = lambda: fwd_adj(psi32)
        step64 = lambda: fwd_adj(psi64)

        for _ in range(args.warmup):
            step32()
            step64()
        with clocks:
            ms32 = _timed_loop(step32, args.steps, device, flush)
            ms64 = _timed_loop(step64, args.steps, device, flush)
        prof = _profiled(native, step32, device)
        e32 = float(qmb.variational_energy(ham, ci, psi32))
        e64 = float(qmb.variational_energy(ham, ci, psi64))
        units = T * (ci.shape[0] + cj.shape[0])
        line.update({"metric": "apply_within term-applications/s (FP32-compensated forward + adjoint)",
                     "value": units / (ms32 * 1e-3), "unit": "term-applications/s", "higher_is_better": True,
                     "dtype": "f32", "ms_per_step": ms32, "fp64_ms_per_step": ms64,
                     "speedup_fp32c_vs_fp64": ms64 / ms32,
                     "energy_fp64": e64, "energy_fp32c": e32, "energy_abs_error_ha": abs(e32 - e64),
                     "walks_per_step": prof["groups"]["enumerate"][0],
                     "roofline": walk_roofline(prof, n, cj.shape[0], 8, "term walk"),
                     "kernel_groups_ms_per_step": {g: v[1] for g, v in prof["groups"].items()}})
    elif args.workload == "lanczos":
        n_steps = wl["spec"]["lanczos_steps"]
        gen = torch.Generator(device=device).manual_seed(wl["spec"]["seed"])
        start = torch.randn([n], dtype=torch.complex128, device=device, generator=gen)
        for _ in range(args.warmup):
            qmb.lanczos_energy(ham, ci, 2, start=start)
        result = {}

        def run():
            result["e"] = qmb.lanczos_energy(ham, ci, n_steps, start=start)[0]

        with clocks:
            ms = _timed_loop(run, args.steps, device, flush)
            ms_walks = _timed_loop(lambda: qmb.lanczos_energy(ham, ci, n_steps, start=start, materialize=False),
                                   max(1, args.steps // 5), device, flush)
        prof = _profiled(native, run, device)
        mat = ham.matrix(ci)
        n_spmv, ms_spmv = prof["groups"]["spmv"]
        # a product reads every entry (16-byte value, 4-byte column), the row pointers, x through the columns
        # (at least once per row) and writes y
        spmv_bytes = mat.nnz * 20 + (n + 1) * 8 + 2 * n * 16
        line.update({"metric": "Lanczos wall time (20 iterations, FP64, Ritz value on the host)", "value": ms,
                     "unit": "ms", "ms_per_step": ms, "higher_is_better": False, "dtype": "f64",
                     "ms_per_iteration": ms / (n_steps + 2), "energy": result["e"],
                     "matrix": {"nnz": mat.nnz, "walks_to_build": prof["groups"]["enumerate"][0],
                                "build_ms": prof["groups"]["enumerate"][1] + prof["groups"]["diagonal"][1],
                                "products": n_spmv},
                     "through_walks_ms": ms_walks,
                     "roofline": hbm_roofline(spmv_bytes, ms_spmv / max(n_spmv, 1),
                                              "sparse matrix-vector product (spmv_kernel)", None, launches=n_spmv),
                     "kernel_groups_ms_per_run": {g: v[1] for g, v in prof["groups"].items()}})
    elif args.workload == "pt2":
        psi = torch.from_numpy(wl["psi"]).to(device)
        K = wl["spec"]["count_selected"]
        for _ in range(args.warmup):
            qmb.pt2_energy(ham, ci, psi, K)
        result = {}

        def run():
            result["e"] = qmb.pt2_energy(ham, ci, psi, K)

        with clocks:
            ms = _timed_loop(run, args.steps, device, flush)
        prof = _profiled(native, run, device)
        line.update({"metric": "PT2 step wall time (E0, selection of the connected space, H psi on it, "
                               "denominators, Epstein-Nesbet sum)", "value": ms, "unit": "ms", "ms_per_step": ms,
                     "higher_is_better": False, "dtype": "f64", "count_selected": K, "e0": result["e"][0],
                     "e2": result["e"][1],
                     "roofline": walk_roofline(prof, n, n, 16, "term walk"),
                     "kernel_groups_ms_per_run": {g: v[1] for g, v in prof["groups"].items()}})
    elif args.workload == "sampler":
        from oracle import sampler as oracle_sampler

        spec = wl["spec"]
        sites = spec["n_orbit"]
        torch.manual_seed(spec["seed"])
        net = qmb.sampler.WaveFunctionElectronUpDown(double_sites=2 * sites, physical_dim=2, is_complex=True,
                                                     spin_up=spec["n_alpha"], spin_down=spec["n_beta"],
                                                     hidden_size=spec["hidden"], ordering=+1).to(device)
        params = {k: v.detach() for k, v in net.state_dict().items()}
        batch = spec["n_i"]
        for _ in range(args.warmup):
            net.generate_unique(batch)
        out = {}

        def run():
            out["n"] = net.generate_unique(batch)[0].shape[0]

        def run_ref():
            oracle_sampler.generate_unique(params, sites, spec["n_alpha"], spec["n_beta"], batch,
                                           lambda site, rows: torch.rand((rows, 4), device=device))

        run_ref()
        with clocks:
            ms = _timed_loop(run, args.steps, device, flush)
            ms_ref = _timed_loop(run_ref, max(1, args.steps // 2), device, flush)
        prof = _profiled(native, run, device)
        line.update({"metric": "generate_unique wall time (65,536 configurations)", "value": ms, "unit": "ms",
                     "ms_per_step": ms, "higher_is_better": False, "dtype": "f32", "rows_out": out["n"],
                     "reference_algorithm_torch_ms": ms_ref, "speedup_vs_reference_algorithm": ms_ref / ms,
                     "reference_algorithm": "oracle/sampler.py: the reference's generate_unique restated in plain "
                                            "torch (pinned to the reference's own outputs), same GPU, same network",
                     "kernel_groups_ms_per_run": {g: v[1] for g, v in prof["groups"].items()}})
    else:  # c5: find_relative
        psi = torch.from_numpy(wl["psi"]).to(device)
        K = wl["spec"]["count_selected"]
        rel = ham.find_relative(ci, psi, K)
        for _ in range(args.warmup):
            rel = ham.find_relative(ci, psi, K)
        with clocks:
            ms = _timed_loop(lambda: ham.find_relative(ci, psi, K), args.steps, device, flush)
        prof = _profiled(native, lambda: ham.find_relative(ci, psi, K), device)
        stats = native.find_relative_stats()
        n_sort, ms_sort = prof["groups"]["sort"]
        line.update({"metric": "find_relative wall time (top K of all connected records)", "value": ms, "unit": "ms",
                     "ms_per_step": ms, "higher_is_better": False, "dtype": "f64", "count_selected": K,
                     "rows_out": int(rel.shape[0]), "term_applications_per_s": T * n / (ms * 1e-3),
                     "stats": stats,
                     "roofline": walk_roofline(prof, n, ci.shape[0], 16, "term walk (pivot_kernel)"),
                     "sort_roofline": hbm_roofline(stats["sort_bytes"], ms_sort, "radix sort of the selected rows",
                                                   None, launches_per_call=n_sort) if ms_sort > 0 else None,
                     "kernel_groups_ms_per_run": {g: v[1] for g, v in prof["groups"].items()}})
    line["clocks"] = clocks.summary()
    return line


def run_reference(args, wl) -> dict:
    """The reference arm: the reference's CPU algorithm on every host core, K sampled steps after W warm-up ones.

    Each step walks the same fraction of the forward rows (configs_i against
    configs_j) and of the adjoint rows (configs_j against configs_i with the
    daggered table, the reference's way to apply H^dagger), split across the
    host cores; the value is the pairs walked over the wall time.  A 1-core
    figure rides along (the reference's CPU loops are serial).
    """
    cores = os.cpu_count() or 1
    frac = args.ref_fraction
    ref = CpuReference(wl, cores)
    try:
        for _ in range(max(args.warmup, 1)):
            ref.step(frac)
        pairs = secs = 0.0
        times = []
        for _ in range(args.steps):
            p, w = ref.step(frac)
            pairs += p
            secs += w
            times.append(w)
    finally:
        ref.close()
    value = pairs / secs
    one = cpu_reference_rate(wl, budget_s=2.0, cores=1, fraction=frac / 16)
    n_i, n_j = wl["configs_i"].shape[0], wl["configs_j"].shape[0]
    sample = (f"each step: apply_within forward over {frac:.2%} of the {n_i} configs_i rows (targets: all {n_j} "
              f"configs_j) and adjoint over {frac:.2%} of the {n_j} configs_j rows (daggered table, targets: "
              f"configs_i), split over {cores} processes; targets sorted once per process")
    return {
        "impl": "reference",
        "metric": "apply_within term-applications/s (FP32-compensated forward + adjoint)",
        "value": value,
        "unit": "term-applications/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": secs * 1e3 / max(args.steps, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": workload_config(args, wl),
        "cpu_baseline": {"value": value, "unit": "term-applications/s", "cores": cores, "kind": "port",
                         "sample": sample, "one_core": one,
                         "step_ms_min_max": [min(times) * 1e3, max(times) * 1e3]},
        "e2e": {"value": value, "unit": "term-applications/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "what": "the oracle port of qmb/_hamiltonian_cpu.cpp (bit-identical results; within 16 % of the "
                "reference's own build on one core where both run), on a sample of every step",
    }


def main():
    parser = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=50)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", choices=["ours", "reference"], default="ours")
    parser.add_argument("--workload", choices=sorted(WORKLOADS), default="c2")
    parser.add_argument("--cpu-seconds", type=float, default=8.0, help="wall budget of the cpu_baseline sample")
    parser.add_argument("--ref-fraction", type=float, default=0.02,
                        help="fraction of each direction's rows a reference-arm step walks")
    args = parser.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        if rank != 0:
            return
        wl = make_workload(args.workload)
        print(json.dumps(run_reference(args, wl)), flush=True)
        return

    import torch

    if args.workload in ("c1", "c3", "c4", "c5", "lanczos", "pt2", "sampler"):
        if rank == 0:
            print(json.dumps(run_extra(args, make_workload(args.workload))), flush=True)
        return
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    wl = make_workload(args.workload)
    line = run_ours(args, wl, rank, world)
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
