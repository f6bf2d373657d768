"""Benchmark of the Hamiltonian engine's hot path on one GB300.

Default workload (``--workload c2``): a synthetic ab-initio Hamiltonian on 28
spin orbitals (14 spatial, n_qubytes 4; 55,371 normal-ordered terms from
seeded integrals), configs_i = 20,000 and configs_j = 200,000 unique random
determinants with 5 alpha + 5 beta electrons, complex N(0,1) amplitudes.

One step is the FP32-compensated apply_within forward (configs_i ->
configs_j) followed by its adjoint (configs_j -> configs_i), i.e. the work of
one energy-gradient evaluation.  The metric is term applications per second,
T * (N_i + N_j) per step (the reference's thread grid is T * N_i for a
forward application).  The same line reports the FP64 path, find_relative
(top 50,000 excluding configs_i), the energy error of the FP32 path, the
end-to-end rate through the public API with host buffers, the roofline of the
enumeration kernel, and the CPU oracle's rate on the host cores.

``--impl reference`` times the CPU restatement of the reference engine
(oracle/, the reference's own CPU code cannot be built on the GPU host) on a
bounded sample of the same workload with every host core.
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
                                "20 Lanczos iterations"),
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
# CPU oracle timing (reference arm and cpu_baseline)
# ---------------------------------------------------------------------------


def _oracle_worker(args):
    site, kind, coef, rows, psi, configs_j, budget_s, chunk = args
    sys.path.insert(0, REPO)
    import oracle

    done = 0
    start = time.perf_counter()
    while done < rows.shape[0] and time.perf_counter() - start < budget_s:
        hi = min(done + chunk, rows.shape[0])
        oracle.apply_within(site, kind, coef, rows[done:hi], psi[done:hi], configs_j)
        done = hi
    return done, time.perf_counter() - start


def oracle_rate(wl, budget_s: float, cores: int | None = None) -> dict:
    """Term applications per second of the CPU oracle's apply_within, every host core on a row slice."""
    import numpy as np

    import oracle

    oracle.build()
    cores = cores or os.cpu_count() or 1
    rows = wl["configs_i"]
    psi = wl["psi"]
    slices = np.array_split(np.arange(rows.shape[0]), cores)
    chunk = 16
    jobs = [(wl["site"], wl["kind"], wl["coef"], rows[s], psi[s], wl["configs_j"], budget_s, chunk) for s in slices]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        results = pool.map(_oracle_worker, jobs)
    done = sum(r[0] for r in results)
    elapsed = max(r[1] for r in results)
    rate = wl["n_terms"] * done / elapsed
    return {"value": rate, "unit": "term-applications/s", "cores": cores, "kind": "port",
            "sample": f"apply_within forward of {done} of {rows.shape[0]} configs_i rows against all "
                      f"{wl['configs_j'].shape[0]} configs_j, {cores} processes, {elapsed:.1f} s"}


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


def ncu_figure(workload: str, name: str):
    """A per-launch figure of the term walk (`name: value`) from the committed ncu summary, or None."""
    path = os.path.join(REPO, "profiles", f"term_walk_{workload}.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(name + r":\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


def ncu_traffic(workload: str):
    """DRAM bytes per enumeration launch from the committed ncu summary, or None."""
    return ncu_figure(workload, "traffic_bytes_per_launch")


def issue_roofline(workload: str, launch_ms: float, device, clocks: dict):
    """The walk's binding resource: warp instructions issued per second against the SMs' issue slots.

    The walk is sparse integer work (bit tests, hashing, L2 lookups), so its
    HBM fraction is small by construction; this second roofline divides the
    warp instructions of one launch (ncu, committed summary) by the live
    launch time, against 4 issue slots per SM per clock at the sampled clock.
    """
    import torch

    inst = ncu_figure(workload, "warp_instructions_per_launch")
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if inst is None or not mhz or launch_ms <= 0:
        return None
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    achieved = inst / (launch_ms * 1e-3)
    peak = sms * 4 * mhz * 1e6
    return {"achieved": achieved, "peak": peak, "unit": "warp-inst/s", "frac": achieved / peak,
            "warp_instructions_per_launch": inst, "sms": sms, "sm_mhz": mhz}


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

    # the FP32 pipeline: complex64 in and out, compensated accumulation inside
    def step32():
        y = ham.apply_within(ci, psi32, cj)
        return ham.apply_within_adjoint(ci, y, cj)

    def step64():
        y = ham.apply_within(ci, psi64, cj)
        return ham.apply_within_adjoint(ci, y, cj)

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

    # find_relative (top K excluding configs_i)
    K = wl["spec"]["count_selected"]
    ham.find_relative(ci, psi64, K)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    reps = max(1, min(args.steps, 5))
    for _ in range(reps):
        rel = ham.find_relative(ci, psi64, K)
    torch.cuda.synchronize(device)
    ms_rel = (time.perf_counter() - t0) * 1e3 / reps

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
        p = psi_h.to(device, non_blocking=True)
        y = ham.apply_within(a_i, p, a_j)
        x = ham.apply_within_adjoint(a_i, y, a_j)
        y_h.copy_(y, non_blocking=True)
        x_h.copy_(x, non_blocking=True)

    step_e2e()
    ms_e2e = timed(step_e2e, args.steps)
    clocks.__exit__(None, None, None)
    h2d = ci_h.numel() + cj_h.numel() + psi_h.numel() * 8
    d2h = y_h.numel() * 8 + x_h.numel() * 8
    ms32, ms64, ms_e2e = max_over_ranks([ms32, ms64, ms_e2e], device)

    # per-kernel-group device time, in a separate profiled pass of the same step
    native.profile_enable(True)
    timed(step32, args.steps)
    torch.cuda.synchronize(device)
    prof = native.profile_read()
    native.profile_enable(False)
    n_enum, ms_enum = prof["groups"]["enumerate"]

    if rank != 0:
        return None
    cpu = oracle_rate(wl, budget_s=args.cpu_seconds) if world == 1 else None

    # roofline of the enumeration kernel: algorithmic bytes per launch
    # forward: targets N_j (key + FP64 result), sources N_i (key + FP32 amplitude), terms T (28 B)
    # adjoint: the same with the two sets swapped
    alg_fwd = n_j * (nq + 16) + n_i * (nq + 8) + T * 28
    alg_adj = n_i * (nq + 16) + n_j * (nq + 8) + T * 28
    alg = (alg_fwd + alg_adj) / 2
    per_launch_ms = ms_enum / max(n_enum, 1)
    peak, peak_kind = measured_peaks()
    achieved = alg / (per_launch_ms * 1e-3) / 1e9
    ms_step32 = ms32 / args.steps
    value = replica_value(units, ms_step32, world)
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
        "config": {"workload": f"{args.workload}: {wl['spec']['description']}", "n_terms": T, "n_i": n_i, "n_j": n_j,
                   "n_qubytes": nq, "parallelism": f"replicas x{world}",
                   "l2": "flushed (256 MB write) before every timed step"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": ncu_traffic(args.workload), "kernel": "term walk (grouped_kernel)",
                     "algorithmic_bytes_per_launch": alg, "launch_ms": per_launch_ms,
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "issue_roofline": issue_roofline(args.workload, per_launch_ms, device, clocks.summary()),
        "cpu_baseline": cpu,
        "e2e": {"value": world * units / (ms_e2e / args.steps * 1e-3), "unit": "term-applications/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e / args.steps},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "fp64": {"value": world * units / (ms64 / args.steps * 1e-3), "ms_per_step": ms64 / args.steps},
        "speedup_fp32c_vs_fp64": ms64 / ms32,
        "find_relative": {"ms": ms_rel, "count_selected": K, "rows_out": int(rel.shape[0])},
        "energy": {"fp64": e64, "fp32c": e32, "abs_error_ha": abs(e32 - e64)},
        "kernel_groups_ms_per_step": {g: prof["groups"][g][1] / args.steps for g in prof["groups"]},
        "clock_window": "nvidia-smi every 50 ms across the FP32c, FP64 and end-to-end timed loops",
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


def run_extra(args, wl) -> dict:
    """The other benchmark shapes: c3 (energy + gradient through an MLP), c4 (Hubbard 1M), c5 (find_relative 1M),
    and the engine's callers: lanczos (20 iterations on the c3 basis) and pt2 (one PT2 step on the c5 shape)."""
    import torch

    qmb = importlib.import_module("qmb-public_gb300")
    native = importlib.import_module("qmb-public_gb300._native")
    device = torch.device("cuda", 0)
    kind = "fermi"
    ham = qmb.Hamiltonian((torch.from_numpy(wl["site"]), torch.from_numpy(wl["kind"]), torch.from_numpy(wl["coef"])),
                          kind=kind)
    ci = torch.from_numpy(wl["configs_i"]).to(device)
    T, nq, n = wl["n_terms"], wl["nq"], ci.shape[0]
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)
    line = {"workload": f"{args.workload}: {wl['spec']['description']}", "n_terms": T, "n_rows": n, "n_qubytes": nq}
    if args.workload == "c3":
        mlp = _Mlp(8 * nq, device, seed=wl["spec"]["seed"])

        def step(dtype):
            for p in mlp.net.parameters():
                p.grad = None
            psi = mlp(ci)
            e = qmb.variational_energy(ham, ci, psi if dtype == torch.complex64 else psi.to(torch.complex128))
            e.backward()
            return e

        for _ in range(args.warmup):
            step(torch.complex64)
            step(torch.complex128)
        native.profile_enable(True)
        ms32 = _timed_loop(lambda: step(torch.complex64), args.steps, device, flush)
        prof = native.profile_read()
        native.profile_enable(False)
        ms64 = _timed_loop(lambda: step(torch.complex128), args.steps, device, flush)
        e32 = float(step(torch.complex64).detach())
        e64 = float(step(torch.complex128).detach())
        line.update({"metric": "energy forward + backward step (FP32-compensated)", "value": ms32, "unit": "ms",
                     "higher_is_better": False, "fp64_ms": ms64, "speedup_fp32c_vs_fp64": ms64 / ms32,
                     "energy_fp64": e64, "energy_fp32c": e32, "energy_abs_error_ha": abs(e32 - e64),
                     "hermitian": ham._table(device, nq).hermitian,
                     "walks_per_step": prof["groups"]["enumerate"][0] / args.steps,
                     "apply_term_applications_per_s": prof["groups"]["enumerate"][0] * T * n / (prof["groups"]["enumerate"][1] * 1e-3),
                     "kernel_groups_ms_per_step": {g: prof["groups"][g][1] / args.steps for g in prof["groups"]}})
    elif args.workload == "c4":
        psi32 = torch.from_numpy(wl["psi"]).to(torch.complex64).to(device)
        psi64 = psi32.to(torch.complex128)

        def step32():
            y = ham.apply_within(ci, psi32, ci)
            return ham.apply_within_adjoint(ci, y, ci)

        def step64():
            y = ham.apply_within(ci, psi64, ci)
            return ham.apply_within_adjoint(ci, y, ci)

        for _ in range(args.warmup):
            step32()
            step64()
        ms32 = _timed_loop(step32, args.steps, device, flush)
        ms64 = _timed_loop(step64, args.steps, device, flush)
        e32 = float(qmb.variational_energy(ham, ci, psi32))
        e64 = float(qmb.variational_energy(ham, ci, psi64))
        line.update({"metric": "apply_within term-applications/s (FP32-compensated forward + adjoint)",
                     "value": 2 * T * n / (ms32 * 1e-3), "unit": "term-applications/s", "higher_is_better": True,
                     "ms_per_step": ms32, "fp64_ms_per_step": ms64, "speedup_fp32c_vs_fp64": ms64 / ms32,
                     "energy_fp64": e64, "energy_fp32c": e32, "energy_abs_error_ha": abs(e32 - e64)})
    elif args.workload == "lanczos":
        n_steps = wl["spec"]["lanczos_steps"]
        gen = torch.Generator(device=device).manual_seed(wl["spec"]["seed"])
        start = torch.randn([n], dtype=torch.complex128, device=device, generator=gen)
        for _ in range(args.warmup):
            qmb.lanczos_energy(ham, ci, 2, start=start)
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            energy, _vec = qmb.lanczos_energy(ham, ci, n_steps, start=start)
        torch.cuda.synchronize(device)
        ms = (time.perf_counter() - t0) * 1e3 / args.steps
        native.profile_enable(True)
        qmb.lanczos_energy(ham, ci, n_steps, start=start)
        torch.cuda.synchronize(device)
        prof = native.profile_read()
        native.profile_enable(False)
        n_apply = n_steps + 2
        line.update({"metric": "Lanczos wall time (20 iterations, FP64, Ritz value on the host)", "value": ms,
                     "unit": "ms", "higher_is_better": False, "ms_per_iteration": ms / n_apply,
                     "energy": energy, "apply_within_calls": n_apply,
                     "term_applications_per_s": n_apply * T * n / (ms * 1e-3),
                     "kernel_groups_ms_per_run": {g: prof["groups"][g][1] for g in prof["groups"]}})
    elif args.workload == "pt2":
        psi = torch.from_numpy(wl["psi"]).to(device)
        K = wl["spec"]["count_selected"]
        for _ in range(args.warmup):
            qmb.pt2_energy(ham, ci, psi, K)
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e0, e2 = qmb.pt2_energy(ham, ci, psi, K)
        torch.cuda.synchronize(device)
        ms = (time.perf_counter() - t0) * 1e3 / args.steps
        native.profile_enable(True)
        qmb.pt2_energy(ham, ci, psi, K)
        torch.cuda.synchronize(device)
        prof = native.profile_read()
        native.profile_enable(False)
        line.update({"metric": "PT2 step wall time (E0, find_relative, H psi on the selected rows, denominators)",
                     "value": ms, "unit": "ms", "higher_is_better": False, "count_selected": K, "e0": e0, "e2": e2,
                     "kernel_groups_ms_per_run": {g: prof["groups"][g][1] for g in prof["groups"]}})
    else:
        psi = torch.from_numpy(wl["psi"]).to(device)
        K = wl["spec"]["count_selected"]
        rel = ham.find_relative(ci, psi, K)
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rel = ham.find_relative(ci, psi, K)
        torch.cuda.synchronize(device)
        ms = (time.perf_counter() - t0) * 1e3 / args.steps
        line.update({"metric": "find_relative wall time (top K of all connected records)", "value": ms, "unit": "ms",
                     "higher_is_better": False, "count_selected": K, "rows_out": int(rel.shape[0]),
                     "term_applications_per_s": T * n / (ms * 1e-3)})
    line.update({"steps": args.steps, "warmup": args.warmup, "dtype": "f32", "data": "synthetic"})
    return line


def run_reference(args, wl) -> dict:
    cpu = oracle_rate(wl, budget_s=args.cpu_seconds)
    value = cpu["value"]
    return {
        "impl": "reference",
        "metric": "apply_within term-applications/s (FP32-compensated forward + adjoint)",
        "value": value,
        "unit": "term-applications/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": wl["n_terms"] * (wl["configs_i"].shape[0] + wl["configs_j"].shape[0]) / value * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: {wl['spec']['description']}", "n_terms": wl["n_terms"],
                   "n_i": int(wl["configs_i"].shape[0]), "n_j": int(wl["configs_j"].shape[0]),
                   "n_qubytes": wl["nq"]},
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": "term-applications/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    parser = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=50)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", choices=["ours", "reference"], default="ours")
    parser.add_argument("--workload", choices=sorted(WORKLOADS), default="c2")
    parser.add_argument("--cpu-seconds", type=float, default=8.0, help="wall budget of the CPU oracle sample")
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

    if args.workload in ("c3", "c4", "c5", "lanczos", "pt2"):
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
