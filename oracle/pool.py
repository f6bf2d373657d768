"""The oracle split across host processes — TEST INFRASTRUCTURE ONLY.

The benchmark workloads' full sizes (C2: 55,371 terms x 20,000 sources
against 200,000 targets) take the single-threaded oracle tens of seconds per
operator.  Every operator here splits its independent axis into row ranges,
runs each range in a process of a ``spawn`` pool (never ``fork``: a pool
forked after the first CUDA call hangs) and merges:

* apply_within: sources split, results summed (linearity);
* apply_within_adjoint: output rows split, results concatenated;
* find_relative (ranked rule): sources split, each range keeps its top K
  under the ranked total order, the union's top K is the answer;
* dense matrix: columns split.

Only tests/ and bench.py's CPU legs use this module.
"""

from __future__ import annotations

import concurrent.futures
import multiprocessing as mp
import os

import numpy as np

from . import apply_within, apply_within_adjoint, dense_columns, relative_top_records, rows_with_weight


def _ranges(n: int, parts: int) -> list[tuple[int, int]]:
    parts = max(1, min(parts, n))
    edges = np.linspace(0, n, parts + 1).astype(np.int64)
    return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]


def _procs(procs: int | None) -> int:
    return procs or os.cpu_count() or 1


def _run(fn, jobs, procs):
    # an executor, not a Pool: a worker that dies raises BrokenProcessPool
    # here instead of leaving map() waiting forever
    if len(jobs) == 1:
        return [fn(jobs[0])]
    with concurrent.futures.ProcessPoolExecutor(min(procs, len(jobs)), mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(fn, jobs))


def _apply_job(a):
    site, kind, coef, ci, psi, cj, pc = a
    return apply_within(site, kind, coef, ci, psi, cj, pc)


def apply_within_par(site, kind, coef, configs_i, psi_i, configs_j, particle_cut: int = 1, procs=None, parts=None):
    procs = _procs(procs)
    jobs = [(site, kind, coef, configs_i[a:b], psi_i[a:b], configs_j, particle_cut)
            for a, b in _ranges(configs_i.shape[0], parts or 4 * procs)]
    return np.sum(_run(_apply_job, jobs, procs), axis=0)


def _adjoint_job(a):
    site, kind, coef, ci, cj, g, pc, rows = a
    return apply_within_adjoint(site, kind, coef, ci, cj, g, pc, rows)


def apply_within_adjoint_par(site, kind, coef, configs_i, configs_j, g_j, particle_cut: int = 1, procs=None):
    procs = _procs(procs)
    jobs = [(site, kind, coef, configs_i, configs_j, g_j, particle_cut, r)
            for r in _ranges(configs_i.shape[0], 4 * procs)]
    return np.concatenate(_run(_adjoint_job, jobs, procs))


def _top_job(a):
    site, kind, coef, ci, psi, k, ex, pc, rows = a
    return relative_top_records(site, kind, coef, ci, psi, k, ex, pc, rows)


def _tie_job(a):
    site, kind, coef, ci, psi, ex, pc, w = a
    return rows_with_weight(site, kind, coef, ci, psi, w, ex, pc)


def find_relative_ranked_par(site, kind, coef, configs_i, psi_i, count_selected: int, configs_exclude=None,
                             particle_cut: int = 1, procs=None):
    """(rows, kth_weight): find_relative under the ranked rule, sources split across processes."""
    procs = _procs(procs)
    ex = configs_i if configs_exclude is None else configs_exclude
    k = int(count_selected)
    if k <= 0:
        return np.zeros((0, configs_i.shape[1]), dtype=np.uint8), 0.0
    jobs = [(site, kind, coef, configs_i, psi_i, k, ex, particle_cut, r)
            for r in _ranges(configs_i.shape[0], 4 * procs)]
    parts = _run(_top_job, jobs, procs)
    w = np.concatenate([p[0] for p in parts])
    o = np.concatenate([p[1] for p in parts])
    r = np.concatenate([p[2] for p in parts])
    # lexsort's last key is primary: weight descending, then visiting order descending
    order = np.lexsort((~o, -w))
    keep = order[:k]
    kth = float(w[keep[-1]]) if keep.size else 0.0
    rows = np.unique(r[keep], axis=0) if keep.size else np.zeros((0, configs_i.shape[1]), dtype=np.uint8)
    return rows, kth


def tie_rows_par(site, kind, coef, configs_i, psi_i, weight: float, configs_exclude=None, particle_cut: int = 1,
                 procs=None):
    """Distinct rows of every record of exactly `weight` (the boundary-tie class), sources split."""
    procs = _procs(procs)
    ex = configs_i if configs_exclude is None else configs_exclude
    jobs = [(site, kind, coef, configs_i[a:b], psi_i[a:b], ex, particle_cut, weight)
            for a, b in _ranges(configs_i.shape[0], 4 * procs)]
    parts = [p for p in _run(_tie_job, jobs, procs) if p.shape[0]]
    if not parts:
        return np.zeros((0, configs_i.shape[1]), dtype=np.uint8)
    return np.unique(np.concatenate(parts), axis=0)


def _dense_job(a):
    site, kind, coef, c, pc, cols = a
    return dense_columns(site, kind, coef, c, cols, pc)


def dense_matrix_par(site, kind, coef, configs, particle_cut: int = 1, procs=None):
    procs = _procs(procs)
    jobs = [(site, kind, coef, configs, particle_cut, r) for r in _ranges(configs.shape[0], 4 * procs)]
    return np.concatenate(_run(_dense_job, jobs, procs), axis=1)
