"""CPU oracle of the Hamiltonian engine — TEST INFRASTRUCTURE ONLY.

This package wraps ``oracle.c`` (a plain-C restatement of the reference
engine, qmb/_hamiltonian_cpu.cpp and qmb/_hamiltonian_cuda.cu) with ctypes.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import it; the product path never does.

All functions take numpy arrays in the reference's layouts:
``site`` int16[T, 4], ``kind`` uint8[T, 4], ``coef`` float64[T, 2],
configurations uint8[N, n_qubytes], amplitudes complex128[N].
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib: ctypes.CDLL | None = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc only)."""
    src = os.path.join(_HERE, "oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB_PATH


def _load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(_LIB_PATH)
        p = ctypes.c_void_p
        i64 = ctypes.c_int64
        i32 = ctypes.c_int
        lib.oracle_apply_term.argtypes = [i32, i32, p, p, p, p]
        lib.oracle_apply_term.restype = i32
        lib.oracle_apply_within.argtypes = [i32, i32, i64, p, p, p, i64, p, p, i64, p, p]
        lib.oracle_diagonal_term.argtypes = [i32, i32, i64, p, p, p, i64, p, p]
        lib.oracle_find_relative_heap.argtypes = [i32, i32, i64, p, p, p, i64, p, p, i64, i64, p, p]
        lib.oracle_find_relative_heap.restype = i64
        lib.oracle_find_relative_ranked.argtypes = [i32, i32, i64, p, p, p, i64, p, p, i64, i64, p, p, p]
        lib.oracle_find_relative_ranked.restype = i64
        lib.oracle_rows_with_weight.argtypes = [i32, i32, i64, p, p, p, i64, p, p, i64, p, ctypes.c_double, i64, p]
        lib.oracle_rows_with_weight.restype = i64
        lib.oracle_term_uniform.argtypes = [ctypes.c_uint64, i64]
        lib.oracle_term_uniform.restype = ctypes.c_double
        lib.oracle_single_relative.argtypes = [i32, i32, i64, p, p, p, i64, p, ctypes.c_uint64, p, p, p]
        lib.oracle_dense_matrix.argtypes = [i32, i32, i64, p, p, p, i64, p, p]
        lib.oracle_apply_within_adjoint.argtypes = [i32, i32, i64, p, p, p, i64, i64, p, i64, p, p, p]
        lib.oracle_relative_top_records.argtypes = [i32, i32, i64, p, p, p, i64, i64, i64, p, p, i64, i64, p, p, p, p]
        lib.oracle_relative_top_records.restype = i64
        lib.oracle_dense_columns.argtypes = [i32, i32, i64, p, p, p, i64, p, i64, i64, p]
        lib.oracle_sort_rows.argtypes = [p, i64, i32, p]
        lib.oracle_apply_within_sorted.argtypes = [i32, i32, i64, p, p, p, i64, i64, p, p, i64, p, p, p]
        _lib = lib
    return _lib


def _c(a: np.ndarray, dtype) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _table(site, kind, coef):
    site = _c(site, np.int16).reshape(-1, 4)
    kind = _c(kind, np.uint8).reshape(-1, 4)
    coef = _c(coef, np.float64).reshape(-1, 2)
    return site, kind, coef


def _psi(psi) -> np.ndarray:
    flat = np.ascontiguousarray(np.asarray(psi, dtype=np.complex128).reshape(-1))
    return _c(flat.view(np.float64).reshape(-1, 2), np.float64)


def apply_term(site_row, kind_row, config, particle_cut: int = 1):
    """Apply one term to one row; returns (success, parity, new_row)."""
    lib = _load()
    site_row = _c(site_row, np.int16)
    kind_row = _c(kind_row, np.uint8)
    cur = _c(config, np.uint8).copy()
    parity = ctypes.c_int(0)
    ok = lib.oracle_apply_term(cur.size, particle_cut, _ptr(site_row), _ptr(kind_row), _ptr(cur), ctypes.addressof(parity))
    return bool(ok), int(parity.value), cur


def apply_within(site, kind, coef, configs_i, psi_i, configs_j, particle_cut: int = 1) -> np.ndarray:
    lib = _load()
    site, kind, coef = _table(site, kind, coef)
    ci = _c(configs_i, np.uint8)
    cj = _c(configs_j, np.uint8)
    nq = ci.shape[1]
    pi = _psi(psi_i)
    out = np.zeros((cj.shape[0], 2), dtype=np.float64)
    lib.oracle_apply_within(nq, particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), ci.shape[0], _ptr(ci),
                            _ptr(pi), cj.shape[0], _ptr(cj), _ptr(out))
    return out.view(np.complex128).reshape(-1)


def sort_rows(rows) -> np.ndarray:
    """Stable lexicographic order of uint8 rows (int64 indices)."""
    r = _c(rows, np.uint8)
    idx = np.zeros(r.shape[0], dtype=np.int64)
    _load().oracle_sort_rows(_ptr(r), r.shape[0], r.shape[1], _ptr(idx))
    return idx


def apply_within_sorted(site, kind, coef, configs_i, psi_f64, configs_j, idx, acc, rows, particle_cut: int = 1) -> None:
    """apply_within's loop over source rows [begin, end) into acc (float64 [n_j, 2], by sorted position of configs_j).

    Inputs must already be contiguous in the oracle's dtypes (psi_f64 float64
    [n_i, 2]); nothing is copied, so timing loops measure the loop alone.
    """
    begin, end = rows
    _load().oracle_apply_within_sorted(configs_i.shape[1], particle_cut, site.shape[0], _ptr(site), _ptr(kind),
                                       _ptr(coef), begin, end, _ptr(configs_i), _ptr(psi_f64), configs_j.shape[0],
                                       _ptr(configs_j), _ptr(idx), _ptr(acc))


def apply_within_adjoint(site, kind, coef, configs_i, configs_j, g_j, particle_cut: int = 1, rows=None) -> np.ndarray:
    """out_i = H^dagger g_j restricted to configs_i (rows = (begin, end) computes only those rows of configs_i)."""
    lib = _load()
    site, kind, coef = _table(site, kind, coef)
    ci = _c(configs_i, np.uint8)
    cj = _c(configs_j, np.uint8)
    begin, end = (0, ci.shape[0]) if rows is None else rows
    g = _psi(g_j)
    out = np.zeros((max(end - begin, 0), 2), dtype=np.float64)
    lib.oracle_apply_within_adjoint(ci.shape[1], particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), begin,
                                    end, _ptr(ci), cj.shape[0], _ptr(cj), _ptr(g), _ptr(out))
    return out.view(np.complex128).reshape(-1)


def relative_top_records(site, kind, coef, configs_i, psi_i, top: int, configs_exclude=None, particle_cut: int = 1,
                         rows=None):
    """The `top` highest-ranked find_relative records of source rows [begin, end) (all rows when rows is None).

    Returns (weights, orders, rows): ranked order = weight descending, then
    visiting order (term * n_i + row) descending; orders are those of the
    whole configs_i, so results of separate row ranges merge exactly.
    """
    lib = _load()
    site, kind, coef = _table(site, kind, coef)
    ci = _c(configs_i, np.uint8)
    ex = ci if configs_exclude is None else _c(configs_exclude, np.uint8)
    nq = ci.shape[1]
    pi = _psi(psi_i)
    begin, end = (0, ci.shape[0]) if rows is None else rows
    cap = max(int(top), 1)
    w = np.zeros(cap, dtype=np.float64)
    o = np.zeros(cap, dtype=np.uint64)
    r = np.zeros((cap, nq), dtype=np.uint8)
    n = lib.oracle_relative_top_records(nq, particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), ci.shape[0],
                                        begin, end, _ptr(ci), _ptr(pi), int(top), ex.shape[0], _ptr(ex), _ptr(w),
                                        _ptr(o), _ptr(r))
    return w[:n].copy(), o[:n].copy(), r[:n].copy()


def dense_columns(site, kind, coef, configs, cols, particle_cut: int = 1) -> np.ndarray:
    """Columns [begin, end) of the dense matrix <j|H|i> over configs: complex128 [n, end - begin]."""
    lib = _load()
    site, kind, coef = _table(site, kind, coef)
    c = _c(configs, np.uint8)
    n = c.shape[0]
    begin, end = cols
    mat = np.zeros((n, max(end - begin, 0), 2), dtype=np.float64)
    lib.oracle_dense_columns(c.shape[1], particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), n, _ptr(c),
                             begin, end, _ptr(mat))
    return mat.view(np.complex128).reshape(n, max(end - begin, 0))


def diagonal_term(site, kind, coef, configs, particle_cut: int = 1) -> np.ndarray:
    lib = _load()
    site, kind, coef = _table(site, kind, coef)
    c = _c(configs, np.uint8)
    out = np.zeros((c.shape[0], 2), dtype=np.float64)
    lib.oracle_diagonal_term(c.shape[1], particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), c.shape[0],
                             _ptr(c), _ptr(out))
    return out.view(np.complex128).reshape(-1)


def find_relative(site, kind, coef, configs_i, psi_i, count_selected: int, configs_exclude=None, particle_cut: int = 1,
                  rule: str = "heap"):
    """rule='heap' restates the reference's heap; rule='ranked' is the CUDA path's total order.

    With rule='ranked' returns (rows, info) where info = (kth_weight, n_above, n_equal, n_records).
    """
    lib = _load()
    site, kind, coef = _table(site, kind, coef)
    ci = _c(configs_i, np.uint8)
    ex = ci if configs_exclude is None else _c(configs_exclude, np.uint8)
    nq = ci.shape[1]
    pi = _psi(psi_i)
    cap = max(int(count_selected), 1)
    out = np.zeros((cap, nq), dtype=np.uint8)
    if rule == "heap":
        n = lib.oracle_find_relative_heap(nq, particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), ci.shape[0],
                                          _ptr(ci), _ptr(pi), int(count_selected), ex.shape[0], _ptr(ex), _ptr(out))
        return out[:n].copy()
    info = np.zeros(4, dtype=np.float64)
    n = lib.oracle_find_relative_ranked(nq, particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), ci.shape[0],
                                        _ptr(ci), _ptr(pi), int(count_selected), ex.shape[0], _ptr(ex), _ptr(out),
                                        _ptr(info))
    return out[:n].copy(), (float(info[0]), int(info[1]), int(info[2]), int(info[3]))


def rows_with_weight(site, kind, coef, configs_i, psi_i, weight: float, configs_exclude=None, particle_cut: int = 1,
                     cap: int = 1 << 16) -> np.ndarray:
    lib = _load()
    site, kind, coef = _table(site, kind, coef)
    ci = _c(configs_i, np.uint8)
    ex = ci if configs_exclude is None else _c(configs_exclude, np.uint8)
    nq = ci.shape[1]
    pi = _psi(psi_i)
    out = np.zeros((cap, nq), dtype=np.uint8)
    n = lib.oracle_rows_with_weight(nq, particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), ci.shape[0],
                                    _ptr(ci), _ptr(pi), ex.shape[0], _ptr(ex), float(weight), cap, _ptr(out))
    return out[:min(n, cap)].copy()


def term_uniform(seed: int, term: int) -> float:
    return float(_load().oracle_term_uniform(seed & (2**64 - 1), term))


def single_relative(site, kind, coef, configs, seed: int, particle_cut: int = 1):
    """Returns (rows, keys, terms): the sampled neighbour, its key and the term index (-1: none)."""
    lib = _load()
    site, kind, coef = _table(site, kind, coef)
    c = _c(configs, np.uint8)
    out = np.zeros_like(c)
    keys = np.zeros(c.shape[0], dtype=np.float64)
    terms = np.zeros(c.shape[0], dtype=np.int64)
    lib.oracle_single_relative(c.shape[1], particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), c.shape[0],
                               _ptr(c), seed & (2**64 - 1), _ptr(out), _ptr(keys), _ptr(terms))
    return out, keys, terms


def dense_matrix(site, kind, coef, configs, particle_cut: int = 1) -> np.ndarray:
    lib = _load()
    site, kind, coef = _table(site, kind, coef)
    c = _c(configs, np.uint8)
    n = c.shape[0]
    mat = np.zeros((n, n, 2), dtype=np.float64)
    lib.oracle_dense_matrix(c.shape[1], particle_cut, site.shape[0], _ptr(site), _ptr(kind), _ptr(coef), n, _ptr(c),
                            _ptr(mat))
    return mat.view(np.complex128).reshape(n, n)
