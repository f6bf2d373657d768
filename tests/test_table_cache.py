"""The on-disk cache of compiled term tables (hamiltonian.compile_table).

A compiled table written under its checksum is read back byte for byte by
the next compile of the same terms; other terms, row widths or particle
kinds get other files; a damaged or truncated file is rejected by
qmbx_table_check and rebuilt.  Host only: no GPU needed.
"""

from __future__ import annotations

import importlib
import os

import numpy as np
import torch

from conftest import golden

ham_mod = importlib.import_module("qmb-public_gb300.hamiltonian")


def _terms(case="ab_initio_6"):
    g = golden(case)
    return torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"])


def test_cache_round_trip(tmp_path):
    site, kind, coef = _terms()
    fresh = ham_mod.compile_table(site, kind, coef, 2, 1)
    first = ham_mod.compile_table(site, kind, coef, 2, 1, tmp_path)
    files = os.listdir(tmp_path)
    assert len(files) == 1 and files[0].endswith(".qmbx")
    assert torch.equal(first, fresh)
    # the second compile reads the file: make that visible by stamping its mtime
    path = tmp_path / files[0]
    os.utime(path, (1, 1))
    again = ham_mod.compile_table(site, kind, coef, 2, 1, tmp_path)
    assert torch.equal(again, fresh)
    assert os.stat(path).st_mtime == 1


def test_cache_keys_differ_by_terms_width_and_kind(tmp_path):
    site, kind, coef = _terms()
    ham_mod.compile_table(site, kind, coef, 2, 1, tmp_path)
    ham_mod.compile_table(site, kind, coef, 3, 1, tmp_path)
    ham_mod.compile_table(site, kind, coef, 2, 2, tmp_path)
    ham_mod.compile_table(site, kind, coef * 2, 2, 1, tmp_path)
    assert len(os.listdir(tmp_path)) == 4


def test_damaged_cache_file_is_rebuilt(tmp_path):
    site, kind, coef = _terms("random_terms_fermi")
    fresh = ham_mod.compile_table(site, kind, coef, 3, 1, tmp_path)
    path = tmp_path / os.listdir(tmp_path)[0]
    data = np.fromfile(path, dtype=np.uint8)
    data[:data.size // 2].tofile(path)  # truncated
    assert torch.equal(ham_mod.compile_table(site, kind, coef, 3, 1, tmp_path), fresh)
    bad = fresh.numpy().copy()
    bad[:4] = 0  # no magic
    bad.tofile(path)
    assert torch.equal(ham_mod.compile_table(site, kind, coef, 3, 1, tmp_path), fresh)
    # and the rebuilt blob was written back whole
    assert np.array_equal(np.fromfile(path, dtype=np.uint8), fresh.numpy())
