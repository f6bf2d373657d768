"""Host logic of the Lanczos and PT2 callers, on the CPU.

The solvers only call the Hamiltonian's four operators, so a stand-in that
applies a dense FP64 matrix (built by the oracle over a basis closed under H)
exercises their recurrences and sums without a GPU; the GPU tests run the same
solvers on the CUDA engine.
"""

from __future__ import annotations

import numpy as np
import torch

import oracle
from qmb_gb300 import lanczos_energy, pt2_energy, terms


class DenseHam:
    """apply_within / find_relative / diagonal_term over rows of a dense matrix."""

    def __init__(self, rows: np.ndarray, h: np.ndarray):
        self.rows = rows
        self.h = torch.from_numpy(h)
        self.index = {r.tobytes(): k for k, r in enumerate(rows)}

    def _idx(self, configs: torch.Tensor) -> torch.Tensor:
        return torch.tensor([self.index[r.tobytes()] for r in configs.numpy()], dtype=torch.int64)

    def apply_within(self, configs_i, psi_i, configs_j):
        i, j = self._idx(configs_i), self._idx(configs_j)
        return self.h[j][:, i] @ psi_i.to(torch.complex128)

    def diagonal_term(self, configs):
        k = self._idx(configs)
        return self.h[k, k]

    def find_relative(self, configs_i, psi_i, count_selected, configs_exclude):
        # every row connected to configs_i outside configs_exclude (count_selected is large in these tests)
        i = self._idx(configs_i)
        excluded = set(self._idx(configs_exclude).tolist())
        reach = (self.h[:, i].abs() > 0).any(dim=1).nonzero().flatten().tolist()
        keep = sorted(k for k in reach if k not in excluded)
        return torch.from_numpy(self.rows[keep])


def _system(complex_valued: bool):
    site, kind, coef = terms.integral_hamiltonian_tables(5, seed=13, complex_valued=complex_valued)
    rows = terms.all_determinants(5, 2, 2)
    h = oracle.dense_matrix(site.numpy(), kind.numpy(), coef.numpy(), rows, 1)
    return rows, h


def test_lanczos_recurrence_finds_the_lowest_eigenvalue():
    for complex_valued in (False, True):
        rows, h = _system(complex_valued)
        ham = DenseHam(rows, h)
        gen = torch.Generator().manual_seed(3)
        energy, vector = lanczos_energy(ham, torch.from_numpy(rows), step=60, generator=gen)
        exact = np.linalg.eigvalsh(h)[0]
        assert abs(energy - exact) <= 1e-9 * abs(exact)
        v = vector.numpy()
        assert abs(np.vdot(v, h @ v).real / np.vdot(v, v).real - exact) <= 1e-8 * abs(exact)


def test_pt2_sum_matches_the_dense_formula():
    rows, h = _system(True)
    ham = DenseHam(rows, h)
    rng = np.random.default_rng(6)
    chosen = np.sort(rng.choice(rows.shape[0], size=20, replace=False))
    psi = rng.standard_normal(20) + 1j * rng.standard_normal(20)
    e0, e2 = pt2_energy(ham, torch.from_numpy(rows[chosen]), torch.from_numpy(psi), 10**6)
    full = np.zeros(rows.shape[0], dtype=np.complex128)
    full[chosen] = psi
    norm = np.vdot(psi, psi).real
    want0 = np.vdot(full, h @ full).real / norm
    hpsi = h @ full
    outside = np.setdiff1d(np.nonzero(np.abs(h[:, chosen]).sum(axis=1) > 0)[0], chosen)
    want2 = np.sum(np.abs(hpsi[outside]) ** 2 / norm / (want0 - np.diag(h).real[outside]))
    assert abs(e0 - want0) <= 1e-12 * abs(want0)
    assert abs(e2 - want2) <= 1e-10 * abs(want2)
