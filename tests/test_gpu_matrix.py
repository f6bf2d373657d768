"""H materialised on a fixed basis (Hamiltonian.matrix, qmbx_matrix_*).

The sparse matrix of H restricted to a set of distinct rows is compared with
the oracle's dense matrix on the golden cases (1e-12 of the largest
coefficient sum), its product with a vector with apply_within on the same
rows (1e-12 of the per-amplitude absolute sum), repeated products bit for
bit, and the Lanczos energy computed through it with the one computed
through apply_within.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import bench
import oracle
from conftest import GOLDEN_CASES, golden
from qmb_gb300 import Hamiltonian, lanczos_energy

pytestmark = pytest.mark.gpu


def _ham(g):
    return Hamiltonian((torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"])),
                       kind="fermi" if int(g["particle_cut"]) == 1 else "bose2")


@pytest.mark.parametrize("walk", ["auto", "grouped", "tiled", "pivot"])
@pytest.mark.parametrize("case", [c for c in GOLDEN_CASES if not c.endswith("_relative")])
def test_matrix_equals_dense_oracle(case, walk, cuda_device, monkeypatch):
    if walk != "auto":
        monkeypatch.setenv("QMBX_WALK", walk)
    g = golden(case)
    rows = np.unique(np.concatenate([g["configs_i"], g["configs_j"]]), axis=0)
    pc = int(g["particle_cut"])
    want = oracle.dense_matrix(g["site"], g["kind"], g["coef"], rows, pc)
    mat = _ham(g).matrix(torch.from_numpy(rows).to(cuda_device))
    got = mat.to_dense().cpu().numpy()
    scale = np.abs(g["coef"]).sum()
    assert np.abs(got - want).max() <= 1e-12 * scale
    # the diagonal entry leads every row
    first = mat.col[mat.row_ptr[:-1]].cpu().numpy()
    assert np.array_equal(first, np.arange(rows.shape[0]))


def test_matrix_apply_matches_apply_within_on_c1(cuda_device):
    wl = bench.make_workload("c1")
    ham = Hamiltonian((torch.from_numpy(wl["site"]), torch.from_numpy(wl["kind"]), torch.from_numpy(wl["coef"])),
                      kind="fermi")
    rows = torch.from_numpy(wl["configs_i"]).to(cuda_device)
    psi = torch.from_numpy(wl["psi"]).to(cuda_device)
    mat = ham.matrix(rows)
    y = mat.apply(psi)
    ref = ham.apply_within(rows, psi, rows)
    mag = np.zeros_like(wl["coef"])
    mag[:, 0] = np.hypot(wl["coef"][:, 0], wl["coef"][:, 1])
    scale = np.abs(oracle.apply_within(wl["site"], wl["kind"], mag, wl["configs_i"],
                                       np.abs(wl["psi"]).astype(np.complex128), wl["configs_i"], 2))
    assert np.all(np.abs((y - ref).cpu().numpy()) <= 1e-12 * scale + 1e-300)
    y2 = mat.apply(psi)
    assert torch.equal(torch.view_as_real(y), torch.view_as_real(y2))


def test_lanczos_through_the_matrix_matches_the_walks(cuda_device):
    g = golden("ab_initio_10_complex")
    rows = torch.from_numpy(np.unique(np.concatenate([g["configs_i"], g["configs_j"]]), axis=0)).to(cuda_device)
    ham = _ham(g)
    gen = torch.Generator(device=cuda_device).manual_seed(3)
    start = torch.randn(rows.shape[0], dtype=torch.complex128, device=cuda_device, generator=gen)
    e_mat, v_mat = lanczos_energy(ham, rows, 60, start=start)
    e_walk, v_walk = lanczos_energy(ham, rows, 60, start=start, materialize=False)
    assert abs(e_mat - e_walk) <= 1e-10 * (1 + abs(e_walk))


def test_matrix_rejects_repeated_rows(cuda_device):
    g = golden("ab_initio_6")
    rows = torch.from_numpy(np.concatenate([g["configs_i"], g["configs_i"][:3]])).to(cuda_device)
    with pytest.raises(RuntimeError, match="distinct"):
        _ham(g).matrix(rows)


@pytest.mark.parametrize("n_rows", [300, 6000])
def test_matrix_products_one_and_many_vectors(n_rows, cuda_device):
    # a sparse basis (random determinants, a few entries per row: a thread per row) and a denser one
    # (a warp per row); m vectors in one pass equal m single products, to 1e-12 of the absolute sums
    qmb = __import__("qmb_gb300")
    site, kind, coef = (x.numpy() for x in qmb.terms.integral_hamiltonian_tables(12, seed=5))
    rows = qmb.terms.random_determinants(12, 4, 4, n_rows, seed=6)
    ham = Hamiltonian((torch.from_numpy(site), torch.from_numpy(kind), torch.from_numpy(coef)), kind="fermi")
    drows = torch.from_numpy(rows).to(cuda_device)
    mat = ham.matrix(drows)
    assert (mat.nnz < 4 * rows.shape[0]) == (n_rows == 300)  # which product kernel runs
    gen = torch.Generator(device=cuda_device).manual_seed(7)
    x = torch.randn((rows.shape[0], 3), dtype=torch.complex128, device=cuda_device, generator=gen)
    mag = np.zeros_like(coef)
    mag[:, 0] = np.hypot(coef[:, 0], coef[:, 1])
    many = mat.apply(x)
    assert torch.equal(torch.view_as_real(many), torch.view_as_real(mat.apply(x)))
    for c in range(3):
        col = x[:, c].contiguous()
        one = mat.apply(col)
        assert torch.equal(torch.view_as_real(one), torch.view_as_real(mat.apply(col)))
        ref = ham.apply_within(drows, col, drows)
        scale = np.abs(oracle.apply_within(site, kind, mag, rows, np.abs(col.cpu().numpy()).astype(np.complex128),
                                           rows, 2))
        assert np.all(np.abs((one - ref).cpu().numpy()) <= 1e-12 * scale + 1e-300)
        assert np.all(np.abs((many[:, c] - ref).cpu().numpy()) <= 1e-12 * scale + 1e-300)
