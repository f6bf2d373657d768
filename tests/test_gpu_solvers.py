"""The device-side callers of the engine: Lanczos and the PT2 step.

Both run on a 6-orbital synthetic ab-initio Hamiltonian whose full
3-alpha/3-beta determinant space (400 rows) is closed under H, so a dense
FP64 matrix from the CPU oracle gives the exact answers: the Lanczos energy
must match the lowest eigenvalue to 1e-9 (relative), and the PT2 energy must
match the dense Epstein-Nesbet sum over the rows outside the variational set
to 1e-10 (relative).  Both run through the engine's own shortcuts (the
materialised matrix for Lanczos, the fused PT2 call) and through the plain
operator compositions of the reference; on the C5 system the fused PT2 call
is checked against the composition.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from qmb_gb300 import Hamiltonian, lanczos_energy, pt2_energy, terms

pytestmark = pytest.mark.gpu


def _system(complex_valued: bool):
    site, kind, coef = terms.integral_hamiltonian_tables(6, seed=21, complex_valued=complex_valued)
    rows = terms.all_determinants(6, 3, 3)
    h = oracle.dense_matrix(site.numpy(), kind.numpy(), coef.numpy(), rows, 1)
    return Hamiltonian((site, kind, coef), kind="fermi"), rows, h


@pytest.mark.parametrize("materialize", [True, False])
@pytest.mark.parametrize("complex_valued", [False, True])
def test_lanczos_matches_lowest_eigenvalue(complex_valued, materialize, cuda_device):
    ham, rows, h = _system(complex_valued)
    exact = np.linalg.eigvalsh(h)[0]
    gen = torch.Generator(device=cuda_device).manual_seed(5)
    energy, vector = lanczos_energy(ham, torch.from_numpy(rows).to(cuda_device), step=120, generator=gen,
                                    materialize=materialize)
    assert abs(energy - exact) <= 1e-9 * abs(exact)
    v = vector.cpu().numpy()
    rayleigh = np.vdot(v, h @ v).real / np.vdot(v, v).real
    assert abs(rayleigh - exact) <= 1e-8 * abs(exact)


def test_lanczos_stops_on_an_invariant_subspace(cuda_device):
    ham, rows, h = _system(False)
    # a start vector that is an eigenvector: the first residual vanishes
    w, u = np.linalg.eigh(h)
    start = torch.from_numpy(u[:, 0].astype(np.complex128)).to(cuda_device)
    energy, vector = lanczos_energy(ham, torch.from_numpy(rows).to(cuda_device), step=10, threshold=1e-8, start=start)
    assert abs(energy - w[0]) <= 1e-10 * abs(w[0])
    assert vector.shape == (rows.shape[0],)


@pytest.mark.parametrize("fused", [True, False])
@pytest.mark.parametrize("complex_valued", [False, True])
def test_pt2_matches_dense_epstein_nesbet(complex_valued, fused, cuda_device):
    ham, rows, h = _system(complex_valued)
    rng = np.random.default_rng(8)
    chosen = np.sort(rng.choice(rows.shape[0], size=60, replace=False))
    psi0 = rng.standard_normal(60) + 1j * rng.standard_normal(60)
    full = np.zeros(rows.shape[0], dtype=np.complex128)
    full[chosen] = psi0
    norm = np.vdot(psi0, psi0).real
    e0 = np.vdot(full, h @ full).real / norm
    hpsi = h @ full
    outside = np.setdiff1d(np.arange(rows.shape[0]), chosen)
    e2 = np.sum(np.abs(hpsi[outside]) ** 2 / norm / (e0 - np.diag(h).real[outside]))

    c = torch.from_numpy(rows[chosen]).to(cuda_device)
    psi = torch.from_numpy(psi0).to(cuda_device)
    # count_selected caps connection records (one per term and source row), not rows: take them all
    got0, got2 = pt2_energy(ham, c, psi, count_selected=100000, fused=fused)
    assert abs(got0 - e0) <= 1e-12 * abs(e0)
    assert abs(got2 - e2) <= 1e-10 * abs(e2)


@pytest.mark.parametrize("fused", [True, False])
def test_pt2_with_a_capped_selection(fused, cuda_device):
    ham, rows, h = _system(True)
    rng = np.random.default_rng(9)
    chosen = np.sort(rng.choice(rows.shape[0], size=60, replace=False))
    psi0 = rng.standard_normal(60) + 1j * rng.standard_normal(60)
    c = torch.from_numpy(rows[chosen]).to(cuda_device)
    psi = torch.from_numpy(psi0).to(cuda_device)
    other = ham.find_relative(c, psi, 500, c).cpu().numpy()
    assert 0 < other.shape[0] < rows.shape[0] - 60
    index = {r.tobytes(): k for k, r in enumerate(rows)}
    pick = np.array([index[r.tobytes()] for r in other])
    full = np.zeros(rows.shape[0], dtype=np.complex128)
    full[chosen] = psi0
    norm = np.vdot(psi0, psi0).real
    e0 = np.vdot(full, h @ full).real / norm
    hpsi = h @ full
    e2 = np.sum(np.abs(hpsi[pick]) ** 2 / norm / (e0 - np.diag(h).real[pick]))
    got0, got2 = pt2_energy(ham, c, psi, count_selected=500, fused=fused)
    assert abs(got0 - e0) <= 1e-12 * abs(e0)
    assert abs(got2 - e2) <= 1e-10 * abs(e2)


@pytest.mark.parametrize("walk", ["auto", "grouped"])
def test_fused_pt2_matches_composition_on_c5_seeds(walk, cuda_device, monkeypatch):
    # 76 spin orbitals, 3.1M terms (the pivot walk is chosen automatically),
    # 512 of the C5 seed rows, 20,000 selected records
    import bench

    if walk != "auto":
        monkeypatch.setenv("QMBX_WALK", walk)
    wl = bench.make_workload("c5")
    ham = Hamiltonian((torch.from_numpy(wl["site"]), torch.from_numpy(wl["kind"]), torch.from_numpy(wl["coef"])),
                      kind="fermi")
    c = torch.from_numpy(wl["configs_i"][:512]).to(cuda_device)
    psi = torch.from_numpy(wl["psi"][:512]).to(cuda_device)
    f0, f2 = pt2_energy(ham, c, psi, 20000)
    c0, c2 = pt2_energy(ham, c, psi, 20000, fused=False)
    assert abs(f0 - c0) <= 1e-12 * (1 + abs(c0))
    assert abs(f2 - c2) <= 1e-10 * abs(c2)
