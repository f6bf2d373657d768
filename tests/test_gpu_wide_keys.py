"""Configurations of three and four key words (n_qubytes 17 to 32) against the oracle.

The golden cases and the benchmark shapes use one or two key words; these
cases cover the three- and four-word instantiations of every kernel: a
Fermi-Hubbard lattice of 160 and 256 spin orbitals (n_qubytes 20 and 32) and
random operator strings over 256 sites with fermions and hard-core bosons.
Targets include the sources' neighbours, so that lookups hit.  Every walk
kernel is forced in turn.  Tolerances as in the golden parity tests: FP64 and
compensated FP32 (same FP32 amplitudes) to 1e-12 of the per-amplitude
absolute sum, the adjoint through <g, H psi> = <H^dagger g, psi>,
find_relative byte for byte.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from qmb_gb300 import Hamiltonian, terms

pytestmark = pytest.mark.gpu


def _random_rows(rng, n_rows, nq, density):
    bits = (rng.random((n_rows, 8 * nq)) < density).astype(np.uint8)
    return terms.unique_rows(np.packbits(bits, axis=1, bitorder="little"))


def _random_terms(rng, n_terms, n_sites):
    site = np.zeros((n_terms, 4), dtype=np.int16)
    kind = np.full((n_terms, 4), 2, dtype=np.uint8)
    for t in range(n_terms):
        k = rng.integers(1, 5)
        site[t, :k] = rng.integers(0, n_sites, size=k)
        kind[t, :k] = rng.integers(0, 2, size=k)
    coef = rng.standard_normal((n_terms, 2))
    return site, kind, coef


def _cases():
    rng = np.random.default_rng(17)
    out = []
    for m, n in ((10, 8), (16, 8)):
        site, kind, coef = (x.numpy() for x in terms.sort_terms(*terms.prepare(terms.hubbard_dict(m, n, 1.0, 4.0))))
        nq = 2 * m * n // 8
        out.append((f"hubbard_{m}x{n}", site, kind, coef, 1, _random_rows(rng, 300, nq, 0.5)))
    for pc in (1, 2):
        site, kind, coef = _random_terms(rng, 3000, 256)
        out.append((f"random_terms_256_pc{pc}", site, kind, coef, pc, _random_rows(rng, 300, 32, 0.3)))
    return out


CASES = _cases()


@pytest.fixture(params=["auto", "tiled", "grouped", "pivot"])
def walk(request, monkeypatch):
    if request.param != "auto":
        monkeypatch.setenv("QMBX_WALK", request.param)
    return request.param


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_wide_keys_against_oracle(case, walk, cuda_device):
    name, site, kind, coef, pc, rows = case
    ham = Hamiltonian((torch.from_numpy(site), torch.from_numpy(kind), torch.from_numpy(coef)),
                      kind="fermi" if pc == 1 else "bose2")
    rng = np.random.default_rng(5)
    psi = rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])
    near = oracle.find_relative(site, kind, coef, rows, psi, 1 << 16, rows, pc)
    targets = np.concatenate([rows, near[:3000]])
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(cuda_device)  # noqa: E731

    want = oracle.apply_within(site, kind, coef, rows, psi, targets, pc)
    mag = np.zeros_like(coef)
    mag[:, 0] = np.hypot(coef[:, 0], coef[:, 1])
    scale = np.abs(oracle.apply_within(site, kind, mag, rows, np.abs(psi).astype(np.complex128), targets, 2))
    got = ham.apply_within(dev(rows), dev(psi), dev(targets)).cpu().numpy()
    assert np.count_nonzero(want) > 50, name
    assert np.all(np.abs(got - want) <= 1e-12 * scale + 1e-30), name

    # compensated FP32 on the same FP32 amplitudes, and the adjoint against the forward map
    psi32 = psi.astype(np.complex64)
    want32 = oracle.apply_within(site, kind, coef, rows, psi32.astype(np.complex128), targets, pc)
    got32 = ham.apply_within_compensated(dev(rows), dev(psi32), dev(targets)).cpu().numpy()
    assert np.all(np.abs(got32 - want32) <= 1e-12 * scale + 1e-30), name
    g = rng.standard_normal(targets.shape[0]) + 1j * rng.standard_normal(targets.shape[0])
    adj = ham.apply_within_adjoint(dev(rows), dev(g), dev(targets)).cpu().numpy()
    assert abs(np.vdot(g, got) - np.vdot(adj, psi)) <= 1e-11 * (np.abs(g) @ scale + 1), name

    diag = ham.diagonal_term(dev(targets[:200])).cpu().numpy()
    want_diag = oracle.diagonal_term(site, kind, coef, targets[:200], pc)
    assert np.allclose(diag, want_diag, rtol=0, atol=1e-12 * np.abs(coef).sum()), name

    for k in (50, 2000):
        got_rel = ham.find_relative(dev(rows), dev(psi), k).cpu().numpy()
        ranked, _ = oracle.find_relative(site, kind, coef, rows, psi, k, rows, pc, rule="ranked")
        assert np.array_equal(got_rel, ranked), (name, k)

    got_one = ham.single_relative_seeded(dev(rows), 99).cpu().numpy()
    want_one, _, _ = oracle.single_relative(site, kind, coef, rows, 99, pc)
    same = np.all(got_one == want_one, axis=1)
    assert np.count_nonzero(~same) <= 1, name  # last-ulp differences of log may flip a near tie
