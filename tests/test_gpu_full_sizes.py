"""The CUDA path at the benchmark workloads' full sizes.

The oracle cannot walk a whole benchmark workload in test time, so the full
sizes are checked through properties that need only a small oracle run:

* linearity: amplitudes supported on a few hundred source rows, with every
  other structure at full size (all targets, all terms); the oracle walks only
  those sources (for C4, whose random rows are not connected to each other,
  the targets also hold the sources' neighbours).  FP64 agrees to 1e-12 of
  the per-target absolute sum, the compensated FP32 path to 1e-12 of it too
  (same FP32 inputs);
* the adjoint identity <g, H psi> = <H^dagger g, psi> on random full vectors;
* find_relative at C5 size: output sorted, unique, outside the excluded set,
  each row connected to the seeds; and bit-exact against the oracle's ranked
  rule on a subset of seeds (full 3.1M-term table, pivot and grouped walks).

Workloads: C2 (28 spin orbitals, 55,371 terms, 20,000 x 200,000 rows), C4
(Hubbard 8x8, 1,000,000 rows), C5 (76 spin orbitals, 3,076,435 terms, 8,192
seeds), generated with the benchmark's own seeded generators.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import bench
import oracle
from qmb_gb300 import Hamiltonian

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workloads():
    cache = {}

    def get(name):
        if name not in cache:
            wl = bench.make_workload(name)
            wl["ham"] = Hamiltonian((torch.from_numpy(wl["site"]), torch.from_numpy(wl["kind"]),
                                     torch.from_numpy(wl["coef"])), kind="fermi")
            cache[name] = wl
        return cache[name]

    return get


def _abs_scale(wl, rows, psi, targets):
    mag = np.zeros_like(wl["coef"])
    mag[:, 0] = np.hypot(wl["coef"][:, 0], wl["coef"][:, 1])
    return np.abs(oracle.apply_within(wl["site"], wl["kind"], mag, rows, np.abs(psi).astype(np.complex128), targets, 2))


@pytest.mark.parametrize("name,n_src", [("c2", 256), ("c4", 64)])
def test_sparse_sources_against_oracle(workloads, name, n_src, cuda_device):
    wl = workloads(name)
    ci, cj = wl["configs_i"], wl["configs_j"]
    rng = np.random.default_rng(11)
    pick = np.sort(rng.choice(ci.shape[0], size=n_src, replace=False))
    psi = np.zeros(ci.shape[0], dtype=np.complex64)
    psi[pick] = (rng.standard_normal(n_src) + 1j * rng.standard_normal(n_src)).astype(np.complex64)
    if name == "c4":
        # random half-filled Hubbard rows are never connected to each other:
        # append the picked sources' neighbours (outside configs_j) to the targets
        near = oracle.find_relative(wl["site"], wl["kind"], wl["coef"], ci[pick], psi[pick].astype(np.complex128),
                                    1 << 20, cj)
        cj = np.concatenate([cj, near])
    want = oracle.apply_within(wl["site"], wl["kind"], wl["coef"], ci[pick], psi[pick].astype(np.complex128), cj)
    scale = _abs_scale(wl, ci[pick], psi[pick], cj)
    assert np.count_nonzero(want) > 100
    dci, dcj = torch.from_numpy(ci).to(cuda_device), torch.from_numpy(cj).to(cuda_device)
    ham = wl["ham"]
    got64 = ham.apply_within(dci, torch.from_numpy(psi.astype(np.complex128)).to(cuda_device), dcj).cpu().numpy()
    assert np.all(np.abs(got64 - want) <= 1e-12 * scale + 1e-30)
    got32 = ham.apply_within_compensated(dci, torch.from_numpy(psi).to(cuda_device), dcj).cpu().numpy()
    assert np.all(np.abs(got32 - want) <= 1e-12 * scale + 1e-30)


@pytest.mark.parametrize("name", ["c2", "c4"])
def test_adjoint_identity_at_full_size(workloads, name, cuda_device):
    wl = workloads(name)
    ham = wl["ham"]
    dci = torch.from_numpy(wl["configs_i"]).to(cuda_device)
    dcj = torch.from_numpy(wl["configs_j"]).to(cuda_device)
    gen = torch.Generator(device=cuda_device).manual_seed(5)
    x = torch.randn(dci.shape[0], dtype=torch.complex128, device=cuda_device, generator=gen)
    y = torch.randn(dcj.shape[0], dtype=torch.complex128, device=cuda_device, generator=gen)
    ax = ham.apply_within(dci, x, dcj)
    ahy = ham.apply_within_adjoint(dci, y, dcj)
    lhs = torch.vdot(y, ax).item()
    rhs = torch.vdot(ahy, x).item()
    assert abs(lhs - rhs) <= 1e-11 * (torch.abs(y) @ torch.abs(ax)).item()


def _lex_sorted_unique(rows: np.ndarray) -> bool:
    if rows.shape[0] < 2:
        return True
    a, b = rows[:-1], rows[1:]
    diff = a != b
    first = np.argmax(diff, axis=1)
    any_diff = diff.any(axis=1)
    idx = np.arange(a.shape[0])
    return bool(np.all(any_diff) and np.all(a[idx, first] < b[idx, first]))


def test_find_relative_invariants_at_c5_size(workloads, cuda_device):
    wl = workloads("c5")
    ham = wl["ham"]
    ci = torch.from_numpy(wl["configs_i"]).to(cuda_device)
    psi = torch.from_numpy(wl["psi"]).to(cuda_device)
    K = wl["spec"]["count_selected"]
    out = ham.find_relative(ci, psi, K).cpu().numpy()
    assert 0 < out.shape[0] <= K
    assert _lex_sorted_unique(out)
    seeds = {bytes(r) for r in wl["configs_i"]}
    assert not any(bytes(r) in seeds for r in out)
    # every returned row receives amplitude from the seeds
    rng = np.random.default_rng(2)
    sample = out[np.sort(rng.choice(out.shape[0], size=min(2000, out.shape[0]), replace=False))]
    hpsi = ham.apply_within(ci, psi, torch.from_numpy(sample).to(cuda_device)).cpu().numpy()
    assert np.all(np.abs(hpsi) > 0)


@pytest.mark.parametrize("walk", ["auto", "grouped"])
def test_find_relative_exact_on_seed_subset_of_c5(workloads, walk, cuda_device, monkeypatch):
    # the automatic choice takes the pivot walk here; "grouped" forces the
    # warp-per-row walk over two key words
    if walk != "auto":
        monkeypatch.setenv("QMBX_WALK", walk)
    wl = workloads("c5")
    ham = wl["ham"]
    rng = np.random.default_rng(4)
    pick = np.sort(rng.choice(wl["configs_i"].shape[0], size=12, replace=False))
    seeds = wl["configs_i"][pick]
    psi = wl["psi"][pick]
    K = 5000
    want, _ = oracle.find_relative(wl["site"], wl["kind"], wl["coef"], seeds, psi, K, wl["configs_i"], 1, rule="ranked")
    got = ham.find_relative(torch.from_numpy(seeds).to(cuda_device), torch.from_numpy(psi).to(cuda_device), K,
                            torch.from_numpy(wl["configs_i"]).to(cuda_device)).cpu().numpy()
    assert want.shape[0] > 1000
    assert np.array_equal(got, want)


@pytest.mark.parametrize("k", [7, 300, 20000, 1 << 22])
def test_find_relative_with_sampled_threshold(k, cuda_device):
    # 6,000 source rows: pass 1 counts every 16th row and pass 2 confirms
    site, kind, coef = (x.numpy() for x in __import__("qmb_gb300").terms.integral_hamiltonian_tables(9, seed=3))
    rows = __import__("qmb_gb300").terms.random_determinants(9, 4, 4, 6000, seed=8)
    rng = np.random.default_rng(k)
    psi = rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])
    ham = Hamiltonian((torch.from_numpy(site), torch.from_numpy(kind), torch.from_numpy(coef)), kind="fermi")
    want, _ = oracle.find_relative(site, kind, coef, rows, psi, k, rows, 1, rule="ranked")
    got = ham.find_relative(torch.from_numpy(rows).to(cuda_device), torch.from_numpy(psi).to(cuda_device), k).cpu().numpy()
    assert np.array_equal(got, want)


def test_find_relative_when_the_sample_misleads(cuda_device):
    # pass 1 counts every 16th source row; give exactly those rows large amplitudes, so the
    # sample predicts 16 times the records above any weight and puts the threshold too high:
    # the emission pass then keeps fewer than k records, and an unsampled histogram pass and a
    # second emission pass take over (four walks in all)
    qmb = __import__("qmb_gb300")
    native = __import__("importlib").import_module("qmb-public_gb300._native")
    site, kind, coef = (x.numpy() for x in qmb.terms.integral_hamiltonian_tables(9, seed=3))
    rows = qmb.terms.random_determinants(9, 4, 4, 6000, seed=8)
    rng = np.random.default_rng(11)
    psi = (rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])) * 1e-3
    psi[::16] *= 1e6
    ham = Hamiltonian((torch.from_numpy(site), torch.from_numpy(kind), torch.from_numpy(coef)), kind="fermi")
    k = 100000
    want, _ = oracle.find_relative(site, kind, coef, rows, psi, k, rows, 1, rule="ranked")
    got = ham.find_relative(torch.from_numpy(rows).to(cuda_device), torch.from_numpy(psi).to(cuda_device), k).cpu().numpy()
    assert native.find_relative_stats()["walks"] == 4
    assert np.array_equal(got, want)
