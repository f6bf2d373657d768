"""CUDA path against the reference's golden outputs and the CPU oracle.

Tolerances: FP64 apply_within / diagonal_term agree to 1e-12 of the absolute
sum of the contributions to each amplitude (summation order differs from the
reference's); find_relative rows are compared byte for byte.  The main cases
run with each walk kernel (tiled, grouped, pivot) forced in turn, besides the
automatic choice.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from conftest import GOLDEN_CASES, golden
from qmb_gb300 import Hamiltonian, terms

pytestmark = pytest.mark.gpu

RTOL_F64 = 1e-12


def abs_scale(site, kind, coef, configs_i, psi_i, configs_j, pc):
    """Per-target sum of |coef*psi| over contributing pairs (particle_cut 2 drops the signs)."""
    mag = np.zeros_like(coef)
    mag[:, 0] = np.hypot(coef[:, 0], coef[:, 1])
    return np.abs(oracle.apply_within(site, kind, mag, configs_i, np.abs(psi_i).astype(np.complex128), configs_j, 2))


def ham_of(g):
    return Hamiltonian((torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"])),
                       kind="fermi" if int(g["particle_cut"]) == 1 else "bose2")


def dev(x, device):
    return torch.from_numpy(np.ascontiguousarray(x)).to(device)


WALKS = ["auto", "tiled", "grouped", "pivot"]


@pytest.fixture(params=WALKS)
def walk(request, monkeypatch):
    """Every walk kernel on every case: the automatic choice, or one forced through QMBX_WALK."""
    if request.param != "auto":
        monkeypatch.setenv("QMBX_WALK", request.param)
    return request.param


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_apply_within_matches_reference(case, walk, cuda_device):
    g = golden(case)
    ham = ham_of(g)
    got = ham.apply_within(dev(g["configs_i"], cuda_device), dev(g["psi_i"], cuda_device),
                           dev(g["configs_j"], cuda_device)).cpu().numpy()
    ref = g["psi_j"]
    if case == "edge_duplicates":
        want = oracle.apply_within(g["site"], g["kind"], g["coef"], g["configs_i"], g["psi_i"], g["configs_j"])
        scale = abs_scale(g["site"], g["kind"], g["coef"], g["configs_i"], g["psi_i"], g["configs_j"], 1)
        assert np.all(np.abs(got - want) <= RTOL_F64 * scale + 1e-300)
        return
    scale = abs_scale(g["site"], g["kind"], g["coef"], g["configs_i"], g["psi_i"], g["configs_j"],
                      int(g["particle_cut"]))
    assert np.all(np.abs(got - ref) <= RTOL_F64 * scale + 1e-300)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_diagonal_term_matches_reference(case, walk, cuda_device):
    g = golden(case)
    got = ham_of(g).diagonal_term(dev(g["diag_configs"], cuda_device)).cpu().numpy()
    np.testing.assert_allclose(got, g["diag"], rtol=0, atol=RTOL_F64 * np.abs(g["coef"]).sum())


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_find_relative_matches_reference(case, walk, cuda_device):
    g = golden(case)
    ham = ham_of(g)
    pc = int(g["particle_cut"])
    ex = g.get("configs_exclude")
    for k in g["counts"]:
        got = ham.find_relative(dev(g["configs_i"], cuda_device), dev(g["psi_i"], cuda_device), int(k),
                                None if ex is None else dev(ex, cuda_device)).cpu().numpy()
        ranked, (wk, _, _, _) = oracle.find_relative(g["site"], g["kind"], g["coef"], g["configs_i"], g["psi_i"], int(k),
                                                     ex, pc, rule="ranked")
        assert np.array_equal(got, ranked), (case, k)  # bit-exact with the oracle's total order
        ref = g[f"relative_{k}"]
        if not np.array_equal(got, ref):
            # only rows whose records all tie at the k-th weight may differ from the reference heap
            tied = {bytes(r) for r in oracle.rows_with_weight(g["site"], g["kind"], g["coef"], g["configs_i"], g["psi_i"],
                                                              wk, ex, pc)}
            assert ({bytes(r) for r in got} ^ {bytes(r) for r in ref}) <= tied, (case, k)


@pytest.mark.parametrize("case", ["ab_initio_10_complex", "random_terms_fermi", "random_terms_bose2", "ising_4x4"])
def test_adjoint_is_the_conjugate_transpose(case, cuda_device):
    g = golden(case)
    ham = ham_of(g)
    ci, cj = dev(g["configs_i"], cuda_device), dev(g["configs_j"], cuda_device)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(ci.shape[0]) + 1j * rng.standard_normal(ci.shape[0])
    y = rng.standard_normal(cj.shape[0]) + 1j * rng.standard_normal(cj.shape[0])
    ax = ham.apply_within(ci, dev(x, cuda_device), cj).cpu().numpy()
    ahy = ham.apply_within_adjoint(ci, dev(y, cuda_device), cj).cpu().numpy()
    lhs = np.vdot(y, ax)
    rhs = np.vdot(ahy, x)
    assert abs(lhs - rhs) <= 1e-11 * (np.abs(y) @ np.abs(ax) + 1)
    # and against the oracle applied entry by entry
    want = oracle.apply_within(g["site"], g["kind"], g["coef"], g["configs_i"], x, g["configs_j"], int(g["particle_cut"]))
    assert np.allclose(ax, want, rtol=0, atol=1e-11 * (1 + np.abs(want).max()))


def test_adjoint_against_dense_matrix(cuda_device):
    g = golden("ab_initio_10_complex")
    rows = terms.unique_rows(np.concatenate([g["configs_i"], g["configs_j"]]))
    h = oracle.dense_matrix(g["site"], g["kind"], g["coef"], rows)
    ham = ham_of(g)
    c = dev(rows, cuda_device)
    rng = np.random.default_rng(9)
    y = rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])
    got = ham.apply_within_adjoint(c, dev(y, cuda_device), c).cpu().numpy()
    want = h.conj().T @ y
    assert np.allclose(got, want, rtol=0, atol=1e-11 * np.abs(want).max())


@pytest.mark.parametrize("case", ["ab_initio_6", "ab_initio_10_complex", "random_terms_fermi", "ising_4x4"])
def test_compensated_fp32_tracks_fp64(case, walk, cuda_device):
    g = golden(case)
    ham = ham_of(g)
    ci, cj = dev(g["configs_i"], cuda_device), dev(g["configs_j"], cuda_device)
    psi32 = g["psi_i"].astype(np.complex64)
    exact = ham.apply_within(ci, dev(psi32.astype(np.complex128), cuda_device), cj).cpu().numpy()
    comp = ham.apply_within_compensated(ci, dev(psi32, cuda_device), cj).cpu().numpy()
    scale = abs_scale(g["site"], g["kind"], g["coef"], g["configs_i"], psi32, g["configs_j"], int(g["particle_cut"]))
    # compensated FP32: error of order 2^-46 of the absolute sum (coefficients split hi + lo)
    assert np.all(np.abs(comp - exact) <= 1e-12 * scale + 1e-30)
    plain = ham.apply_within(ci, dev(psi32, cuda_device), cj).cpu().numpy()
    assert plain.dtype == np.complex64
    assert np.all(np.abs(plain - exact) <= 2e-7 * (scale + np.abs(exact)))


def test_single_relative_matches_oracle(walk, cuda_device):
    for case in ("ab_initio_10_complex", "random_terms_fermi", "random_terms_bose2", "ising_4x4"):
        g = golden(case)
        ham = ham_of(g)
        rows = g["configs_j"]
        for seed in (1, 12345, 2**63 + 11):
            got = ham.single_relative_seeded(dev(rows, cuda_device), seed).cpu().numpy()
            want, keys, term = oracle.single_relative(g["site"], g["kind"], g["coef"], rows, seed, int(g["particle_cut"]))
            same = np.all(got == want, axis=1)
            if not np.all(same):
                # only near-ties of the log-domain key (last-ulp differences of log) may differ
                bad = np.nonzero(~same)[0]
                assert len(bad) <= max(1, len(rows) // 1000), (case, seed, bad[:5])


def test_single_relative_draws_connected_rows_outside_the_set(cuda_device):
    g = golden("ab_initio_6")
    ham = ham_of(g)
    rows = g["configs_i"][::5]
    out = ham.single_relative(dev(rows, cuda_device)).cpu().numpy()
    inset = {bytes(r) for r in rows}
    for r, o in zip(rows, out):
        if not o.any():
            continue
        assert bytes(o) not in inset
        conn = oracle.apply_within(g["site"], g["kind"], np.abs(g["coef"]) + 1.0, r[None], np.ones(1, np.complex128), o[None])
        assert conn[0] != 0


def test_empty_inputs(cuda_device):
    g = golden("ab_initio_6")
    ham = ham_of(g)
    nq = g["configs_i"].shape[1]
    empty = torch.zeros((0, nq), dtype=torch.uint8, device=cuda_device)
    some = dev(g["configs_i"][:10], cuda_device)
    psi = dev(g["psi_i"][:10], cuda_device)
    assert ham.apply_within(empty, torch.zeros(0, dtype=torch.complex128, device=cuda_device), some).abs().max() == 0
    assert ham.apply_within(some, psi, empty).shape == (0,)
    assert ham.diagonal_term(empty).shape == (0,)
    assert ham.find_relative(some, psi, 0).shape == (0, nq)
    assert ham.find_relative(empty, torch.zeros(0, dtype=torch.complex128, device=cuda_device), 10).shape == (0, nq)
    assert ham.single_relative(empty).shape == (0, nq)


def test_errors_are_raised_not_trapped(cuda_device):
    g = golden("ab_initio_6")
    ham = ham_of(g)
    c = dev(g["configs_i"][:10], cuda_device)
    with pytest.raises(RuntimeError):
        ham.apply_within(c, dev(g["psi_i"][:9], cuda_device), c)
    with pytest.raises(RuntimeError):
        ham.apply_within(c.float(), dev(g["psi_i"][:10], cuda_device), c)
    with pytest.raises(RuntimeError):
        ham.find_relative(c, dev(g["psi_i"][:10], cuda_device), -1)
    with pytest.raises(RuntimeError):
        ham.apply_within(c.cpu(), torch.from_numpy(g["psi_i"][:10]), c.cpu())
    # the context is still usable
    assert ham.diagonal_term(c).shape == (10,)


@pytest.mark.parametrize("case", ["hubbard_3x2", "ab_initio_6"])
def test_single_relative_frequencies_follow_coefficients(case, cuda_device):
    """The reference's sampling law (qmb/_hamiltonian_cuda.cu:854-866): a neighbour is drawn with
    probability sum |c_t| over the terms that lead to it, over sum |c_t| of all candidates; a
    chi-squared test over 4,000 seeds for one row."""
    scipy_stats = pytest.importorskip("scipy.stats")
    g = golden(case)
    ham = ham_of(g)
    pc = int(g["particle_cut"])
    row = g["configs_i"][:1]
    weight = {}
    for t in range(g["site"].shape[0]):
        ok, _, out = oracle.apply_term(g["site"][t], g["kind"][t], row[0], pc)
        if ok and not np.array_equal(out, row[0]):
            key = bytes(out)
            weight[key] = weight.get(key, 0.0) + float(np.hypot(*g["coef"][t]))
    weight = {k: w for k, w in weight.items() if w > 0}
    assert len(weight) >= 4
    keys = sorted(weight)
    total = sum(weight.values())
    counts = dict.fromkeys(keys, 0)
    c = dev(row, cuda_device)
    n = 4000
    for seed in range(n):
        got = bytes(ham.single_relative_seeded(c, 7919 * seed + 1).cpu().numpy()[0])
        counts[got] += 1
    observed = np.array([counts[k] for k in keys], dtype=np.float64)
    expected = np.array([n * weight[k] / total for k in keys])
    stat = float(((observed - expected) ** 2 / expected).sum())
    assert scipy_stats.chi2.sf(stat, len(keys) - 1) > 1e-4, (stat, len(keys))
