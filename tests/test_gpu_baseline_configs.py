"""Parity on the benchmark's own workloads at their full sizes.

The headline workload C2 (28 spin orbitals, 55,371 terms; configs_i 20,000
and configs_j 200,000 random determinants; find_relative top 50,000 outside
configs_i) is compared in full with the oracle, split across host processes
(oracle/pool.py):

* find_relative: byte-exact against the oracle's ranked rule, and against
  the reference's own heap rule except rows whose records all tie exactly at
  the K-th weight (the reference keeps an arbitrary subset of those);
* apply_within and its adjoint in FP64 on every source and target row:
  |delta| <= 1e-12 of the per-amplitude absolute sum sum_t,i |c_t psi_i|;
* the compensated FP32 forward and adjoint on the same FP32 inputs, results
  read as complex128: the same 1e-12 bound.

C3 (52 spin orbitals, 669,579 terms) is checked on a connected subset of
2,048 rows: the energy gradient of an MLP wave function of the benchmark's
shape (4 hidden layers of 512) is sent through the adjoint kernel and
compared with the same network evaluated against a dense FP64 H built by the
oracle, and with central finite differences.
"""

from __future__ import annotations

import copy
import importlib

import numpy as np
import pytest
import torch

import bench
import oracle
from oracle import pool
from qmb_gb300 import Hamiltonian, variational_energy

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2():
    wl = bench.make_workload("c2")
    wl["ham"] = Hamiltonian((torch.from_numpy(wl["site"]), torch.from_numpy(wl["kind"]),
                             torch.from_numpy(wl["coef"])), kind="fermi")
    return wl


def _magnitudes(coef: np.ndarray) -> np.ndarray:
    mag = np.zeros_like(coef)
    mag[:, 0] = np.hypot(coef[:, 0], coef[:, 1])
    return mag


def test_c2_find_relative_exact_at_full_size(c2, cuda_device):
    K = c2["spec"]["count_selected"]
    ci, psi = c2["configs_i"], c2["psi"]
    got = c2["ham"].find_relative(torch.from_numpy(ci).to(cuda_device), torch.from_numpy(psi).to(cuda_device),
                                  K).cpu().numpy()
    want, kth = pool.find_relative_ranked_par(c2["site"], c2["kind"], c2["coef"], ci, psi, K, ci)
    assert want.shape[0] > 0.9 * K
    assert np.array_equal(got, want)
    # the reference's heap: identical except rows that only tie at the K-th weight
    heap = oracle.find_relative(c2["site"], c2["kind"], c2["coef"], ci, psi, K, ci, rule="heap")
    ties = {bytes(r) for r in pool.tie_rows_par(c2["site"], c2["kind"], c2["coef"], ci, psi, kth, ci)}
    a, b = {bytes(r) for r in got}, {bytes(r) for r in heap}
    assert (a ^ b) <= ties


def test_c2_apply_within_fp64_every_row(c2, cuda_device):
    s, k, c = c2["site"], c2["kind"], c2["coef"]
    ci, cj, psi = c2["configs_i"], c2["configs_j"], c2["psi"]
    want = pool.apply_within_par(s, k, c, ci, psi, cj)
    scale = np.abs(pool.apply_within_par(s, k, _magnitudes(c), ci, np.abs(psi).astype(np.complex128), cj, 2))
    assert np.count_nonzero(want) > 0.5 * cj.shape[0]
    dci, dcj = torch.from_numpy(ci).to(cuda_device), torch.from_numpy(cj).to(cuda_device)
    got = c2["ham"].apply_within(dci, torch.from_numpy(psi).to(cuda_device), dcj).cpu().numpy()
    assert np.all(np.abs(got - want) <= 1e-12 * scale + 1e-300)


def test_c2_adjoint_fp64_every_row(c2, cuda_device):
    s, k, c = c2["site"], c2["kind"], c2["coef"]
    ci, cj = c2["configs_i"], c2["configs_j"]
    rng = np.random.default_rng(21)
    g = rng.standard_normal(cj.shape[0]) + 1j * rng.standard_normal(cj.shape[0])
    want = pool.apply_within_adjoint_par(s, k, c, ci, cj, g)
    scale = np.abs(pool.apply_within_adjoint_par(s, k, _magnitudes(c), ci, cj, np.abs(g).astype(np.complex128), 2))
    assert np.count_nonzero(want) > 0.9 * ci.shape[0]
    dci, dcj = torch.from_numpy(ci).to(cuda_device), torch.from_numpy(cj).to(cuda_device)
    got = c2["ham"].apply_within_adjoint(dci, torch.from_numpy(g).to(cuda_device), dcj).cpu().numpy()
    assert np.all(np.abs(got - want) <= 1e-12 * scale + 1e-300)


def test_c2_compensated_fp32_every_row(c2, cuda_device):
    s, k, c = c2["site"], c2["kind"], c2["coef"]
    ci, cj = c2["configs_i"], c2["configs_j"]
    psi32 = c2["psi"].astype(np.complex64)
    rng = np.random.default_rng(22)
    g32 = (rng.standard_normal(cj.shape[0]) + 1j * rng.standard_normal(cj.shape[0])).astype(np.complex64)
    ham = c2["ham"]
    dci, dcj = torch.from_numpy(ci).to(cuda_device), torch.from_numpy(cj).to(cuda_device)
    # forward on the same FP32 inputs, compensated result read as complex128
    want = pool.apply_within_par(s, k, c, ci, psi32.astype(np.complex128), cj)
    scale = np.abs(pool.apply_within_par(s, k, _magnitudes(c), ci, np.abs(psi32).astype(np.complex128), cj, 2))
    got = ham.apply_within_compensated(dci, torch.from_numpy(psi32).to(cuda_device), dcj).cpu().numpy()
    assert np.all(np.abs(got - want) <= 1e-12 * scale + 1e-300)
    # adjoint, compensated, complex128 out
    want = pool.apply_within_adjoint_par(s, k, c, ci, cj, g32.astype(np.complex128))
    scale = np.abs(pool.apply_within_adjoint_par(s, k, _magnitudes(c), ci, cj, np.abs(g32).astype(np.complex128), 2))
    got = ham._apply(dci, torch.from_numpy(g32).to(cuda_device), dcj, adjoint=True,
                     out_dtype=torch.complex128).cpu().numpy()
    assert np.all(np.abs(got - want) <= 1e-12 * scale + 1e-300)


# ---------------------------------------------------------------------------
# C3: the energy gradient through the adjoint kernel on a 2,048-row subset
# ---------------------------------------------------------------------------


@pytest.fixture(scope="module")
def c3_subset():
    """2,048 rows of the C3 system that are connected to each other, its dense H and an MLP of the benchmark's shape.

    Random determinants of 52 spin orbitals are almost never connected (a
    row reaches ~6e4 of the 4e11 possible rows), so a subset of the random
    rows would give a nearly diagonal H.  The subset is 32 benchmark rows
    and the 2,016 rows the oracle's find_relative ranks highest from them.
    """
    wl = bench.make_workload("c3")
    s, k, c = wl["site"], wl["kind"], wl["coef"]
    seeds, psi = wl["configs_i"][:32], wl["psi"][:32]
    near, _ = pool.find_relative_ranked_par(s, k, c, seeds, psi, 2016, seeds)
    rows = np.unique(np.concatenate([seeds, near]), axis=0)
    extra = wl["configs_i"][32:]
    have = {bytes(r) for r in rows}
    fill = [r for r in extra if bytes(r) not in have][: 2048 - rows.shape[0]]
    if fill:
        rows = np.unique(np.concatenate([rows, np.stack(fill)]), axis=0)
    assert rows.shape[0] == 2048
    h = pool.dense_matrix_par(s, k, c, rows)
    ham = Hamiltonian((torch.from_numpy(s), torch.from_numpy(k), torch.from_numpy(c)), kind="fermi")
    return dict(rows=rows, h=h, ham=ham, nq=wl["nq"], seed=wl["spec"]["seed"])


def _mlp(c3, device):
    return bench._Mlp(8 * c3["nq"], device, seed=c3["seed"])


def _engine_walks(fn, replays: bool = False):
    """Term-walk launches made by fn (the forward walk plus, when taken, the adjoint walk); with
    ``replays`` also the launches that replay a hit log or apply a stored matrix."""
    native = importlib.import_module("qmb-public_gb300._native")
    native.profile_enable(True)
    fn()
    torch.cuda.synchronize()
    prof = native.profile_read()
    native.profile_enable(False)
    walks = prof["groups"]["enumerate"][0]
    return (walks, prof["groups"]["spmv"][0]) if replays else walks


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_c3_gradient_through_adjoint_matches_dense(c3_subset, dtype, cuda_device):
    c3 = c3_subset
    assert np.count_nonzero(c3["h"]) > 20 * c3["rows"].shape[0]  # far from diagonal
    mlp = _mlp(c3, cuda_device)
    rows = torch.from_numpy(c3["rows"]).to(cuda_device)
    hd = torch.from_numpy(c3["h"]).to(cuda_device)
    ham = c3["ham"]
    assert ham._table(cuda_device, c3["nq"]).hermitian

    def grads(kind):
        for p in mlp.net.parameters():
            p.grad = None
        psi = mlp(rows)
        if kind == "dense":
            p64 = psi.to(torch.complex128)
            e = (p64.conj() @ (hd @ p64)).real / (p64.conj() @ p64).real
        else:
            e = variational_energy(ham, rows, psi.to(dtype), hermitian_shortcut=(kind == "shortcut"))
        e.backward()
        return e.item(), [p.grad.detach().clone() for p in mlp.net.parameters()]

    e_dense, g_dense = grads("dense")
    holder = {}
    # the backward through the adjoint kernel: the forward walk and the adjoint walk both run
    ham.hit_log = False
    try:
        walks = _engine_walks(lambda: holder.setdefault("adj", grads("adjoint")))
    finally:
        ham.hit_log = True
    e_adj, g_adj = holder["adj"]
    assert walks == 2
    # the backward from the forward walk's hit log: one walk, then the replay (a first call on
    # rows of this shape may find the log too small and walk; the second one fits)
    grads("adjoint")
    walks, replays = _engine_walks(lambda: holder.setdefault("log", grads("adjoint")), replays=True)
    assert walks == 1 and replays >= 1
    e_log, g_log = holder["log"]
    # the Hermitian shortcut: the forward walk only
    assert _engine_walks(lambda: holder.setdefault("cut", grads("shortcut"))) == 1
    e_cut, g_cut = holder["cut"]
    if dtype == torch.complex128:
        e_tol, rtol = 1e-12 * (1 + abs(e_dense)), 1e-5
    else:
        # compensated FP32 products and sums, complex64 gradient: energy within
        # 1e-7 Ha of FP64 (the path's stated bound), gradients to FP32 rounding
        e_tol, rtol = 1e-7, 1e-4
    assert abs(e_adj - e_dense) <= e_tol
    assert abs(e_log - e_dense) <= e_tol
    assert abs(e_cut - e_dense) <= e_tol
    # elementwise to rtol, with an absolute floor of rtol times the largest
    # gradient entry: some entries vanish exactly in FP64 (the log-amplitude
    # bias: E does not change when psi is scaled) and carry FP32 rounding here
    atol = rtol * max(b.abs().max().item() for b in g_dense)
    for a, b, lg, cut in zip(g_adj, g_dense, g_log, g_cut):
        assert torch.allclose(a, b, rtol=rtol, atol=atol)
        assert torch.allclose(lg, b, rtol=rtol, atol=atol)
        assert torch.allclose(cut, b, rtol=rtol, atol=atol)


def test_c3_gradient_through_adjoint_matches_finite_differences(c3_subset, cuda_device):
    c3 = c3_subset
    mlp = _mlp(c3, cuda_device)
    net = copy.deepcopy(mlp.net).double()
    rows = torch.from_numpy(c3["rows"]).to(cuda_device)
    bitspack = importlib.import_module("qmb-public_gb300.bitspack")
    bits = bitspack.unpack_int(rows, 1, 8 * c3["nq"]).to(torch.float64)
    ham = c3["ham"]

    def energy():
        out = net(bits)
        psi = torch.polar(torch.exp(out[:, 0]), out[:, 1])
        return variational_energy(ham, rows, psi, hermitian_shortcut=False)

    for p in net.parameters():
        p.grad = None
    energy().backward()
    params = list(net.parameters())
    grad = [p.grad.detach().clone() for p in params]
    gen = torch.Generator(device=cuda_device).manual_seed(7)
    h = 1e-4
    for _ in range(2):
        d = [torch.randn(p.shape, dtype=p.dtype, device=cuda_device, generator=gen) for p in params]
        norm = torch.sqrt(sum((x * x).sum() for x in d))
        d = [x / norm for x in d]
        analytic = sum((g * x).sum() for g, x in zip(grad, d)).item()
        with torch.no_grad():
            for p, x in zip(params, d):
                p.add_(h * x)
            plus = energy().item()
            for p, x in zip(params, d):
                p.sub_(2 * h * x)
            minus = energy().item()
            for p, x in zip(params, d):
                p.add_(h * x)
        fd = (plus - minus) / (2 * h)
        assert abs(fd - analytic) <= 1e-6 * max(1.0, abs(analytic))
