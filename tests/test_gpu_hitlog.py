"""Adjoint products replayed from a forward walk's hit log (qmbx_*_logged; the autograd backward).

The backward of apply_within needs exactly the (term, row) pairs the forward
walk found.  A logged forward records them; the adjoint replayed from the
record must equal the adjoint walk (qmbx_apply_within_adjoint) -- FP64 and
compensated FP32, both walk directions (scatter: the output side larger;
gather: the same rows), every walk kernel, repeated rows -- to 1e-12 of the
per-amplitude absolute sum.  A record too small for the forward's hits is
detected, the backward falls back to the walk, and the next call on rows of
the same shape records them all.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import bench
import oracle
from conftest import golden
from qmb_gb300 import Hamiltonian

pytestmark = pytest.mark.gpu


def _ham(g):
    return Hamiltonian((torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"])),
                       kind="fermi" if int(g["particle_cut"]) == 1 else "bose2")


def _adjoint_scale(site, kind, coef, pc, ci, cj, g):
    """Per-row sum of |coef * g| over the contributing pairs (particle_cut 2: the same pairs, no
    fermionic sign, so nothing cancels)."""
    mag = np.zeros_like(coef)
    mag[:, 0] = np.hypot(coef[:, 0], coef[:, 1])
    return np.abs(oracle.apply_within_adjoint(site, kind, mag, ci, cj, np.abs(g).astype(np.complex128), 2))


@pytest.mark.parametrize("walk", ["auto", "grouped", "tiled", "pivot"])
@pytest.mark.parametrize("swap", [False, True])
@pytest.mark.parametrize("case", ["ab_initio_6", "ab_initio_10_complex", "random_terms_fermi", "random_terms_bose2",
                                  "edge_duplicates"])
def test_adjoint_from_log_equals_adjoint_walk(case, swap, walk, cuda_device, monkeypatch):
    if walk != "auto":
        monkeypatch.setenv("QMBX_WALK", walk)
    g = golden(case)
    ci, cj = (g["configs_j"], g["configs_i"]) if swap else (g["configs_i"], g["configs_j"])
    pc = int(g["particle_cut"])
    ham = _ham(g)
    rng = np.random.default_rng(9)
    psi = rng.standard_normal(ci.shape[0]) + 1j * rng.standard_normal(ci.shape[0])
    gj = rng.standard_normal(cj.shape[0]) + 1j * rng.standard_normal(cj.shape[0])
    dci, dcj = torch.from_numpy(ci).to(cuda_device), torch.from_numpy(cj).to(cuda_device)
    scale = _adjoint_scale(g["site"], g["kind"], g["coef"], pc, ci, cj, gj)
    want = oracle.apply_within_adjoint(g["site"], g["kind"], g["coef"], ci, cj, gj, pc)
    for dtype in (torch.complex128, torch.complex64):
        p = torch.from_numpy(psi).to(cuda_device).to(dtype)
        y, record = ham._apply(dci, p, dcj, adjoint=False, log=True)
        got = ham._adjoint_from_log(record, torch.from_numpy(gj).to(cuda_device).to(dtype), torch.complex128)
        assert got is not None
        # the FP32 path replays on FP32 inputs: compare with the oracle on the same rounded g
        ref = want if dtype == torch.complex128 else oracle.apply_within_adjoint(
            g["site"], g["kind"], g["coef"], ci, cj, gj.astype(np.complex64).astype(np.complex128), pc)
        assert np.all(np.abs(got.cpu().numpy() - ref) <= 1e-12 * scale + 1e-300)


def test_autograd_backward_replays_the_log_at_c2(cuda_device):
    wl = bench.make_workload("c2")
    ham = Hamiltonian((torch.from_numpy(wl["site"]), torch.from_numpy(wl["kind"]), torch.from_numpy(wl["coef"])),
                      kind="fermi")
    ci = torch.from_numpy(wl["configs_i"]).to(cuda_device)
    cj = torch.from_numpy(wl["configs_j"]).to(cuda_device)
    gen = torch.Generator(device=cuda_device).manual_seed(3)
    g = torch.randn(cj.shape[0], dtype=torch.complex128, device=cuda_device, generator=gen)
    native = __import__("importlib").import_module("qmb-public_gb300._native")
    for dtype in (torch.complex128, torch.complex64):
        p = torch.from_numpy(wl["psi"]).to(cuda_device).to(dtype).requires_grad_(True)
        native.profile_enable(True)
        y = ham.apply_within(ci, p, cj)
        (gi,) = torch.autograd.grad(y, p, grad_outputs=g.to(dtype))
        torch.cuda.synchronize()
        prof = native.profile_read()
        native.profile_enable(False)
        # one term walk (the forward); the adjoint came from the record
        assert prof["groups"]["enumerate"][0] == 1 and prof["groups"]["spmv"][0] >= 1
        walk = ham.apply_within_adjoint(ci, g.to(dtype), cj)
        scale = walk.abs().max().item()
        tol = 1e-12 if dtype == torch.complex128 else 1e-6
        assert (gi - walk).abs().max().item() <= tol * scale


@pytest.mark.parametrize("walk", ["auto", "tiled", "pivot"])
@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
@pytest.mark.parametrize("case", ["ab_initio_6", "ab_initio_10_complex", "edge_duplicates"])
def test_small_record_falls_back_then_grows(case, dtype, walk, cuda_device, monkeypatch):
    # a record far too small for the forward's hits: the adjoint is walked instead (decided on the
    # device, over the row sets the forward left in the log), the result is the same, and the next
    # call of this shape records every hit
    if walk != "auto":
        monkeypatch.setenv("QMBX_WALK", walk)
    g = golden(case)
    ham = _ham(g)
    ham._LOG_FIRST_GUESS = 4
    ci = torch.from_numpy(g["configs_i"]).to(cuda_device)
    cj = torch.from_numpy(g["configs_j"]).to(cuda_device)
    psi = torch.from_numpy(g["psi_i"]).to(cuda_device).to(dtype)
    gj = torch.randn(cj.shape[0], dtype=torch.complex128, device=cuda_device).to(dtype)
    walk = ham.apply_within_adjoint(ci, gj, cj)
    key = (cuda_device.index if cuda_device.index is not None else 0, ci.shape[0], cj.shape[0])
    tol = 1e-12 if dtype == torch.complex128 else 1e-6
    for attempt in range(3):
        p = psi.clone().requires_grad_(True)
        (gi,) = torch.autograd.grad(ham.apply_within(ci, p, cj), p, grad_outputs=gj)
        assert (gi - walk).abs().max().item() <= tol * walk.abs().max().item()
    assert ham._log_caps[key]["cap"] > 4


def test_adjoint_of_a_buffer_without_a_log_is_nan(cuda_device):
    # the device checks the log's header: arguments that do not match it give NaN, not garbage
    g = golden("ab_initio_6")
    ham = _ham(g)
    ci = torch.from_numpy(g["configs_i"]).to(cuda_device)
    cj = torch.from_numpy(g["configs_j"]).to(cuda_device)
    psi = torch.from_numpy(g["psi_i"]).to(cuda_device)
    y, record = ham._apply(ci, psi, cj, adjoint=False, log=True)
    record.buf.zero_()
    got = ham._adjoint_from_log(record, y.new_ones(cj.shape[0]), torch.complex128)
    assert torch.isnan(got.real).all()


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_backward_on_the_same_rows(dtype, cuda_device):
    # configs_i and configs_j the same tensor (one row set; the forward gathers): the backward
    # through the log equals the oracle's adjoint
    g = golden("ab_initio_10_complex")
    rows = np.unique(np.concatenate([g["configs_i"], g["configs_j"]]), axis=0)
    ham = _ham(g)
    rng = np.random.default_rng(5)
    psi = rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])
    gj = rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])
    c = torch.from_numpy(rows).to(cuda_device)
    p = torch.from_numpy(psi).to(cuda_device).to(dtype).requires_grad_(True)
    gt = torch.from_numpy(gj).to(cuda_device).to(dtype)
    (gi,) = torch.autograd.grad(ham.apply_within(c, p, c), p, grad_outputs=gt)
    g_used = gj if dtype == torch.complex128 else gj.astype(np.complex64).astype(np.complex128)
    want = oracle.apply_within_adjoint(g["site"], g["kind"], g["coef"], rows, rows, g_used, 1)
    scale = _adjoint_scale(g["site"], g["kind"], g["coef"], 1, rows, rows, g_used)
    tol = 1e-12 if dtype == torch.complex128 else 1e-6
    assert np.all(np.abs(gi.to(torch.complex128).cpu().numpy() - want) <= tol * scale + 1e-300)


@pytest.mark.parametrize("swap", [False, True])
def test_replay_keeps_subnormal_sums(swap, cuda_device):
    # The compensated FP32 replay widens its float run sums to FP64 with integer bit operations.
    # A gradient scaled by 2^-140 makes every product and run sum an FP32 subnormal: they must
    # reach the FP64 output, not be flushed or mis-scaled.  Each product of a subnormal keeps the
    # subnormal grid (2^-149), so a row may differ from the FP64 oracle by its pair count times
    # a few grid steps.
    g = golden("ab_initio_6")
    ci, cj = (g["configs_j"], g["configs_i"]) if swap else (g["configs_i"], g["configs_j"])
    ham = _ham(g)
    rng = np.random.default_rng(11)
    psi = rng.standard_normal(ci.shape[0]) + 1j * rng.standard_normal(ci.shape[0])
    gj = ((rng.standard_normal(cj.shape[0]) + 1j * rng.standard_normal(cj.shape[0])) * 2.0 ** -140).astype(np.complex64)
    assert np.all(np.abs(gj.real) < 2.0 ** -126) and np.count_nonzero(gj.real) > cj.shape[0] // 2
    dci, dcj = torch.from_numpy(ci).to(cuda_device), torch.from_numpy(cj).to(cuda_device)
    p = torch.from_numpy(psi).to(cuda_device).to(torch.complex64)
    _, record = ham._apply(dci, p, dcj, adjoint=False, log=True)
    got = ham._adjoint_from_log(record, torch.from_numpy(gj).to(cuda_device), torch.complex128)
    assert got is not None
    got = got.cpu().numpy()
    want = oracle.apply_within_adjoint(g["site"], g["kind"], g["coef"], ci, cj, gj.astype(np.complex128),
                                       int(g["particle_cut"]))
    ones = np.zeros_like(g["coef"])
    ones[:, 0] = 1.0
    pairs = np.abs(oracle.apply_within_adjoint(g["site"], g["kind"], ones, ci, cj, np.ones(cj.shape[0], np.complex128), 2))
    assert np.all(np.abs(got - want) <= (pairs + 1.0) * 8 * 2.0 ** -149)
    # nothing flushed to zero or scaled: the rows sum to the oracle's total magnitude
    assert np.median(np.abs(want)) > 1e3 * 2.0 ** -149
    assert np.sum(np.abs(got)) == pytest.approx(np.sum(np.abs(want)), rel=0.02)
