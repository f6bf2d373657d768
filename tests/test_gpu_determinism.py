"""Run twice, compare bytes.

The gather walks (the grouped, tiled and row-serial walks of the side whose
rows receive the sums) add each row's contributions in a fixed order, so
their results repeat bit for bit; so do diagonal_term, find_relative (a total
order decides every selection) and single_relative for a given seed.  The
scatter walk and the pivot-major walk add into their outputs with FP64
atomics, whose order varies: with QMBX_DETERMINISTIC=1 apply_within and its
adjoint avoid both, and the results repeat bit for bit on every workload.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import bench
from conftest import GOLDEN_CASES, golden
from qmb_gb300 import Hamiltonian

pytestmark = pytest.mark.gpu


def _ham(g):
    return Hamiltonian((torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"])),
                       kind="fermi" if int(g["particle_cut"]) == 1 else "bose2")


def _same_bits(a: torch.Tensor, b: torch.Tensor) -> bool:
    return a.dtype == b.dtype and a.shape == b.shape and bool(torch.equal(a.view(torch.uint8), b.view(torch.uint8)))


def _twice(fn):
    a = fn()
    b = fn()
    torch.cuda.synchronize()
    return a, b


@pytest.mark.parametrize("walk", ["auto", "grouped", "tiled"])
@pytest.mark.parametrize("case", [c for c in GOLDEN_CASES if not c.endswith("_relative")])
def test_gather_paths_repeat_bit_for_bit(case, walk, cuda_device, monkeypatch):
    if walk != "auto":
        monkeypatch.setenv("QMBX_WALK", walk)
    g = golden(case)
    ham = _ham(g)
    # distinct rows: repeated source rows are summed with atomics before the walk
    rows = torch.from_numpy(np.unique(np.concatenate([g["configs_i"], g["configs_j"]]), axis=0)).to(cuda_device)
    rng = np.random.default_rng(3)
    psi = torch.from_numpy(rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])).to(cuda_device)
    # configs_i is configs_j: the gather walk over the distinct rows
    for fn in (lambda: ham.apply_within(rows, psi, rows),
               lambda: ham.apply_within(rows, psi.to(torch.complex64), rows),
               lambda: ham.apply_within_adjoint(rows, psi, rows),
               lambda: ham.diagonal_term(rows),
               lambda: ham.find_relative(rows, psi, 17),
               lambda: ham.single_relative_seeded(rows, 99)):
        a, b = _twice(fn)
        assert _same_bits(a, b)


@pytest.mark.parametrize("walk", ["auto", "pivot"])
def test_deterministic_mode_repeats_bit_for_bit(walk, cuda_device, monkeypatch):
    # C2: the forward map would scatter from the 20,000 sources into the 200,000 targets
    monkeypatch.setenv("QMBX_DETERMINISTIC", "1")
    if walk != "auto":
        monkeypatch.setenv("QMBX_WALK", walk)
    wl = bench.make_workload("c2")
    ham = Hamiltonian((torch.from_numpy(wl["site"]), torch.from_numpy(wl["kind"]), torch.from_numpy(wl["coef"])),
                      kind="fermi")
    ci = torch.from_numpy(wl["configs_i"]).to(cuda_device)
    cj = torch.from_numpy(wl["configs_j"]).to(cuda_device)
    psi = torch.from_numpy(wl["psi"]).to(cuda_device)
    gen = torch.Generator(device=cuda_device).manual_seed(4)
    g = torch.randn(cj.shape[0], dtype=torch.complex128, device=cuda_device, generator=gen)
    outs = {}
    for name, fn in (("fwd64", lambda: ham.apply_within(ci, psi, cj)),
                     ("fwd32", lambda: ham.apply_within(ci, psi.to(torch.complex64), cj)),
                     ("adj64", lambda: ham.apply_within_adjoint(ci, g, cj)),
                     ("adj32", lambda: ham.apply_within_adjoint(ci, g.to(torch.complex64), cj))):
        a, b = _twice(fn)
        assert _same_bits(a, b), name
        outs[name] = a
    # the deterministic walks compute the same map as the default ones
    monkeypatch.delenv("QMBX_DETERMINISTIC")
    ref = ham.apply_within(ci, psi, cj)
    scale = ref.abs().max().item()
    assert (outs["fwd64"] - ref).abs().max().item() <= 1e-12 * scale
