"""The reference's own CUDA apply_within, run from its cubin, against the oracle.

bench.py times the reference's CUDA kernel (compiled from its sources into
oracle/_ref/ref_cuda_4_1.cubin by oracle/ref_build.py) as the FP64 GPU path
to beat; this checks that the harness that loads and launches it
(oracle/ref_cuda.py) computes apply_within: on a slice of the C2 workload
against the oracle (1e-12 of the per-amplitude absolute sum; the kernel adds
with FP64 atomics in no fixed order), and on the full C2 forward and its
adjoint (the same kernel on the daggered table) against this engine.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import bench
import oracle
from oracle import ref_cuda

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cuda.available(4, 1), reason="reference cubin absent (oracle/ref_build.py)")]


@pytest.fixture(scope="module")
def c2():
    return bench.make_workload("c2")


def test_reference_kernel_matches_oracle_on_a_slice(c2, cuda_device):
    ref = ref_cuda.ReferenceCuda(4, 1, cuda_device)
    table = ref.table(c2["site"], c2["kind"], c2["coef"])
    ci, psi, cj = c2["configs_i"][:500], c2["psi"][:500], c2["configs_j"][:50000]
    got = ref.apply_within(table, torch.from_numpy(ci).to(cuda_device), torch.from_numpy(psi).to(cuda_device),
                           torch.from_numpy(cj).to(cuda_device)).cpu().numpy()
    want = oracle.apply_within(c2["site"], c2["kind"], c2["coef"], ci, psi, cj)
    mag = np.zeros_like(c2["coef"])
    mag[:, 0] = np.hypot(c2["coef"][:, 0], c2["coef"][:, 1])
    scale = np.abs(oracle.apply_within(c2["site"], c2["kind"], mag, ci, np.abs(psi).astype(np.complex128), cj, 2))
    assert np.count_nonzero(want) > 1000
    assert np.all(np.abs(got - want) <= 1e-12 * scale + 1e-300)


def test_reference_kernel_matches_engine_at_full_size(c2, cuda_device):
    from qmb_gb300 import Hamiltonian

    ref = ref_cuda.ReferenceCuda(4, 1, cuda_device)
    fwd = ref.table(c2["site"], c2["kind"], c2["coef"])
    adj = ref.table(*ref_cuda.daggered(c2["site"], c2["kind"], c2["coef"]))
    ham = Hamiltonian((torch.from_numpy(c2["site"]), torch.from_numpy(c2["kind"]), torch.from_numpy(c2["coef"])),
                      kind="fermi")
    ci = torch.from_numpy(c2["configs_i"]).to(cuda_device)
    cj = torch.from_numpy(c2["configs_j"]).to(cuda_device)
    psi = torch.from_numpy(c2["psi"]).to(cuda_device)
    y_ref = ref.apply_within(fwd, ci, psi, cj)
    y = ham.apply_within(ci, psi, cj)
    assert (y - y_ref).abs().max().item() <= 1e-12 * y.abs().max().item() * 50
    x_ref = ref.apply_within(adj, cj, y, ci)
    x = ham.apply_within_adjoint(ci, y, cj)
    assert (x - x_ref).abs().max().item() <= 1e-12 * x.abs().max().item() * 50
