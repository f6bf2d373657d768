"""torch.ops.qmb_hamiltonian_<nq>_<pc> backed by this engine give the engine's results (and the reference's).

The operators are called the way the reference's Hamiltonian class calls
them (qmb/hamiltonian.py:104-206): term tensors on the device, amplitudes as
float64 [N, 2]; their results are compared with the golden fixtures the
reference produced and with the Hamiltonian methods.
"""

from __future__ import annotations

import importlib

import numpy as np
import pytest
import torch

from conftest import golden

torch_ops = importlib.import_module("qmb-public_gb300.torch_ops")

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["ab_initio_6_relative", "ab_initio_10_complex", "random_terms_bose2", "hubbard_3x2"])
def test_operators_reproduce_the_reference(case, cuda_device):
    g = golden(case)
    pc = int(g["particle_cut"])
    nq = g["configs_i"].shape[1]
    ops = getattr(torch.ops, torch_ops.register(nq, pc))
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda_device)  # noqa: E731
    site, kind, coef = d(g["site"]), d(g["kind"]), d(g["coef"])
    psi = torch.view_as_real(d(g["psi_i"])).contiguous()
    out = torch.view_as_complex(ops.apply_within(d(g["configs_i"]), psi, d(g["configs_j"]), site, kind, coef))
    scale = np.abs(g["coef"]).sum() * np.abs(g["psi_i"]).sum()
    assert np.abs(out.cpu().numpy() - g["psi_j"]).max() <= 1e-12 * scale
    diag = torch.view_as_complex(ops.diagonal_term(d(g["diag_configs"]), site, kind, coef)).cpu().numpy()
    assert np.abs(diag - g["diag"]).max() <= 1e-12 * np.abs(g["coef"]).sum()
    for key in [k for k in g if k.startswith("relative_")]:
        k = int(key.split("_")[1])
        rows = ops.find_relative(d(g["configs_i"]), psi, k, site, kind, coef, d(g["configs_i"])).cpu().numpy()
        assert np.array_equal(rows, g[key])
    srel = ops.single_relative(d(g["configs_i"]), site, kind, coef)
    assert srel.shape == (g["configs_i"].shape[0], nq) and srel.dtype == torch.uint8
