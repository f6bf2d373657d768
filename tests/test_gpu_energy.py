"""Variational energy and its gradient through the adjoint kernel.

E(psi) = Re<psi|H|psi> / <psi|psi> with H psi from apply_within (FP64 or the
FP32-compensated path) and the backward pass through the hand-written
adjoint (a replay of the forward walk's hits, or the adjoint walk).  Checked against a dense FP64 H built by the CPU oracle (energy to
1e-12 relative, gradient to 1e-10 relative), against central finite
differences (1e-6 relative), and, through a small MLP wave function, against
the same network evaluated with the dense matrix in torch.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from conftest import golden
from qmb_gb300 import Hamiltonian, terms, variational_energy

pytestmark = pytest.mark.gpu


def _setup(case="ab_initio_10_complex"):
    g = golden(case)
    rows = terms.unique_rows(np.concatenate([g["configs_i"], g["configs_j"]]))
    h = oracle.dense_matrix(g["site"], g["kind"], g["coef"], rows, int(g["particle_cut"]))
    ham = Hamiltonian((torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"])),
                      kind="fermi" if int(g["particle_cut"]) == 1 else "bose2")
    return g, rows, h, ham


def _dense_energy_and_grad(h, psi):
    n = np.vdot(psi, psi).real
    e = np.vdot(psi, h @ psi).real / n
    grad = ((h + h.conj().T) @ psi - 2 * e * psi) / n
    return e, grad


@pytest.mark.parametrize("hit_log", [True, False])
@pytest.mark.parametrize("case", ["ab_initio_10_complex", "ab_initio_6", "random_terms_fermi"])
def test_energy_and_gradient_match_dense_fp64(case, hit_log, cuda_device):
    """Non-Hermitian operators (random_terms_fermi) take the backward of apply_within: from the
    forward walk's hit log, or (hit_log False) from the adjoint kernel's walk."""
    g, rows, h, ham = _setup(case)
    ham.hit_log = hit_log
    rng = np.random.default_rng(1)
    psi0 = rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])
    c = torch.from_numpy(rows).to(cuda_device)
    psi = torch.from_numpy(psi0).to(cuda_device).requires_grad_(True)
    energy = variational_energy(ham, c, psi)
    energy.backward()
    e_ref, grad_ref = _dense_energy_and_grad(h, psi0)
    scale = np.abs(h).sum() / rows.shape[0] + 1.0
    assert abs(energy.item() - e_ref) <= 1e-12 * scale
    grad = psi.grad.cpu().numpy()
    assert np.abs(grad - grad_ref).max() <= 1e-10 * np.abs(grad_ref).max()


def test_energy_gradient_matches_finite_differences(cuda_device):
    g, rows, h, ham = _setup()
    rng = np.random.default_rng(2)
    psi0 = rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])
    c = torch.from_numpy(rows).to(cuda_device)
    psi = torch.from_numpy(psi0).to(cuda_device).requires_grad_(True)
    variational_energy(ham, c, psi).backward()
    grad = psi.grad.cpu().numpy()
    eps = 1e-6
    with torch.no_grad():
        for _ in range(3):
            d = rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])
            dt = torch.from_numpy(d).to(cuda_device)
            plus = variational_energy(ham, c, torch.from_numpy(psi0).to(cuda_device) + eps * dt).item()
            minus = variational_energy(ham, c, torch.from_numpy(psi0).to(cuda_device) - eps * dt).item()
            fd = (plus - minus) / (2 * eps)
            # torch's gradient of a real loss is dL/dRe + i dL/dIm
            analytic = np.sum(grad.real * d.real + grad.imag * d.imag)
            assert abs(fd - analytic) <= 1e-6 * max(1.0, abs(analytic))


def test_compensated_fp32_energy_and_gradient(cuda_device):
    g, rows, h, ham = _setup()
    rng = np.random.default_rng(3)
    psi0 = (rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])).astype(np.complex64)
    c = torch.from_numpy(rows).to(cuda_device)
    p32 = torch.from_numpy(psi0).to(cuda_device).requires_grad_(True)
    p64 = torch.from_numpy(psi0.astype(np.complex128)).to(cuda_device).requires_grad_(True)
    e32 = variational_energy(ham, c, p32)
    e64 = variational_energy(ham, c, p64)
    e32.backward()
    e64.backward()
    # energy error of the FP32 path against FP64 on the same amplitudes: well below 1e-7 Ha
    assert abs(e32.item() - e64.item()) <= 1e-9 * (1 + abs(e64.item()))
    g32 = p32.grad.cpu().numpy().astype(np.complex128)
    g64 = p64.grad.cpu().numpy()
    assert np.abs(g32 - g64).max() <= 1e-6 * np.abs(g64).max()


class _TinyNet(torch.nn.Module):
    """Unpacked occupation bits -> (log|psi|, phase); FP32 like the reference's networks."""

    def __init__(self, n_sites: int):
        super().__init__()
        self.n_sites = n_sites
        self.body = torch.nn.Sequential(torch.nn.Linear(n_sites, 32), torch.nn.SiLU(), torch.nn.Linear(32, 32),
                                        torch.nn.SiLU(), torch.nn.Linear(32, 2))

    def forward(self, configs: torch.Tensor) -> torch.Tensor:
        from qmb_gb300 import bitspack

        bits = bitspack.unpack_int(configs, 1, self.n_sites).to(torch.float32)
        out = self.body(bits)
        return torch.polar(torch.exp(out[:, 0]), out[:, 1])


def test_energy_backpropagates_into_network(cuda_device):
    g, rows, h, ham = _setup()
    torch.manual_seed(0)
    net = _TinyNet(8 * rows.shape[1]).to(cuda_device)
    c = torch.from_numpy(rows).to(cuda_device)
    hd = torch.from_numpy(h).to(cuda_device)

    def dense_energy(psi):
        psi = psi.to(torch.complex128)
        return (psi.conj() @ (hd @ psi)).real / (psi.conj() @ psi).real

    for use_engine in (True, False):
        net.zero_grad()
        psi = net(c)
        e = variational_energy(ham, c, psi.to(torch.complex128)) if use_engine else dense_energy(psi)
        e.backward()
        grads = [p.grad.detach().clone() for p in net.parameters()]
        if use_engine:
            engine = (e.item(), grads)
        else:
            dense = (e.item(), grads)
    assert abs(engine[0] - dense[0]) <= 1e-10 * (1 + abs(dense[0]))
    for a, b in zip(engine[1], dense[1]):
        assert torch.allclose(a, b, rtol=1e-4, atol=1e-6 * (1 + b.abs().max().item()))
