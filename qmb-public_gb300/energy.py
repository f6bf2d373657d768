"""Variational energy Re<psi|H|psi> / <psi|psi> with FP64 reductions.

The reference evaluates this on the caller side (qmb/vmc.py:104-116,
qmb/haar.py:491) with the Hamiltonian application detached from autograd.
Here H psi goes through ``Hamiltonian.apply_within``'s autograd function, whose
backward is the adjoint kernel, so the energy backpropagates into psi (and
from there into whatever produced psi).  complex64 amplitudes use the
compensated FP32 kernels for H psi and H^dagger g; the diagonal term, the
norm and the quotient stay in FP64.
"""

from __future__ import annotations

import torch

from .hamiltonian import Hamiltonian

__all__ = ["variational_energy"]


def variational_energy(ham: Hamiltonian, configs: torch.Tensor, psi: torch.Tensor) -> torch.Tensor:
    """Re<psi|H|psi> / <psi|psi> over one set of configurations; a float64 scalar."""
    if psi.dtype == torch.complex64:
        hpsi = ham.apply_within_compensated(configs, psi, configs)
    elif psi.dtype == torch.complex128:
        hpsi = ham.apply_within(configs, psi, configs)
    else:
        raise RuntimeError("psi must be complex64 or complex128")
    psi64 = psi.to(torch.complex128)
    numerator = torch.sum(psi64.conj() * hpsi).real
    denominator = torch.sum(psi64.conj() * psi64).real
    return numerator / denominator
