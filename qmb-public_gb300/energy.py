"""Variational energy Re<psi|H|psi> / <psi|psi> with FP64 reductions.

The reference evaluates this on the caller side (qmb/vmc.py:104-116,
qmb/haar.py:491) with the Hamiltonian application detached from autograd.
Here the energy backpropagates into psi (and from there into whatever
produced psi).  For a Hermitian operator (checked once per compiled table)
the gradient needs H psi only: dE/dpsi* = (H psi - E psi) / <psi|psi>, so one
term walk serves the energy and its gradient.  Otherwise H psi goes through
``Hamiltonian.apply_within``'s autograd function, whose backward is the
adjoint kernel.  complex64 amplitudes use the compensated FP32 kernels; the
diagonal term, the norm and the quotient stay in FP64.
"""

from __future__ import annotations

import torch

from .hamiltonian import Hamiltonian

__all__ = ["variational_energy"]


class _HermitianEnergy(torch.autograd.Function):
    """E = Re<psi|H psi> / <psi|psi> for Hermitian H; backward from the saved H psi."""

    @staticmethod
    def forward(ctx, ham: Hamiltonian, configs, psi):
        if psi.dtype == torch.complex64:
            hpsi = ham.apply_within_compensated(configs, psi.detach(), configs)
        else:
            hpsi = ham.apply_within(configs, psi.detach(), configs)
        psi64 = psi.detach().to(torch.complex128)
        norm = torch.sum(psi64.conj() * psi64).real
        energy = torch.sum(psi64.conj() * hpsi).real / norm
        ctx.in_dtype = psi.dtype
        ctx.save_for_backward(hpsi, psi64, energy, norm)
        return energy

    @staticmethod
    def backward(ctx, grad):
        hpsi, psi64, energy, norm = ctx.saved_tensors
        # torch's gradient of a real loss in a complex input is 2 dL/dpsi*
        g = grad * 2.0 * (hpsi - energy * psi64) / norm
        return None, None, g.to(ctx.in_dtype)


def variational_energy(ham: Hamiltonian, configs: torch.Tensor, psi: torch.Tensor, *,
                       hermitian_shortcut: bool = True) -> torch.Tensor:
    """Re<psi|H|psi> / <psi|psi> over one set of configurations; a float64 scalar.

    With ``hermitian_shortcut`` (the default) a Hermitian operator takes its
    gradient from the saved H psi; ``hermitian_shortcut=False`` always sends
    the backward pass through the adjoint kernel (``apply_within``'s autograd
    function), which the gradient checks use to exercise that kernel.
    """
    if psi.dtype not in (torch.complex64, torch.complex128):
        raise RuntimeError("psi must be complex64 or complex128")
    if hermitian_shortcut and psi.requires_grad and torch.is_grad_enabled() and configs.dim() == 2 and \
            ham._table(configs.device, configs.shape[1]).hermitian:
        return _HermitianEnergy.apply(ham, configs, psi)
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
