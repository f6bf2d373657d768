"""Callers of the engine that run on the device: Lanczos and the PT2 step.

``lanczos_energy`` restates the Lanczos iteration of qmb/rldiag.py:19-52 (and
the loop of qmb/haar.py:107-183): repeated square applications of H on a
fixed basis, the three-term recurrence on device in complex128, and the
lowest Ritz pair from SciPy's ``eigh_tridiagonal`` ('stebz').  Unlike the
reference, H is materialised once on the basis as a sparse matrix
(``Hamiltonian.matrix``: two term walks) and every iteration is a sparse
matrix-vector product, unless the matrix would not fit the memory budget, in
which case every iteration walks the terms (``apply_within``) as the
reference does; the Krylov vectors stay in device memory (a GB300 holds
~280 GB), so no vector is copied to the host inside the loop.

``pt2_energy`` restates the Epstein-Nesbet second-order step of
qmb/pert.py:37-61: E0 = <psi|H|psi>/<psi|psi>, the connected space from
``find_relative``, H psi on it from ``apply_within`` and the denominators
from ``diagonal_term``; by default as one engine call (``Hamiltonian.pt2``)
that takes E0 from find_relative's own walk.
"""

from __future__ import annotations

import functools

import scipy.linalg
import torch

from .hamiltonian import Hamiltonian

__all__ = ["lanczos_energy", "pt2_energy"]


def _matrix_budget(device: torch.device) -> int:
    """Entries of a materialised matrix allowed on `device`: a quarter of its free memory at 20 bytes each."""
    free, _total = torch.cuda.mem_get_info(device)
    return free // 4 // 20


def lanczos_energy(ham: Hamiltonian, configs: torch.Tensor, step: int, threshold: float = 1e-12, *,
                   start: torch.Tensor | None = None, generator: torch.Generator | None = None,
                   materialize: bool = True):
    """Lowest eigenvalue (float) and eigenvector (complex128) of H restricted to ``configs``.

    With ``materialize`` (the default) H is stored once as a sparse matrix on
    the distinct rows of ``configs`` when it fits a quarter of the free
    device memory; otherwise every iteration calls ``apply_within``.
    """
    if start is None:
        start = torch.randn([configs.size(0)], dtype=torch.complex128, device=configs.device, generator=generator)
    apply = functools.partial(ham.apply_within, configs, configs_j=configs)
    if materialize and configs.is_cuda and configs.size(0) > 0:
        mat = ham.matrix(configs, max_entries=_matrix_budget(configs.device)) \
            if torch.unique(configs, dim=0).shape[0] == configs.shape[0] else None
        if mat is not None:
            apply = mat.apply
    v = [start.to(torch.complex128) / torch.linalg.norm(start)]
    alpha: list[torch.Tensor] = []
    beta: list[torch.Tensor] = []
    w = apply(v[-1])
    alpha.append((w.conj() @ v[-1]).real)
    w = w - alpha[-1] * v[-1]
    i = 0
    while True:
        norm_w = torch.linalg.norm(w)
        if norm_w < threshold:
            break
        beta.append(norm_w)
        v.append(w / beta[-1])
        w = apply(v[-1])
        alpha.append((w.conj() @ v[-1]).real)
        if i == step:
            break
        w = w - alpha[-1] * v[-1] - beta[-1] * v[-2]
        i += 1
    if len(beta) == 0:
        return alpha[0].item(), v[0]
    vals, vecs = scipy.linalg.eigh_tridiagonal(torch.stack(alpha).cpu().numpy(), torch.stack(beta).cpu().numpy(),
                                               lapack_driver="stebz", select="i", select_range=(0, 0))
    result = functools.reduce(torch.add, (float(weight[0]) * vector for weight, vector in zip(vecs, v)))
    return float(vals[0]), result


def pt2_energy(ham: Hamiltonian, configs: torch.Tensor, psi: torch.Tensor, count_selected: int, *,
               fused: bool = True):
    """(E0, E2): the variational energy of psi and its second-order correction over the connected space.

    ``fused`` (the default) runs the step as one engine call (``Hamiltonian.pt2``:
    E0 summed by find_relative's emission pass, everything on the device);
    ``fused=False`` composes the four operators as qmb/pert.py:37-61 does.
    """
    if fused and count_selected > 0 and configs.is_cuda:
        e0, e2, _ = ham.pt2(configs, psi, count_selected)
        return e0, e2
    psi = psi.to(torch.complex128)
    energy0 = ((psi.conj() @ ham.apply_within(configs, psi, configs)) / (psi.conj() @ psi)).real.item()
    other = ham.find_relative(configs, psi, count_selected, configs)
    hpsi = ham.apply_within(configs, psi, other)
    numerator = (hpsi.conj() * hpsi).real / (psi.conj() @ psi).real
    denominator = energy0 - ham.diagonal_term(other).real
    return energy0, (numerator / denominator).sum().item()
