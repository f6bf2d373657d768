"""The engine under the reference's torch operator schemas (qmb/_hamiltonian.cpp:83-89).

The reference reaches its engine through ``torch.ops.qmb_hamiltonian_<nq>_<pc>``
(qmb/hamiltonian.py:37-69 loads a JIT extension that defines these four
operators).  ``register(n_qubytes, particle_cut)`` defines the same namespace
and schemas and implements them with this engine on CUDA tensors, so code
written against the operators runs unchanged:

    apply_within(Tensor configs_i, Tensor psi_i, Tensor configs_j, Tensor site, Tensor kind, Tensor coef) -> Tensor
    find_relative(Tensor configs_i, Tensor psi_i, int count_selected, Tensor site, Tensor kind, Tensor coef,
                  Tensor configs_exclude) -> Tensor
    diagonal_term(Tensor configs, Tensor site, Tensor kind, Tensor coef) -> Tensor
    single_relative(Tensor configs, Tensor site, Tensor kind, Tensor coef) -> Tensor

Amplitudes cross the operators as float64 [N, 2] (real, imaginary), as in
the reference.  Compiled term tables are cached per (site, kind, coef)
tensors and their versions.  Only CUDA implementations are registered: a
call with CPU tensors fails (this engine has no CPU path).
"""

from __future__ import annotations

import torch

from .hamiltonian import Hamiltonian

__all__ = ["register"]

_libraries: dict[str, torch.library.Library] = {}
_hamiltonians: dict = {}

SCHEMAS = {
    "apply_within": "apply_within(Tensor configs_i, Tensor psi_i, Tensor configs_j, Tensor site, Tensor kind, "
                    "Tensor coef) -> Tensor",
    "find_relative": "find_relative(Tensor configs_i, Tensor psi_i, int count_selected, Tensor site, Tensor kind, "
                     "Tensor coef, Tensor configs_exclude) -> Tensor",
    "diagonal_term": "diagonal_term(Tensor configs, Tensor site, Tensor kind, Tensor coef) -> Tensor",
    "single_relative": "single_relative(Tensor configs, Tensor site, Tensor kind, Tensor coef) -> Tensor",
}


def _hamiltonian(site: torch.Tensor, kind: torch.Tensor, coef: torch.Tensor, particle_cut: int) -> Hamiltonian:
    key = (particle_cut, site.data_ptr(), kind.data_ptr(), coef.data_ptr(), site._version, kind._version,
           coef._version, site.shape[0])
    ham = _hamiltonians.get(key)
    if ham is None:
        ham = Hamiltonian((site, kind, coef), kind="fermi" if particle_cut == 1 else "bose2")
        # one live entry per term table: older versions of the same tensors are stale
        for k in [k for k in _hamiltonians if k[:4] == key[:4]]:
            del _hamiltonians[k]
        _hamiltonians[key] = ham
    return ham


def _complex(psi: torch.Tensor) -> torch.Tensor:
    if psi.dtype != torch.float64 or psi.dim() != 2 or psi.shape[1] != 2:
        raise RuntimeError("psi must be float64 of shape [N, 2].")
    return torch.view_as_complex(psi.contiguous())


def register(n_qubytes: int, particle_cut: int) -> str:
    """Define torch.ops.qmb_hamiltonian_<n_qubytes>_<particle_cut> backed by this engine; returns the namespace."""
    if particle_cut not in (1, 2):
        raise ValueError("particle_cut must be 1 (fermions) or 2 (hard-core bosons)")
    ns = f"qmb_hamiltonian_{int(n_qubytes)}_{int(particle_cut)}"
    if ns in _libraries:
        return ns
    lib = torch.library.Library(ns, "DEF")
    for schema in SCHEMAS.values():
        lib.define(schema)

    def apply_within(configs_i, psi_i, configs_j, site, kind, coef):
        ham = _hamiltonian(site, kind, coef, particle_cut)
        return torch.view_as_real(ham.apply_within(configs_i, _complex(psi_i), configs_j)).contiguous()

    def find_relative(configs_i, psi_i, count_selected, site, kind, coef, configs_exclude):
        ham = _hamiltonian(site, kind, coef, particle_cut)
        return ham.find_relative(configs_i, _complex(psi_i), count_selected, configs_exclude)

    def diagonal_term(configs, site, kind, coef):
        ham = _hamiltonian(site, kind, coef, particle_cut)
        return torch.view_as_real(ham.diagonal_term(configs)).contiguous()

    def single_relative(configs, site, kind, coef):
        return _hamiltonian(site, kind, coef, particle_cut).single_relative(configs)

    for name, fn in (("apply_within", apply_within), ("find_relative", find_relative),
                     ("diagonal_term", diagonal_term), ("single_relative", single_relative)):
        lib.impl(name, fn, "CUDA")
    _libraries[ns] = lib
    return ns
