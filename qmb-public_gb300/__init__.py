"""GB300-native second-quantized Hamiltonian engine (drop-in for qmb.hamiltonian).

``Hamiltonian`` keeps the reference's constructor and its four operators
(apply_within, find_relative, diagonal_term, single_relative); the work runs
in hand-written sm_103a CUDA kernels behind the C ABI of include/qmbx.h.
"""

from . import bitspack, sampler, terms  # noqa: F401
from .energy import variational_energy  # noqa: F401
from .hamiltonian import Hamiltonian, HamiltonianMatrix  # noqa: F401
from .solvers import lanczos_energy, pt2_energy  # noqa: F401

__all__ = ["Hamiltonian", "HamiltonianMatrix", "variational_energy", "lanczos_energy", "pt2_energy", "bitspack", "sampler", "terms"]
