"""GB300-native second-quantized Hamiltonian engine (drop-in for qmb.hamiltonian)."""

from . import bitspack, terms  # noqa: F401
