"""The engine registered under the reference's operator schemas (torch_ops.register), host side.

The namespace and the four schemas must be exactly the reference's
(qmb/_hamiltonian.cpp:83-89), registration is idempotent, and a call with
CPU tensors fails (the engine registers CUDA implementations only).
"""

from __future__ import annotations

import importlib

import pytest
import torch

from conftest import golden

torch_ops = importlib.import_module("qmb-public_gb300.torch_ops")

REFERENCE_SCHEMAS = {
    "apply_within": "(Tensor configs_i, Tensor psi_i, Tensor configs_j, Tensor site, Tensor kind, Tensor coef) -> Tensor",
    "find_relative": "(Tensor configs_i, Tensor psi_i, int count_selected, Tensor site, Tensor kind, Tensor coef, "
                     "Tensor configs_exclude) -> Tensor",
    "diagonal_term": "(Tensor configs, Tensor site, Tensor kind, Tensor coef) -> Tensor",
    "single_relative": "(Tensor configs, Tensor site, Tensor kind, Tensor coef) -> Tensor",
}


def test_schemas_are_the_reference_ones():
    ns = torch_ops.register(2, 1)
    assert ns == "qmb_hamiltonian_2_1"
    assert torch_ops.register(2, 1) == ns  # idempotent
    ops = getattr(torch.ops, ns)
    for name, args in REFERENCE_SCHEMAS.items():
        schema = str(getattr(ops, name).default._schema)
        assert schema == f"{ns}::{name}{args}", schema


def test_cpu_tensors_are_rejected():
    ns = torch_ops.register(2, 1)
    g = golden("ab_initio_6")
    ops = getattr(torch.ops, ns)
    psi = torch.view_as_real(torch.from_numpy(g["psi_i"])).contiguous()
    with pytest.raises(Exception):
        ops.apply_within(torch.from_numpy(g["configs_i"]), psi, torch.from_numpy(g["configs_j"]),
                         torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"]))
