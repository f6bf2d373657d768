"""The oracle against the reference's own compiled CPU engine.

oracle/ref_build.py compiles the reference's qmb/_hamiltonian.cpp and
qmb/_hamiltonian_cpu.cpp (with the flags its JIT build uses) into
oracle/_ref/libqmb_ref_cpu_4_1.so where the reference's sources are present.
When that library exists, the oracle must reproduce its apply_within and
find_relative exactly on slices of the benchmark workload C2 (n_qubytes 4).
The library is host code for the machine that built it, so elsewhere these
tests skip.
"""

from __future__ import annotations

import os

import numpy as np
import pytest
import torch

import bench
import oracle
from oracle import ref_build

LIB = ref_build.cpu_library(4, 1)

pytestmark = pytest.mark.skipif(not os.path.exists(LIB), reason="reference CPU build absent (oracle/ref_build.py)")


@pytest.fixture(scope="module")
def ref_ops():
    torch.ops.load_library(LIB)
    return torch.ops.qmb_hamiltonian_4_1


@pytest.fixture(scope="module")
def c2():
    return bench.make_workload("c2")


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a))


@pytest.mark.parametrize("rows", [(0, 300), (9000, 9400)])
def test_oracle_apply_within_equals_reference_build(ref_ops, c2, rows):
    a, b = rows
    ci, psi, cj = c2["configs_i"][a:b], c2["psi"][a:b], c2["configs_j"]
    ref = ref_ops.apply_within(_t(ci), torch.view_as_real(_t(psi)).contiguous(), _t(cj), _t(c2["site"]),
                               _t(c2["kind"]), _t(c2["coef"]))
    got = oracle.apply_within(c2["site"], c2["kind"], c2["coef"], ci, psi, cj)
    assert np.array_equal(torch.view_as_complex(ref).numpy(), got)


@pytest.mark.parametrize("k", [1, 500, 20000])
def test_oracle_find_relative_equals_reference_build(ref_ops, c2, k):
    ci, psi = c2["configs_i"][:400], c2["psi"][:400]
    ref = ref_ops.find_relative(_t(ci), torch.view_as_real(_t(psi)).contiguous(), k, _t(c2["site"]), _t(c2["kind"]),
                                _t(c2["coef"]), _t(c2["configs_i"]))
    got = oracle.find_relative(c2["site"], c2["kind"], c2["coef"], ci, psi, k, c2["configs_i"], rule="heap")
    assert np.array_equal(ref.numpy(), got)
