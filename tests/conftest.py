"""Shared test set-up: the ``gpu`` marker, import paths and golden-fixture loading."""

from __future__ import annotations

import importlib
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)

# The package directory is named qmb-public_gb300; expose it as qmb_gb300.
if "qmb_gb300" not in sys.modules:
    sys.modules["qmb_gb300"] = importlib.import_module("qmb-public_gb300")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libqmbx.so")


def golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as data:
        return {k: data[k] for k in data.files}


GOLDEN_CASES = [
    "ab_initio_6",
    "ab_initio_6_relative",
    "ab_initio_10_complex",
    "random_terms_fermi",
    "random_terms_bose2",
    "ising_4x4",
    "ising_4x4_relative",
    "hubbard_3x2",
    "edge_duplicates",
]


@pytest.fixture(scope="session")
def cuda_device():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
