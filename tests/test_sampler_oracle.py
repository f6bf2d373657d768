"""The oracle's restatement of the reference's network and unique sampler, pinned to the reference.

tests/golden/sampler_*.npz hold what the reference's own
WaveFunctionElectronUpDown (qmb/mlp.py) computed on the CPU: psi of seeded
configurations and the configurations generate_unique drew, with the
uniforms its Gumbel perturbation used.  The oracle (oracle/sampler.py) must
reproduce them on the CPU from the same parameters and uniforms: the same
rows in the same order, psi to FP32 rounding.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import golden
from oracle import sampler

CASES = ["sampler_6", "sampler_14", "sampler_10_custom"]


def load(case):
    g = golden(case)
    params = {k[6:]: torch.from_numpy(v) for k, v in g.items() if k.startswith("param:")}
    uniforms = [torch.from_numpy(g[f"uniform:{i}"]) for i in range(int(g["sites"]))]
    return g, params, uniforms


@pytest.mark.parametrize("case", CASES)
def test_oracle_forward_matches_reference(case):
    g, params, _ = load(case)
    psi = sampler.forward(params, int(g["sites"]), int(g["spin_up"]), int(g["spin_down"]),
                          torch.from_numpy(g["configs"])).numpy()
    assert np.allclose(psi, g["psi"], rtol=1e-5, atol=0)


@pytest.mark.parametrize("case", CASES)
def test_oracle_sampler_matches_reference(case):
    g, params, uniforms = load(case)
    configs, psi = sampler.generate_unique(params, int(g["sites"]), int(g["spin_up"]), int(g["spin_down"]),
                                           int(g["batch"]), uniforms)
    assert np.array_equal(configs.numpy(), g["sampled"])
    assert np.allclose(psi.numpy(), g["sampled_psi"], rtol=1e-5, atol=0)
    # unique rows, each with the right electron counts
    assert np.unique(g["sampled"], axis=0).shape[0] == g["sampled"].shape[0]
