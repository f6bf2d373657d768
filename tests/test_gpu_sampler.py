"""The autoregressive network and its unique sampler (qmb-public_gb300/sampler.py) on the GPU.

Against the reference itself (tests/golden/sampler_*.npz, produced by the
reference's qmb/mlp.py on the CPU): the reference's parameters load into
this module unchanged, psi agrees to 1e-5 (FP32 networks, cuBLAS against
the CPU's matrix products), and generate_unique replayed with the
reference's recorded uniforms draws the same rows in the same order (up to a
row traded across a near-tie of the final cut, as the GPU's FP32 products
round differently from the CPU's).  The
CUDA backward of the fused site sum is checked against torch autograd
through the oracle's plain-torch restatement, and a larger sampling run
against the oracle on the same GPU.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import golden
from oracle import sampler as oracle_sampler
from qmb_gb300 import sampler

pytestmark = pytest.mark.gpu

CASES = ["sampler_6", "sampler_14", "sampler_10_custom"]


def _network(g, device):
    net = sampler.WaveFunctionElectronUpDown(double_sites=2 * int(g["sites"]), physical_dim=2, is_complex=True,
                                             spin_up=int(g["spin_up"]), spin_down=int(g["spin_down"]),
                                             hidden_size=tuple(int(h) for h in g["hidden"]),
                                             ordering=[int(o) for o in g["ordering"]])
    state = {k[6:]: torch.from_numpy(v) for k, v in g.items() if k.startswith("param:")}
    net.load_state_dict(state, strict=True)
    return net.to(device), {k: v.to(device) for k, v in state.items()}


@pytest.mark.parametrize("case", CASES)
def test_forward_matches_reference(case, cuda_device):
    g = golden(case)
    net, _ = _network(g, cuda_device)
    with torch.no_grad():
        psi = net(torch.from_numpy(g["configs"]).to(cuda_device)).cpu().numpy()
    assert np.allclose(psi, g["psi"], rtol=1e-5, atol=0)


@pytest.mark.parametrize("case", CASES)
def test_sampler_replays_reference(case, cuda_device):
    g = golden(case)
    net, _ = _network(g, cuda_device)
    uniforms = [torch.from_numpy(g[f"uniform:{i}"]).to(cuda_device) for i in range(int(g["sites"]))]
    configs, psi, _, _ = net.generate_unique(int(g["batch"]), uniforms=uniforms)
    got, want = configs.cpu().numpy(), g["sampled"]
    assert got.shape == want.shape
    if not np.array_equal(got, want):
        # the GPU's FP32 matrix products round differently from the CPU's: a row may trade places
        # with another across a near-tie of the final cut (the output's last rows), nowhere else
        a, b = [bytes(r) for r in got], [bytes(r) for r in want]
        diff = set(a) ^ set(b)
        assert len(diff) <= 4
        n = len(a)
        for r in diff:
            at = a.index(r) if r in a else b.index(r)
            assert at >= n - max(4, n // 100), at
    rows = {bytes(r): i for i, r in enumerate(want)}
    common = [(i, rows[bytes(r)]) for i, r in enumerate(got) if bytes(r) in rows]
    mine, theirs = np.array([c[0] for c in common]), np.array([c[1] for c in common])
    assert np.allclose(psi.cpu().numpy()[mine], g["sampled_psi"][theirs], rtol=1e-5, atol=0)


def test_backward_matches_autograd_of_the_restatement(cuda_device):
    g = golden("sampler_14")
    net, params = _network(g, cuda_device)
    configs = torch.from_numpy(g["configs"]).to(cuda_device)
    # a loss linear in log psi, so that gradients keep their scale
    weights = torch.linspace(0.5, 1.5, configs.shape[0], device=cuda_device, dtype=torch.float64)
    loss = (torch.log(net(configs)).real * weights).sum()
    loss.backward()
    ref = {k: v.clone().requires_grad_(v.is_floating_point()) for k, v in params.items()}
    psi = oracle_sampler.forward(ref, int(g["sites"]), int(g["spin_up"]), int(g["spin_down"]), configs)
    (torch.log(psi).real * weights).sum().backward()
    named = dict(net.named_parameters())
    # elementwise to 1e-4, with an absolute floor of 1e-6 of the largest gradient entry of any
    # parameter: gradients that vanish in exact arithmetic (a site whose occupation the particle
    # numbers already fix) are FP32 rounding noise in both
    scale = max(v.grad.abs().max().item() for v in ref.values() if v.grad is not None)
    for k, v in ref.items():
        if k in named and v.grad is not None:
            got = named[k].grad
            assert torch.allclose(got, v.grad, rtol=1e-4, atol=1e-6 * scale), k


def test_large_sampling_run_matches_the_restatement_on_the_gpu(cuda_device):
    # 26 sites (52 spin orbitals), 7 + 7 electrons, 8,192 rows
    torch.manual_seed(5)
    net = sampler.WaveFunctionElectronUpDown(double_sites=52, physical_dim=2, is_complex=True, spin_up=7,
                                             spin_down=7, hidden_size=(256, 256), ordering=+1).to(cuda_device)
    with torch.no_grad():
        for p in net.parameters():
            p.mul_(3.0)
    params = {k: v.detach() for k, v in net.state_dict().items()}
    gen = torch.Generator(device=cuda_device).manual_seed(6)
    pool = [torch.rand((4 * 8192, 4), generator=gen, device=cuda_device) for _ in range(26)]
    draw = lambda site, rows: pool[site][:rows]  # noqa: E731  (both samplers draw the same uniforms)
    configs, psi, _, _ = net.generate_unique(8192, uniforms=draw)
    want, want_psi = oracle_sampler.generate_unique(params, 26, 7, 7, 8192, draw)
    assert configs.shape[0] == 8192
    a, b = {bytes(r) for r in configs.cpu().numpy()}, {bytes(r) for r in want.cpu().numpy()}
    # the same rows; a row may only trade places with another across a near-tie at the cut
    assert len(a ^ b) <= 8
    common = torch.from_numpy(np.array([np.frombuffer(r, dtype=np.uint8) for r in sorted(a & b)])).to(cuda_device)
    with torch.no_grad():
        assert torch.allclose(net(common), oracle_sampler.forward(params, 26, 7, 7, common), rtol=1e-5, atol=0)
        # psi summed while sampling equals the network's forward on the sampled rows
        assert torch.allclose(psi, net(configs), rtol=1e-5, atol=0)
