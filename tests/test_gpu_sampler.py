"""The autoregressive network and its unique sampler (qmb-public_gb300/sampler.py) on the GPU.

Against the reference itself (tests/golden/sampler_*.npz, produced by the
reference's qmb/mlp.py on the CPU): the reference's parameters load into
this module unchanged, psi agrees to 1e-5 (FP32 networks, cuBLAS against
the CPU's matrix products), and generate_unique replayed with the
reference's recorded uniforms draws the same rows (up to a few rows in 200
that trade places across near-ties, as the GPU's FP32 arithmetic rounds
differently from the CPU's).  The
CUDA backward of the fused site sum is checked against torch autograd
through the oracle's plain-torch restatement.  On the same GPU as the
restatement: a sharpened 26-site network site by site (the restatement's
state through this library's site kernel at every site), and a whole run
of an unsharpened network end to end.
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
        # the GPU's FP32 matrix products and exp/log round differently from the CPU's: where two
        # candidates tie to within that rounding, their order (and with it which uniforms their
        # children draw) can differ, so a few rows in 200 may differ from the reference's own run
        a, b = [bytes(r) for r in got], [bytes(r) for r in want]
        diff = set(a) ^ set(b)
        assert len(diff) <= max(4, len(a) // 200)
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


def test_sampling_steps_match_the_restatement_site_by_site(cuda_device):
    # 26 sites (52 spin orbitals), 7 + 7 electrons, 8,192 rows, sharpened parameters (x3). At every
    # site the restatement's state (rows, counts, log probabilities, Gumbel values, uniforms) goes
    # through this library's site kernel, which must give the restatement's children to FP32
    # rounding, and the same selected rows except across near-ties of the cut. (Run end to end,
    # an ulp-level difference that swaps two rows' order also swaps their uniforms at the next
    # site, so whole runs of a sharp network are compared step by step.)
    native = __import__("importlib").import_module("qmb-public_gb300._native")
    torch.manual_seed(5)
    sites, up, down, batch = 26, 7, 7, 8192
    net = sampler.WaveFunctionElectronUpDown(double_sites=2 * sites, physical_dim=2, is_complex=True, spin_up=up,
                                             spin_down=down, hidden_size=(256, 256), ordering=+1).to(cuda_device)
    with torch.no_grad():
        for p in net.parameters():
            p.mul_(3.0)
    params = {k: v.detach() for k, v in net.state_dict().items()}
    gen = torch.Generator(device=cuda_device).manual_seed(6)
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    x = torch.empty([1, 0, 2], dtype=torch.uint8, device=cuda_device)
    lp = torch.zeros(1, dtype=torch.float32, device=cuda_device)
    gp = torch.zeros(1, dtype=torch.float32, device=cuda_device)
    tail = torch.tensor([[0, 0], [0, 1], [1, 0], [1, 1]], dtype=torch.uint8, device=cuda_device)
    with torch.no_grad():
        for i in range(sites):
            n = x.shape[0]
            d = oracle_sampler._mlp(params, f"amplitude.{i}", x.to(torch.float32).reshape(n, 2 * i)).view(n, 2, 2)
            # the module's own network gives the restatement's raw amplitudes bit for bit
            assert torch.equal(net.amplitude[i](x.to(torch.float32).reshape(n, 2 * i)).view(n, 2, 2), d)
            dm = d + torch.where(oracle_sampler._mask(x, sites, up, down), 0.0, -torch.inf)
            lk = lp.view(n, 1) + (2 * oracle_sampler._normalize(dm)).view(n, 4)
            u = torch.rand((n, 4), generator=gen, device=cuda_device)
            g = lk - (-u.log()).log()
            z = g.max(dim=-1).values.view(n, 1)
            t = -torch.log(torch.exp(-gp.view(n, 1)) - torch.exp(-z) + torch.exp(-g))
            want_l, want_t = lk.t().reshape(4 * n), t.t().reshape(4 * n)
            counts = x.sum(dim=1).to(torch.int32).contiguous()
            got_l = torch.empty(4 * n, dtype=torch.float32, device=cuda_device)
            got_t = torch.empty(4 * n, dtype=torch.float32, device=cuda_device)
            native.call("qmbx_sampler_site", n, i, sites, up, down, d.contiguous().data_ptr(), counts.data_ptr(),
                        lp.contiguous().data_ptr(), gp.contiguous().data_ptr(), u.contiguous().data_ptr(),
                        got_l.data_ptr(), got_t.data_ptr(), None, None, None, stream)
            torch.cuda.synchronize(cuda_device)
            for got, want in ((got_l, want_l), (got_t, want_t)):
                fin = torch.isfinite(want)
                assert torch.equal(torch.isfinite(got), fin) and torch.equal(got[~fin], want[~fin])
                assert torch.allclose(got[fin], want[fin], rtol=2e-6, atol=1e-5)
            # the same rows selected, up to rows whose values tie the cut within FP32 rounding
            keep = want_t.argsort(descending=True)[:batch]
            mine = got_t.argsort(descending=True)[:batch]
            diff = set(keep.tolist()) ^ set(mine.tolist())
            if diff and 4 * n > batch:
                cut = want_t[keep[-1]].item()
                near = torch.tensor(sorted(diff), device=cuda_device)
                assert torch.allclose(want_t[near], torch.full_like(want_t[near], cut), rtol=1e-5, atol=1e-5)
            # the restatement's selection carries on
            x = torch.cat([x.repeat(4, 1, 1), tail.repeat_interleave(n, 0).unsqueeze(1)], dim=1)[keep]
            lp, gp = want_l[keep], want_t[keep]
            finite = gp.isfinite()
            x, lp, gp = x[finite], lp[finite], gp[finite]
    assert x.shape[0] == batch


def test_sampling_run_matches_the_restatement_end_to_end(cuda_device):
    # an unsharpened network (no near-ties to speak of): the whole run gives the restatement's rows
    torch.manual_seed(7)
    net = sampler.WaveFunctionElectronUpDown(double_sites=40, physical_dim=2, is_complex=True, spin_up=6,
                                             spin_down=6, hidden_size=(128, 128), ordering=-1).to(cuda_device)
    params = {k: v.detach() for k, v in net.state_dict().items()}
    gen = torch.Generator(device=cuda_device).manual_seed(8)
    pool = [torch.rand((4 * 4096, 4), generator=gen, device=cuda_device) for _ in range(20)]
    draw = lambda site, rows: pool[site][:rows]  # noqa: E731  (both samplers draw the same uniforms)
    configs, psi, _, _ = net.generate_unique(4096, uniforms=draw)
    want, want_psi = oracle_sampler.generate_unique(params, 20, 6, 6, 4096, draw)
    a, b = {bytes(r) for r in configs.cpu().numpy()}, {bytes(r) for r in want.cpu().numpy()}
    assert configs.shape[0] == want.shape[0]
    assert len(a ^ b) <= max(2, configs.shape[0] // 500)
    common = torch.from_numpy(np.array([np.frombuffer(r, dtype=np.uint8) for r in sorted(a & b)])).to(cuda_device)
    with torch.no_grad():
        assert torch.allclose(net(common), oracle_sampler.forward(params, 20, 6, 6, common), rtol=1e-5, atol=0)
        # psi summed while sampling equals the network's forward on the sampled rows
        assert torch.allclose(psi, net(configs), rtol=1e-5, atol=0)


def test_site_kernel_sorts_nan_and_inf_values_after_the_finite_ones(cuda_device):
    # a row whose children's perturbed log probabilities all lie below -88 has exp(-Z) = inf and
    # conditioned values NaN; the reference's descending sort puts those first and then drops them.
    # With a counter the site kernel writes them as -FLT_MAX (after the finite values) and counts
    # them, and the take kernel drops the places they took at the top of the reference's sort.
    native = __import__("importlib").import_module("qmb-public_gb300._native")
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    sites, up, down, n, batch = 4, 2, 2, 3, 5
    delta = torch.zeros((n, 4), dtype=torch.float32, device=cuda_device)
    counts = torch.zeros((n, 2), dtype=torch.int32, device=cuda_device)
    lp = torch.tensor([0.0, -400.0, -1.0], dtype=torch.float32, device=cuda_device)  # row 1: far below -88
    gp = torch.tensor([0.0, -0.5, -0.25], dtype=torch.float32, device=cuda_device)
    u = torch.tensor([[0.1, 0.3, 0.5, 0.7]] * n, dtype=torch.float32, device=cuda_device)  # no ties
    l_all = torch.empty(4 * n, dtype=torch.float32, device=cuda_device)
    t_all = torch.empty(4 * n, dtype=torch.float32, device=cuda_device)
    raw = torch.empty(4 * n, dtype=torch.float32, device=cuda_device)
    native.call("qmbx_sampler_site", n, 0, sites, up, down, delta.data_ptr(), counts.data_ptr(), lp.data_ptr(),
                gp.data_ptr(), u.data_ptr(), l_all.data_ptr(), raw.data_ptr(), None, None, None, stream)
    bad = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    native.call("qmbx_sampler_site", n, 0, sites, up, down, delta.data_ptr(), counts.data_ptr(), lp.data_ptr(),
                gp.data_ptr(), u.data_ptr(), l_all.data_ptr(), t_all.data_ptr(), None, None, bad.data_ptr(), stream)
    torch.cuda.synchronize(cuda_device)
    not_finite = ~torch.isfinite(raw) & (raw != -torch.inf)  # NaN or +inf
    k = int(not_finite.sum())
    assert k > 0 and int(bad.item()) == k
    assert torch.equal(t_all[not_finite], torch.full((k,), torch.finfo(torch.float32).min, device=cuda_device))
    assert torch.equal(t_all[~not_finite], raw[~not_finite])
    # the reference keeps the finite values among the first `batch` of its descending sort (NaN first)
    ref_order = torch.argsort(torch.where(torch.isnan(raw), torch.inf, raw), descending=True)[:batch]
    kept_ref = [int(i) for i in ref_order if torch.isfinite(raw[i])]
    index = torch.argsort(t_all, descending=True)[:batch].contiguous()
    m = index.shape[0]
    occ = torch.zeros((n, sites), dtype=torch.uint8, device=cuda_device)
    out = dict(occ=torch.empty((m, sites), dtype=torch.uint8, device=cuda_device),
               xf=torch.zeros((m, 2 * sites), dtype=torch.float32, device=cuda_device),
               counts=torch.empty((m, 2), dtype=torch.int32, device=cuda_device),
               lp=torch.empty(m, dtype=torch.float32, device=cuda_device),
               gp=torch.empty(m, dtype=torch.float32, device=cuda_device))
    native.call("qmbx_sampler_take", m, n, 0, sites, index.data_ptr(), occ.data_ptr(), counts.data_ptr(),
                l_all.data_ptr(), t_all.data_ptr(), out["occ"].data_ptr(), out["xf"].data_ptr(),
                out["counts"].data_ptr(), out["lp"].data_ptr(), out["gp"].data_ptr(), None, None, batch,
                bad.data_ptr(), stream)
    torch.cuda.synchronize(cuda_device)
    kept = [int(index[j]) for j in range(m) if torch.isfinite(out["gp"][j])]
    assert kept == kept_ref
