"""The reference's autoregressive network and its unique sampler, restated in plain torch — TEST INFRASTRUCTURE ONLY.

A restatement of qmb/mlp.py:60-314 (``WaveFunctionElectronUpDown``:
``forward`` and ``generate_unique``, the Gumbel top-k sampling without
replacement of https://arxiv.org/pdf/2408.07625) as functions of a
parameter dictionary with the reference module's state_dict keys
(``amplitude.<site>.model.<layer>.weight|bias``, ``phase.model.<layer>...``,
``ordering``).  The uniforms of the Gumbel perturbation are passed in, one
[L, 4] tensor per site, so that a run can be replayed.  Pinned by
tests/golden/sampler_*.npz, which the reference itself produced; used by the
tests and by bench.py's reference arm for the sampler, never by the product.
"""

from __future__ import annotations

import torch


def _unpack(configs: torch.Tensor, n_bits: int) -> torch.Tensor:
    """uint8 rows (bit b of byte k is element 8k + b) -> [rows, n_bits] uint8 (qmb/bitspack.py layout)."""
    shifts = torch.arange(8, device=configs.device, dtype=torch.uint8)
    bits = (configs.unsqueeze(-1) >> shifts) & 1
    return bits.reshape(configs.shape[0], -1)[:, :n_bits]


def _pack(bits: torch.Tensor) -> torch.Tensor:
    """[rows, n] 0/1 uint8 -> uint8 rows (bitspack layout, last byte zero-padded)."""
    n = bits.shape[1]
    pad = (-n) % 8
    if pad:
        bits = torch.nn.functional.pad(bits, (0, pad))
    weights = (1 << torch.arange(8, device=bits.device, dtype=torch.int32))
    return (bits.reshape(bits.shape[0], -1, 8).to(torch.int32) * weights).sum(-1).to(torch.uint8)


def _mlp(params: dict, prefix: str, x: torch.Tensor) -> torch.Tensor:
    """The layers prefix.model.<k> (Linear, SiLU, ..., Linear); a layer without weight is a bias alone."""
    layers = sorted({int(k[len(prefix) + 7:].split(".")[0]) for k in params if k.startswith(prefix + ".model.")})
    for n, k in enumerate(layers):
        if n > 0:
            x = torch.nn.functional.silu(x)
        w = params.get(f"{prefix}.model.{k}.weight")
        b = params[f"{prefix}.model.{k}.bias"]
        x = b.view(1, -1).expand(x.shape[0], -1) if w is None else torch.nn.functional.linear(x, w, b)
    return x


def _mask(x: torch.Tensor, sites: int, up: int, down: int) -> torch.Tensor:
    """[L, 2, 2] bool: which (up, down) pair may follow the partial configurations x [L, i, 2]."""
    i = x.shape[1]
    count = x.sum(dim=1)
    n_up, n_down = count[:, 0], count[:, 1]
    can_up = torch.stack([(i - n_up) < sites - up, n_up < up], dim=-1)
    can_down = torch.stack([(i - n_down) < sites - down, n_down < down], dim=-1)
    return can_up.unsqueeze(-1) & can_down.unsqueeze(-2)


def _normalize(d: torch.Tensor) -> torch.Tensor:
    """Shift the log amplitudes of every [2, 2] block so that their squared exponentials sum to one."""
    return d - ((2 * d).exp().sum(dim=[-2, -1]).log() / 2).unsqueeze(-1).unsqueeze(-1)


def forward(params: dict, sites: int, up: int, down: int, configs: torch.Tensor) -> torch.Tensor:
    """psi (complex128) of packed configurations (qmb/mlp.py forward)."""
    dtype = params["phase.model.0.bias"].dtype
    b = configs.shape[0]
    order = params["ordering"]
    inverse = torch.empty_like(order)
    inverse[order] = torch.arange(sites, device=order.device)
    x = _unpack(configs, 2 * sites).view(b, sites, 2).index_select(1, inverse)
    xf = x.to(dtype)
    rows = torch.arange(b, device=configs.device)
    total = torch.zeros(b, dtype=torch.float64, device=configs.device)
    for i in range(sites):
        d = _mlp(params, f"amplitude.{i}", xf[:, :i].reshape(b, 2 * i)).view(b, 2, 2)
        d = d + torch.where(_mask(x[:, :i], sites, up, down), 0.0, -torch.inf)
        nd = _normalize(d)
        xi = x[:, i].to(torch.int64)
        total = total + nd[rows, xi[:, 0], xi[:, 1]].double()
    phase = _mlp(params, "phase", xf.reshape(b, 2 * sites)).view(b)
    return torch.complex(total, phase.double()).exp()


def generate_unique(params: dict, sites: int, up: int, down: int, batch: int, uniforms):
    """(packed configurations, psi): the reference's unique sampler with the given per-site uniforms.

    ``uniforms``: one [rows, 4] tensor per site, or a function (site, rows) -> such a tensor.
    """
    device = params["phase.model.0.bias"].device
    dtype = params["phase.model.0.bias"].dtype
    x = torch.empty([1, 0, 2], dtype=torch.uint8, device=device)
    lp = torch.zeros(1, dtype=dtype, device=device)   # unperturbed log probability
    gp = torch.zeros(1, dtype=dtype, device=device)   # perturbed (Gumbel) log probability
    for i in range(sites):
        n = x.shape[0]
        d = _mlp(params, f"amplitude.{i}", x.to(dtype).reshape(n, 2 * i)).view(n, 2, 2)
        d = d + torch.where(_mask(x, sites, up, down), 0.0, -torch.inf)
        l = lp.view(n, 1) + (2 * _normalize(d)).view(n, 4)
        u = uniforms(i, n) if callable(uniforms) else uniforms[i]
        g = l - (-u.log()).log()
        z = g.max(dim=-1).values.view(n, 1)
        t = -torch.log(torch.exp(-gp.view(n, 1)) - torch.exp(-z) + torch.exp(-g))
        # candidates: every row with (0, 0), then every row with (0, 1), (1, 0), (1, 1)
        tail = torch.tensor([[0, 0], [0, 1], [1, 0], [1, 1]], dtype=torch.uint8, device=device)
        x = torch.cat([x.repeat(4, 1, 1), tail.repeat_interleave(n, 0).unsqueeze(1)], dim=1)
        lp = l.t().reshape(4 * n)
        gp = t.t().reshape(4 * n)
        keep = gp.argsort(descending=True)[:batch]
        x, lp, gp = x[keep], lp[keep], gp[keep]
        finite = gp.isfinite()
        x, lp, gp = x[finite], lp[finite], gp[finite]
    x = x.index_select(1, params["ordering"]).reshape(x.shape[0], 2 * sites)
    configs = _pack(x)
    return configs, forward(params, sites, up, down, configs)
