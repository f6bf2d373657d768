"""The autoregressive MLP wave function and its unique sampler (drop-in for qmb/mlp.py:60-314).

``WaveFunctionElectronUpDown`` keeps the reference's constructor, submodule
names and parameter layout (``amplitude.<site>.model.<k>``, ``phase.model.<k>``,
``ordering``), so a reference state_dict loads unchanged, and its two
methods:

* ``forward(configs)``: psi of packed configurations (complex128);
* ``generate_unique(batch_size, block_num=1)``: Gumbel top-k sampling without
  replacement, site by site (https://arxiv.org/pdf/2408.07625), returning
  ``(configs, psi, None, None)``.  The reference ends by running the whole
  network again on the sampled rows for psi; here the log amplitudes are
  summed while sampling (the same normalised FP32 terms, summed in FP64 in
  the same site order) and only the phase network runs at the end, which
  halves the matrix products.  The reference drops the candidates whose
  value is not finite after every site (a host round trip for their
  count); here they ride along as rows without children and are dropped
  once at the end.  The rows kept, their order and the uniforms they draw
  are the same.  psi is
  returned detached (callers use it as data: qmb/vmc.py:84,
  qmb/haar.py:373).

The per-site networks are torch ``Linear`` layers (cuBLAS matrix products);
everything elementwise between them runs in this package's CUDA kernels
(libqmbx.so, csrc/sampler.cu): the particle-number mask, the normalisation
and the per-row sum over sites of ``forward`` (one kernel, with its own
backward for training), and each sampling site's mask, normalisation,
Gumbel perturbation and conditioning (one kernel) followed by the
reference's selection (a descending sort, cut at batch_size) and one
gather of the chosen children.  Inputs must be CUDA
tensors; there is no CPU path.
"""

from __future__ import annotations

import itertools

import torch

from . import _native
from .bitspack import pack_int, unpack_int

__all__ = ["MLP", "WaveFunctionElectronUpDown"]


class _BiasOnly(torch.nn.Module):
    """The first layer of the site-0 network: no inputs, so its output is its bias."""

    def __init__(self, dim_out: int) -> None:
        super().__init__()
        self.bias = torch.nn.Parameter(torch.zeros([dim_out]))

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        return self.bias.view(1, -1).expand(x.shape[0], -1)


class MLP(torch.nn.Module):
    """Linear layers dim_input -> hidden_size... -> dim_output with SiLU between them (qmb/mlp.py:38-57)."""

    def __init__(self, dim_input: int, dim_output: int, hidden_size: tuple[int, ...]) -> None:
        super().__init__()
        self.dim_input, self.dim_output, self.hidden_size = dim_input, dim_output, tuple(hidden_size)
        widths = [dim_input, *hidden_size, dim_output]
        layers: list[torch.nn.Module] = []
        for k, (a, b) in enumerate(itertools.pairwise(widths)):
            if k:
                layers.append(torch.nn.SiLU())
            layers.append(_BiasOnly(b) if a == 0 else torch.nn.Linear(a, b))
        self.model = torch.nn.Sequential(*layers)

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        return self.model(x)


def _stream(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class _LogAmplitude(torch.autograd.Function):
    """Sum over sites of each row's normalised, masked log amplitude; backward in CUDA as well."""

    @staticmethod
    def forward(ctx, deltas: torch.Tensor, occ: torch.Tensor, sites: int, up: int, down: int) -> torch.Tensor:
        rows = occ.shape[0]
        deltas = deltas.contiguous()
        total = torch.empty(rows, dtype=torch.float64, device=deltas.device)
        with torch.cuda.device(deltas.device):
            _native.call("qmbx_sampler_log_amplitude", rows, sites, up, down, deltas.data_ptr(), occ.data_ptr(),
                         total.data_ptr(), _stream(deltas.device))
        ctx.save_for_backward(deltas, occ)
        ctx.shape = (sites, up, down)
        return total

    @staticmethod
    def backward(ctx, grad: torch.Tensor):
        deltas, occ = ctx.saved_tensors
        sites, up, down = ctx.shape
        grad = grad.to(torch.float64).contiguous()
        out = torch.empty_like(deltas)
        with torch.cuda.device(deltas.device):
            _native.call("qmbx_sampler_log_amplitude_grad", occ.shape[0], sites, up, down, deltas.data_ptr(),
                         occ.data_ptr(), grad.data_ptr(), out.data_ptr(), _stream(deltas.device))
        return out, None, None, None, None


class WaveFunctionElectronUpDown(torch.nn.Module):
    """Autoregressive wave function conserving the up and down electron numbers (qmb/mlp.py:60-314)."""

    def __init__(self, *, double_sites: int, physical_dim: int, is_complex: bool, spin_up: int, spin_down: int,
                 hidden_size: tuple[int, ...], ordering: int | list[int]) -> None:
        super().__init__()
        if double_sites % 2 or physical_dim != 2 or not is_complex:
            raise ValueError("double_sites must be even, physical_dim 2 and is_complex True")
        self.double_sites = double_sites
        self.sites = double_sites // 2
        self.spin_up, self.spin_down = spin_up, spin_down
        self.hidden_size = tuple(hidden_size)
        # the network of site i sees the 2 i occupations before it and gives the
        # four log amplitudes of the site's (up, down) occupation
        self.amplitude = torch.nn.ModuleList([MLP(2 * i, 4, self.hidden_size) for i in range(self.sites)])
        self.phase = MLP(self.double_sites, 1, self.hidden_size)
        if isinstance(ordering, int):
            if ordering not in (+1, -1):
                raise ValueError("ordering must be +1, -1 or a list of sites")
            ordering = list(range(self.sites)) if ordering == 1 else list(reversed(range(self.sites)))
        order = torch.tensor(ordering, dtype=torch.int64)
        inverse = torch.empty_like(order)
        inverse[order] = torch.arange(self.sites)
        self.register_buffer("ordering", order)
        self.register_buffer("ordering_reversed", inverse)
        self.dummy_param = torch.nn.Parameter(torch.empty(0))

    # -- psi -----------------------------------------------------------------------

    def _occupations(self, configs: torch.Tensor) -> torch.Tensor:
        """[rows, sites, 2] uint8 occupations in sampling order."""
        bits = unpack_int(configs, size=1, last_dim=self.double_sites).view(configs.shape[0], self.sites, 2)
        return torch.index_select(bits, 1, self.ordering_reversed)

    def forward(self, configs: torch.Tensor) -> torch.Tensor:
        """psi (complex128) of packed configurations; differentiable in the parameters."""
        if not configs.is_cuda:
            raise RuntimeError("this sampler runs on CUDA devices only")
        rows = configs.shape[0]
        x = self._occupations(configs)
        dtype = self.dummy_param.dtype
        xf = x.to(dtype).reshape(rows, self.double_sites)
        # site i's network on the first 2 i inputs: [sites, rows, 4]
        deltas = torch.stack([net(xf[:, :2 * i]) for i, net in enumerate(self.amplitude)]) if self.sites else \
            torch.empty((0, rows, 4), dtype=dtype, device=configs.device)
        occ = (2 * x[..., 0] + x[..., 1]).to(torch.uint8).contiguous()
        total = _LogAmplitude.apply(deltas.to(torch.float32), occ, self.sites, self.spin_up, self.spin_down)
        phase = self.phase(xf).view(rows)
        return torch.view_as_complex(torch.stack([total, phase.double()], dim=-1)).exp()

    # -- sampling --------------------------------------------------------------------

    @torch.no_grad()
    def generate_unique(self, batch_size: int, block_num: int = 1,
                        uniforms=None) -> tuple[torch.Tensor, torch.Tensor, None, None]:
        """Up to batch_size distinct configurations drawn without replacement, and their psi.

        ``uniforms`` (optional: one [rows, 4] tensor per site in sampling
        order, or a function (site, rows) -> such a tensor) replaces the
        Gumbel noise draws, to replay a run; ``block_num``
        splits every network evaluation into that many row blocks, as the
        reference does to bound memory.
        """
        device = self.dummy_param.device
        if device.type != "cuda":
            raise RuntimeError("this sampler runs on CUDA devices only")
        dtype = self.dummy_param.dtype
        sites, up, down = self.sites, self.spin_up, self.spin_down
        stream = _stream(device)
        n = 1
        occ = torch.zeros((1, sites), dtype=torch.uint8, device=device)
        xf = torch.zeros((1, 2 * sites), dtype=dtype, device=device)
        counts = torch.zeros((1, 2), dtype=torch.int32, device=device)
        lp = torch.zeros(1, dtype=torch.float32, device=device)
        gp = torch.zeros(1, dtype=torch.float32, device=device)
        la = torch.zeros(1, dtype=torch.float64, device=device)  # log amplitude so far (the forward's sum)
        bad = torch.zeros(1, dtype=torch.int32, device=device)  # NaN / +inf values of a site (see the kernels)
        with torch.cuda.device(device):
            for i, net in enumerate(self.amplitude):
                inputs = xf[:, :2 * i]
                blocks = [net(part) for part in torch.tensor_split(inputs, max(1, min(block_num, n)))]
                delta = torch.cat(blocks).to(torch.float32).contiguous()
                if uniforms is None:
                    u = torch.rand((n, 4), dtype=torch.float32, device=device)
                else:
                    u = uniforms(i, n) if callable(uniforms) else uniforms[i]
                u = u.to(device=device, dtype=torch.float32)[:n]
                if u.shape[0] < n:
                    # a replay gives the reference's rows only; the rows carried past them have no
                    # children whatever they draw
                    u = torch.cat([u, torch.full((n - u.shape[0], 4), 0.5, dtype=torch.float32, device=device)])
                u = u.contiguous()
                l_all = torch.empty(4 * n, dtype=torch.float32, device=device)
                t_all = torch.empty(4 * n, dtype=torch.float32, device=device)
                a_all = torch.empty(4 * n, dtype=torch.float64, device=device)
                bad.zero_()
                _native.call("qmbx_sampler_site", n, i, sites, up, down, delta.data_ptr(), counts.data_ptr(),
                             lp.data_ptr(), gp.data_ptr(), u.data_ptr(), l_all.data_ptr(), t_all.data_ptr(),
                             la.data_ptr(), a_all.data_ptr(), bad.data_ptr(), stream)
                # the batch_size largest conditioned Gumbel values, largest first -- the
                # reference's own selection (argsort).  The reference then drops the values
                # that are not finite; here those rows are carried along (the take kernel
                # marks them, the site kernel gives them no children) and dropped once at the
                # end, so the row count stays known on the host and the loop never waits for
                # the device.  NaN and +inf, which the reference's sort puts first, are sorted
                # after the finite values here, so the kept rows come first, as there
                index = torch.argsort(t_all, descending=True)[:batch_size].contiguous()
                m = index.shape[0]
                occ_n = torch.empty((m, sites), dtype=torch.uint8, device=device)
                xf_n = torch.zeros((m, 2 * sites), dtype=torch.float32, device=device)
                counts_n = torch.empty((m, 2), dtype=torch.int32, device=device)
                lp_n = torch.empty(m, dtype=torch.float32, device=device)
                gp_n = torch.empty(m, dtype=torch.float32, device=device)
                la_n = torch.empty(m, dtype=torch.float64, device=device)
                _native.call("qmbx_sampler_take", m, n, i, sites, index.data_ptr(), occ.data_ptr(), counts.data_ptr(),
                             l_all.data_ptr(), t_all.data_ptr(), occ_n.data_ptr(), xf_n.data_ptr(), counts_n.data_ptr(),
                             lp_n.data_ptr(), gp_n.data_ptr(), a_all.data_ptr(), la_n.data_ptr(), batch_size,
                             bad.data_ptr(), stream)
                occ, counts, lp, gp, la, n = occ_n, counts_n, lp_n, gp_n, la_n, m
                xf = xf_n.to(dtype)
        # the rows the reference keeps: those whose value is finite (in the same order)
        keep = torch.isfinite(gp)
        occ, xf, la = occ[keep], xf[keep], la[keep]
        n = occ.shape[0]
        # back to the site order of the configurations, then packed
        bits = torch.stack([occ >> 1, occ & 1], dim=-1)
        bits = torch.index_select(bits, 1, self.ordering).reshape(n, self.double_sites)
        configs = pack_int(bits, size=1)
        # psi = exp(log amplitude + i phase): the log amplitudes were summed site by site while
        # sampling (the forward's own sum of the same normalised terms), so only the phase
        # network runs here, on the sampled rows in sampling order
        if n:
            phase = torch.cat([self.phase(part).view(-1) for part in torch.tensor_split(xf, max(1, min(block_num, n)))])
            psi = torch.view_as_complex(torch.stack([la, phase.double()], dim=-1)).exp()
        else:
            psi = torch.empty(0, dtype=torch.complex128, device=device)
        return configs, psi, None, None
