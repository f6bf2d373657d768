"""The reference's own CUDA apply_within, run from its cubin — MEASUREMENT INFRASTRUCTURE ONLY.

``oracle/ref_build.py cuda`` compiles qmb/_hamiltonian_cuda.cu (the
reference's sources, unmodified) into ``oracle/_ref/ref_cuda_<nq>_<pc>.cubin``.
This module loads that cubin through the CUDA driver API (ctypes on
libcuda) into torch's context and replays the host side of the reference's
``apply_within_interface`` (qmb/_hamiltonian_cuda.cu:171-274):

1. sort a copy of configs_j lexicographically, keeping the permutation
   (the reference: ``thrust::sort_by_key`` with its byte comparator; here a
   stable byte-wise LSD sort with torch, the only step not taken from the
   reference's own code);
2. launch ``apply_within_kernel_interface<4, nq, pc>`` on a grid of
   (terms, ceil(N_i / 512)) blocks of (1, 512) threads, one thread per
   (term, source) pair, FP64 atomics into the sorted result;
3. scatter the result back to configs_j's order (``index_put_``).

bench.py times it as the FP64 GPU path of the reference.  Nothing in the
product imports this module.
"""

from __future__ import annotations

import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def cubin_path(nq: int, pc: int) -> str:
    return os.path.join(OUT, f"ref_cuda_{nq}_{pc}.cubin")


def available(nq: int, pc: int) -> bool:
    return os.path.exists(cubin_path(nq, pc)) and os.path.exists(cubin_path(nq, pc)[:-6] + ".json")


def daggered(site: np.ndarray, kind: np.ndarray, coef: np.ndarray):
    """The table of H^dagger: slots reversed, create <-> annihilate, coefficients conjugated."""
    site = np.ascontiguousarray(site[:, ::-1])
    kind = np.ascontiguousarray(kind[:, ::-1]).copy()
    live = kind != 2
    kind[live] = 1 - kind[live]
    coef = coef.copy()
    coef[:, 1] = -coef[:, 1]
    return site, kind, np.ascontiguousarray(coef)


class ReferenceCuda:
    """apply_within of the reference's CUDA kernel for one (n_qubytes, particle_cut)."""

    def __init__(self, nq: int, pc: int, device):
        import torch

        self.torch = torch
        self.nq, self.pc, self.device = nq, pc, device
        with open(cubin_path(nq, pc)[:-6] + ".json") as f:
            meta = json.load(f)
        name = meta["kernels"]["apply_within_kernel_interface"]
        torch.zeros(1, device=device)  # torch's primary context is current from here on
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                                    ctypes.c_void_p, ctypes.c_void_p]
        self.module = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.module), cubin_path(nq, pc).encode()), "cuModuleLoad")
        self.fn = ctypes.c_void_p()
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(self.fn), self.module, name.encode()),
                    "cuModuleGetFunction")

    @staticmethod
    def _check(res: int, what: str) -> None:
        if res != 0:
            raise RuntimeError(f"{what} failed with CUresult {res}")

    def table(self, site: np.ndarray, kind: np.ndarray, coef: np.ndarray):
        """Device copies of a term table after checking it against the kernel's indexing."""
        torch = self.torch
        site = np.ascontiguousarray(site, dtype=np.int16)
        kind = np.ascontiguousarray(kind, dtype=np.uint8)
        live = kind != 2
        if not np.all(np.isin(kind, (0, 1, 2))) or (live.any() and (site[live].min() < 0 or
                                                                     site[live].max() >= 8 * self.nq)):
            raise ValueError("term table out of the kernel's range")
        return (torch.from_numpy(site).to(self.device), torch.from_numpy(kind).to(self.device),
                torch.from_numpy(np.ascontiguousarray(coef, dtype=np.float64)).to(self.device))

    def sort_rows(self, rows):
        """Stable lexicographic order of uint8 rows (byte 0 most significant): LSD over the bytes."""
        torch = self.torch
        perm = torch.arange(rows.shape[0], device=rows.device)
        for b in range(rows.shape[1] - 1, -1, -1):
            key = rows[perm, b].to(torch.int32)
            order = torch.sort(key, stable=True).indices
            perm = perm[order]
        return perm

    def launch(self, table, configs, psi_f64, sorted_targets, out_sorted, stream) -> None:
        """The reference kernel over every (term, source) pair; out_sorted (zeroed) receives the sums."""
        site, kind, coef = table
        n_terms, batch, result = site.shape[0], configs.shape[0], sorted_targets.shape[0]
        if batch == 0 or n_terms == 0:
            return
        assert configs.shape[1] == self.nq and sorted_targets.shape[1] == self.nq
        assert psi_f64.shape == (batch, 2) and out_sorted.shape == (result, 2)
        grid_y = (batch + 511) // 512
        assert n_terms < 2**31 and grid_y < 65536
        holders = [ctypes.c_int64(n_terms), ctypes.c_int64(batch), ctypes.c_int64(result)]
        holders += [ctypes.c_void_p(t.data_ptr()) for t in (site, kind, coef, configs, psi_f64, sorted_targets,
                                                             out_sorted)]
        params = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.byref(h), ctypes.c_void_p) for h in holders])
        self._check(self.cu.cuLaunchKernel(self.fn, n_terms, grid_y, 1, 1, 512, 1, 0, ctypes.c_void_p(stream),
                                           params, None), "cuLaunchKernel")

    def apply_within(self, table, configs_i, psi_i, configs_j):
        """The reference's apply_within: psi_i complex128 on configs_i -> complex128 on configs_j."""
        torch = self.torch
        stream = torch.cuda.current_stream(self.device).cuda_stream
        perm = self.sort_rows(configs_j)
        sorted_j = configs_j[perm].contiguous()
        out_sorted = torch.zeros((configs_j.shape[0], 2), dtype=torch.float64, device=self.device)
        self.launch(table, configs_i.contiguous(), torch.view_as_real(psi_i).contiguous(), sorted_j, out_sorted, stream)
        out = torch.zeros_like(out_sorted)
        out[perm] = out_sorted
        return torch.view_as_complex(out)
