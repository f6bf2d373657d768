"""The allocation-free apply_within entry point (qmbx_apply_within_static).

It serves callers that cannot allocate device memory (a host program whose
memory pool owns the whole GPU, a latency-critical loop that cannot afford
cudaMalloc's implicit synchronisation, a plain C caller without an
allocator): its scratch is a fixed array inside the library.  These tests call
it through the C ABI twice in a row, on different inputs, and compare each
result with the workspace-taking qmbx_apply_within, and check that inputs too
large for the fixed scratch are refused with an error instead of running.
Collected last so that a failure here comes after every other test has run.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from conftest import golden
from qmb_gb300 import Hamiltonian, _native

pytestmark = pytest.mark.gpu

RTOL_F64 = 1e-12


def _abs_scale(g, configs_i, psi_i, configs_j):
    import oracle

    mag = np.zeros_like(g["coef"])
    mag[:, 0] = np.hypot(g["coef"][:, 0], g["coef"][:, 1])
    return np.abs(oracle.apply_within(g["site"], g["kind"], mag, configs_i, np.abs(psi_i).astype(np.complex128),
                                      configs_j, 2))


def _with_workspace(table, ci, psi, cj, device, same=0):
    lib = _native.library()
    need = ctypes.c_uint64()
    _native.check(lib.qmbx_apply_within_workspace(table.h, ci.shape[0], cj.shape[0], ctypes.byref(need)))
    ws = torch.empty(max(need.value, 256), dtype=torch.uint8, device=device)
    out = torch.empty(cj.shape[0], dtype=torch.complex128, device=device)
    _native.check(lib.qmbx_apply_within(table.h, table.d, ci.data_ptr(), psi.data_ptr(), ci.shape[0], cj.data_ptr(),
                                        cj.shape[0], same, out.data_ptr(), ws.data_ptr(), ws.numel(),
                                        torch.cuda.current_stream(device).cuda_stream))
    return out


def _static(table, ci, psi, cj, device, same=0):
    out = torch.empty(cj.shape[0], dtype=torch.complex128, device=device)
    _native.check(_native.library().qmbx_apply_within_static(table.h, table.d, ci.data_ptr(), psi.data_ptr(),
                                                             ci.shape[0], cj.data_ptr(), cj.shape[0], same,
                                                             out.data_ptr(),
                                                             torch.cuda.current_stream(device).cuda_stream))
    return out


def test_static_scratch_matches_workspace_entry_point_twice(cuda_device):
    cases = [golden("ab_initio_10_complex"), golden("random_terms_fermi")]
    for g in cases:
        ham = Hamiltonian((torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"])),
                          kind="fermi")
        with torch.cuda.device(cuda_device):
            table = ham._table(cuda_device, g["configs_i"].shape[1])
            ci = torch.from_numpy(g["configs_i"]).to(cuda_device)
            cj = torch.from_numpy(g["configs_j"]).to(cuda_device)
            rng = np.random.default_rng(17)
            # two calls in a row on different amplitudes and row sets: the second
            # call must not see anything the first one left in the shared scratch
            inputs = [(ci, g["psi_i"], cj, g["configs_i"], g["configs_j"])]
            half = g["configs_j"][::2].copy()
            psi_b = (rng.standard_normal(half.shape[0]) + 1j * rng.standard_normal(half.shape[0]))
            inputs.append((torch.from_numpy(half).to(cuda_device), psi_b, ci, half, g["configs_i"]))
            for rows_i, psi_np, rows_j, np_i, np_j in inputs:
                psi = torch.from_numpy(np.ascontiguousarray(psi_np)).to(cuda_device)
                got = _static(table, rows_i, psi, rows_j, cuda_device).cpu().numpy()
                want = _with_workspace(table, rows_i, psi, rows_j, cuda_device).cpu().numpy()
                scale = _abs_scale(g, np_i, psi_np, np_j)
                assert np.all(np.abs(got - want) <= RTOL_F64 * scale + 1e-300)


def test_static_scratch_refuses_oversized_inputs(cuda_device):
    g = golden("ab_initio_6")
    ham = Hamiltonian((torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"])),
                      kind="fermi")
    lib = _native.library()
    with torch.cuda.device(cuda_device):
        table = ham._table(cuda_device, g["configs_i"].shape[1])
        big = 4_000_000
        need = ctypes.c_uint64()
        _native.check(lib.qmbx_apply_within_workspace(table.h, big, big, ctypes.byref(need)))
        assert need.value > (32 << 20)
        rows = torch.zeros((big, g["configs_i"].shape[1]), dtype=torch.uint8, device=cuda_device)
        psi = torch.zeros(big, dtype=torch.complex128, device=cuda_device)
        out = torch.empty(big, dtype=torch.complex128, device=cuda_device)
        status = lib.qmbx_apply_within_static(table.h, table.d, rows.data_ptr(), psi.data_ptr(), big, rows.data_ptr(),
                                              big, 0, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert status == _native.QMBX_ERR_ARGUMENT
        assert b"static scratch" in lib.qmbx_last_error()
        # the library is still usable afterwards
        small = torch.from_numpy(g["configs_i"][:8]).to(cuda_device)
        p = torch.from_numpy(g["psi_i"][:8]).to(cuda_device)
        got = _static(table, small, p, small, cuda_device).cpu().numpy()
        want = _with_workspace(table, small, p, small, cuda_device).cpu().numpy()
        assert np.allclose(got, want, rtol=0, atol=1e-12 * (1 + np.abs(want).max()))


def test_static_scratch_same_configs_after_a_larger_call(cuda_device):
    # same_configs = 1 builds one row set in the shared scratch; run it right
    # after a larger call (two sets of 20,000 random rows) so that anything
    # that call left behind would show
    g = golden("random_terms_fermi")
    ham = Hamiltonian((torch.from_numpy(g["site"]), torch.from_numpy(g["kind"]), torch.from_numpy(g["coef"])),
                      kind="fermi")
    nq = g["configs_i"].shape[1]
    rng = np.random.default_rng(5)
    with torch.cuda.device(cuda_device):
        table = ham._table(cuda_device, nq)
        big_i = torch.from_numpy(rng.integers(0, 256, size=(20000, nq), dtype=np.uint8)).to(cuda_device)
        big_j = torch.from_numpy(rng.integers(0, 256, size=(20000, nq), dtype=np.uint8)).to(cuda_device)
        big_psi = torch.randn(20000, dtype=torch.complex128, device=cuda_device)
        _static(table, big_i, big_psi, big_j, cuda_device)
        rows = np.unique(np.concatenate([g["configs_i"], g["configs_j"]]), axis=0)
        psi_np = rng.standard_normal(rows.shape[0]) + 1j * rng.standard_normal(rows.shape[0])
        r = torch.from_numpy(rows).to(cuda_device)
        psi = torch.from_numpy(psi_np).to(cuda_device)
        got = _static(table, r, psi, r, cuda_device, same=1).cpu().numpy()
        want = _with_workspace(table, r, psi, r, cuda_device, same=1).cpu().numpy()
        scale = _abs_scale(g, rows, psi_np, rows)
        assert np.count_nonzero(want) > 100
        assert np.all(np.abs(got - want) <= RTOL_F64 * scale + 1e-300)
