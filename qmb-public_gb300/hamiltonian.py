"""Drop-in replacement for qmb.hamiltonian.Hamiltonian on GB300 GPUs.

Same constructor and methods as qmb/hamiltonian.py:12-206:

* ``Hamiltonian(dict or (site, kind, coef), *, kind="fermi" | "bose2")``
* ``apply_within(configs_i, psi_i, configs_j)``
* ``find_relative(configs_i, psi_i, count_selected, configs_exclude=None)``
* ``diagonal_term(configs)``
* ``single_relative(configs)``

and the public ``site``, ``kind``, ``coef`` tensors.  Every method runs the
CUDA kernels of libqmbx.so on the configurations' device through the C ABI
(include/qmbx.h); tensors on the CPU are rejected (there is no CPU path).

Additions over the reference: complex64 amplitudes select the FP32 path with
compensated accumulation; ``apply_within`` is differentiable in ``psi_i``
(its backward is the adjoint kernel); ``apply_within_adjoint`` exposes that
kernel directly; ``matrix`` materialises H on a fixed basis (for iterative
eigensolvers); ``pt2`` runs the Epstein-Nesbet step of qmb/pert.py in one
call; ``table_cache=`` (or QMBX_TABLE_CACHE) caches compiled term tables on
disk.
"""

from __future__ import annotations

import ctypes
import hashlib
import os
import struct

import numpy as np
import torch

from . import _native
from .terms import prepare, sort_terms

__all__ = ["Hamiltonian", "HamiltonianMatrix"]


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _stream(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _workspace(nbytes: int, device: torch.device) -> torch.Tensor:
    ws = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
    if ws.data_ptr() % 256:
        raise RuntimeError("workspace allocation is not 256-byte aligned")
    return ws


def _pinned(nbytes: int) -> torch.Tensor:
    """A host buffer for a table blob: page-locked where a GPU is present, so the device copy is one DMA."""
    buf = torch.empty(nbytes, dtype=torch.uint8)
    return buf.pin_memory() if torch.cuda.is_available() else buf


def compile_table(site: torch.Tensor, kind: torch.Tensor, coef: torch.Tensor, n_qubytes: int, particle_cut: int,
                  cache_dir: str | os.PathLike | None = None) -> torch.Tensor:
    """The compiled term table (host blob) for these terms, read from / written to ``cache_dir`` when given.

    Like qmb/fcidump.py:143-169, which caches the raw (site, kind, coef) table
    under a checksum of its source, the compiled blob is cached under a
    SHA-256 of the term tensors, the row width, the particle kind and the
    library's ABI version; a cached file is used only when qmbx_table_check
    accepts it (same table format, whole blob), otherwise it is rebuilt.
    """
    lib = _native.library()
    site = site.detach().to("cpu", torch.int16).contiguous()
    kind = kind.detach().to("cpu", torch.uint8).contiguous()
    coef = coef.detach().to("cpu", torch.float64).contiguous()
    if site.dim() != 2 or site.shape[1] != 4 or kind.shape != site.shape or coef.shape != (site.shape[0], 2):
        raise RuntimeError("site, kind and coef must have shapes [T, 4], [T, 4] and [T, 2]")
    path = None
    if cache_dir is not None:
        h = hashlib.sha256()
        for t in (site, kind, coef):
            h.update(t.numpy().tobytes())
        h.update(struct.pack("<iii", n_qubytes, particle_cut, lib.qmbx_version()))
        path = os.path.join(os.fspath(cache_dir), f"{h.hexdigest()}.qmbx")
        if os.path.exists(path):
            data = np.fromfile(path, dtype=np.uint8)
            host = _pinned(data.size)
            host.numpy()[:] = data
            if lib.qmbx_table_check(host.data_ptr(), host.numel()) == _native.QMBX_OK:
                return host
    nbytes = ctypes.c_uint64(0)
    _native.check(lib.qmbx_table_bytes(site.data_ptr(), kind.data_ptr(), site.shape[0], n_qubytes, particle_cut,
                                       ctypes.byref(nbytes)))
    host = _pinned(nbytes.value)
    _native.check(lib.qmbx_table_build(site.data_ptr(), kind.data_ptr(), coef.data_ptr(), site.shape[0], n_qubytes,
                                       particle_cut, host.data_ptr(), nbytes.value))
    if path is not None:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = f"{path}.{os.getpid()}.tmp"
        host.numpy().tofile(tmp)
        os.replace(tmp, path)
    return host


class _Table:
    """A compiled term table: host blob (header read by the host) and its device copy."""

    def __init__(self, site: torch.Tensor, kind: torch.Tensor, coef: torch.Tensor, n_qubytes: int, particle_cut: int,
                 device: torch.device, cache_dir: str | os.PathLike | None = None):
        lib = _native.library()
        self.host = compile_table(site, kind, coef, n_qubytes, particle_cut, cache_dir)
        nbytes = self.host.numel()
        self.dev = torch.empty(nbytes, dtype=torch.uint8, device=device)
        if self.dev.data_ptr() % 256:
            raise RuntimeError("table allocation is not 256-byte aligned")
        self.dev.copy_(self.host, non_blocking=False)
        counts = (ctypes.c_int64 * 6)()
        _native.check(lib.qmbx_table_counts(self.host.data_ptr(), counts))
        self.n_terms, self.n_live, self.n_diag, self.n_qubytes, self.particle_cut, self.n_words = list(counts)
        self._hermitian: bool | None = None

    @property
    def hermitian(self) -> bool:
        """Whether the compiled operator equals its adjoint (checked once, on the host)."""
        if self._hermitian is None:
            flag = ctypes.c_int32()
            _native.check(_native.library().qmbx_table_hermitian(self.host.data_ptr(), ctypes.byref(flag)))
            self._hermitian = bool(flag.value)
        return self._hermitian

    def use_on(self, stream: torch.cuda.Stream) -> None:
        """Mark the device blob as used by work on `stream`, so that torch's caching allocator does not
        hand its memory out again (after the table is dropped) before that work has finished."""
        self.dev.record_stream(stream)

    @property
    def h(self) -> int:
        return self.host.data_ptr()

    @property
    def d(self) -> int:
        return self.dev.data_ptr()


class Hamiltonian:
    """Second-quantized Hamiltonian over bit-packed configurations (see module docstring)."""

    def __init__(self, hamiltonian: dict | tuple[torch.Tensor, torch.Tensor, torch.Tensor], *, kind: str,
                 table_cache: str | os.PathLike | None = None) -> None:
        self.site: torch.Tensor
        self.kind: torch.Tensor
        self.coef: torch.Tensor
        if isinstance(hamiltonian, dict):
            self.site, self.kind, self.coef = sort_terms(*prepare(hamiltonian))
        else:
            self.site, self.kind, self.coef = hamiltonian
        self.particle_cut: int
        match kind:
            case "fermi":
                self.particle_cut = 1
            case "bose2":
                self.particle_cut = 2
            case _:
                raise ValueError(f"Unknown kind: {kind}")
        self._tables: dict = {}
        self._log_caps: dict = {}
        # where compiled term tables are cached across processes (compile_table); QMBX_TABLE_CACHE by default
        self.table_cache = table_cache if table_cache is not None else os.environ.get("QMBX_TABLE_CACHE")

    # -- plumbing -----------------------------------------------------------

    def _prepare_data(self, device: torch.device) -> None:
        """Move the public term tensors to ``device`` as the reference does (qmb/hamiltonian.py:99-102)."""
        self.site = self.site.to(device=device).contiguous()
        self.kind = self.kind.to(device=device).contiguous()
        self.coef = self.coef.to(device=device).contiguous()

    def _table(self, device: torch.device, n_qubytes: int) -> _Table:
        if device.type != "cuda":
            raise RuntimeError("this engine runs on CUDA devices only; move the configurations to a GPU")
        self._prepare_data(device)
        key = (device.index, n_qubytes, self.site.data_ptr(), self.kind.data_ptr(), self.coef.data_ptr(),
               self.site._version, self.kind._version, self.coef._version)
        table = self._tables.get(key)
        if table is None:
            with torch.cuda.device(device):
                table = _Table(self.site, self.kind, self.coef, n_qubytes, self.particle_cut, device, self.table_cache)
            # tables of this device compiled from other term tensors (or older
            # versions of them) are stale; those for other row widths are kept
            self._tables = {k: v for k, v in self._tables.items() if k[0] != device.index or k[2:] == key[2:]}
            self._tables[key] = table
        # every caller launches work that reads the table on the current stream
        table.use_on(torch.cuda.current_stream(device))
        return table

    @staticmethod
    def _configs(configs: torch.Tensor, name: str, device: torch.device | None = None) -> torch.Tensor:
        if configs.dtype != torch.uint8:
            raise RuntimeError(f"{name} must be uint8.")
        if configs.dim() != 2:
            raise RuntimeError(f"{name} must be 2D.")
        if device is not None and configs.device != device:
            raise RuntimeError(f"{name} must be on the same device as others.")
        return configs.contiguous()

    @staticmethod
    def _amplitudes(psi: torch.Tensor, n: int, name: str, device: torch.device) -> torch.Tensor:
        if psi.dtype not in (torch.complex128, torch.complex64):
            raise RuntimeError(f"{name} must be complex128 (or complex64 for the FP32 path).")
        if psi.dim() != 1 or psi.shape[0] != n:
            raise RuntimeError(f"{name} must have shape [{n}].")
        if psi.device != device:
            raise RuntimeError(f"{name} must be on the same device as others.")
        return psi.contiguous()

    # -- apply_within ---------------------------------------------------------

    # hit records a logged forward call may keep (16 bytes each): a first guess, then what the
    # last call on rows of the same shape needed
    _LOG_FIRST_GUESS = 1 << 22
    # differentiable apply_within records the forward walk's hits for its backward; False: the
    # backward walks the terms again with the adjoint kernel
    hit_log = True

    def _log_capacity(self, n_i: int, n_j: int, device: torch.device) -> int:
        """Hit records to reserve for a logged forward on rows of this shape: a first guess, then 1.25x
        the count of the last call of this shape whose count has arrived (read without waiting)."""
        key = (device.index, n_i, n_j)
        state = self._log_caps.get(key)
        if state is None:
            free, _ = torch.cuda.mem_get_info(device)
            state = self._log_caps[key] = {"cap": int(min(self._LOG_FIRST_GUESS, free // 8 // 16)), "pending": None}
        pending = state["pending"]
        if pending is not None and pending[1].query():
            count = int(pending[0][0])
            state["pending"] = None
            if count > state["cap"] or count < state["cap"] // 4:
                state["cap"] = int(count * 1.25) + 1024
        return state["cap"]

    def _apply(self, configs_i: torch.Tensor, psi_i: torch.Tensor, configs_j: torch.Tensor, *, adjoint: bool,
               out_dtype: torch.dtype | None = None, include_diagonal: bool = True, log: bool = False):
        """Forward (psi_i on configs_i -> configs_j) or adjoint (g on configs_j -> configs_i) application.

        With ``log`` (forward only) the walk also records its hits and the
        result is ``(out, record)``; ``_adjoint_from_log(record, g)`` then gives
        the adjoint product on the same rows without walking the terms again.
        """
        device = configs_i.device
        configs_i = self._configs(configs_i, "configs_i")
        configs_j = self._configs(configs_j, "configs_j", device)
        nq = configs_i.shape[1]
        if configs_j.shape[1] != nq:
            raise RuntimeError("configs_i and configs_j must have the same number of qubytes.")
        n_i, n_j = configs_i.shape[0], configs_j.shape[0]
        n_in, n_out = (n_j, n_i) if adjoint else (n_i, n_j)
        psi = self._amplitudes(psi_i, n_in, "psi", device)
        table = self._table(device, nq)
        same = int(configs_i.data_ptr() == configs_j.data_ptr() and n_i == n_j)
        lib = _native.library()
        with torch.cuda.device(device):
            ws = None
            if not (log and not adjoint):
                need = ctypes.c_uint64(0)
                _native.check(lib.qmbx_apply_within_workspace(table.h, n_i, n_j, ctypes.byref(need)))
                ws = _workspace(need.value, device)
            stream = _stream(device)
            record = None
            log_args = ()
            if log and not adjoint:
                # the log holds the hit records and the forward's own workspace (its row sets are the
                # adjoint's), so the forward takes no separate workspace
                cap = self._log_capacity(n_i, n_j, device)
                nbytes = ctypes.c_uint64(0)
                _native.check(lib.qmbx_hitlog_bytes(table.h, n_i, n_j, same, cap, ctypes.byref(nbytes)))
                buf = _workspace(nbytes.value, device)
                record = _HitRecord(table, buf, cap, n_i, n_j, same, psi.dtype, include_diagonal)
                log_args = (buf.data_ptr(), buf.numel(), cap)
            if psi.dtype == torch.complex128:
                out = torch.empty(n_out, dtype=torch.complex128, device=device)
                if adjoint:
                    _native.call("qmbx_apply_within_adjoint", table.h, table.d, configs_i.data_ptr(), n_i,
                                 configs_j.data_ptr(), psi.data_ptr(), n_j, same, out.data_ptr(), ws.data_ptr(),
                                 ws.numel(), stream)
                elif record:
                    _native.call("qmbx_apply_within_logged", table.h, table.d, configs_i.data_ptr(), psi.data_ptr(),
                                 n_i, configs_j.data_ptr(), n_j, same, out.data_ptr(), *log_args, stream)
                else:
                    _native.call("qmbx_apply_within", table.h, table.d, configs_i.data_ptr(), psi.data_ptr(), n_i,
                                 configs_j.data_ptr(), n_j, same, out.data_ptr(), ws.data_ptr(), ws.numel(), stream)
                out = out if out_dtype in (None, torch.complex128) else out.to(out_dtype)
                return (out, record) if log and not adjoint else out
            want64 = out_dtype == torch.complex128
            out = torch.empty(n_out, dtype=torch.complex128 if want64 else torch.complex64, device=device)
            o64, o32 = (out.data_ptr(), None) if want64 else (None, out.data_ptr())
            if adjoint:
                _native.call("qmbx_apply_within_adjoint_f32c", table.h, table.d, configs_i.data_ptr(), n_i,
                             configs_j.data_ptr(), psi.data_ptr(), n_j, same, int(include_diagonal), o64, o32,
                             ws.data_ptr(), ws.numel(), stream)
            elif record:
                _native.call("qmbx_apply_within_f32c_logged", table.h, table.d, configs_i.data_ptr(), psi.data_ptr(),
                             n_i, configs_j.data_ptr(), n_j, same, int(include_diagonal), o64, o32, *log_args, stream)
            else:
                _native.call("qmbx_apply_within_f32c", table.h, table.d, configs_i.data_ptr(), psi.data_ptr(), n_i,
                             configs_j.data_ptr(), n_j, same, int(include_diagonal), o64, o32, ws.data_ptr(),
                             ws.numel(), stream)
            return (out, record) if log and not adjoint else out

    def _adjoint_from_log(self, record: "_HitRecord", g: torch.Tensor,
                          out_dtype: torch.dtype | None = None) -> torch.Tensor:
        """The adjoint product of a logged forward call for g on its output rows.

        Nothing waits for the device: the library replays the record, or walks the adjoint when the
        forward found more hits than the record holds.  The hit count is copied back without
        waiting and sizes the next log of this shape."""
        device = record.buf.device
        g = g.to(record.dtype).contiguous()
        if g.shape != (record.n_j,):
            raise RuntimeError(f"g must have shape [{record.n_j}].")
        table = record.table
        with torch.cuda.device(device):
            stream = _stream(device)
            if record.dtype == torch.complex128:
                out = torch.empty(record.n_i, dtype=torch.complex128, device=device)
                _native.call("qmbx_apply_within_adjoint_logged", table.h, table.d, record.buf.data_ptr(),
                             record.buf.numel(), record.cap, record.n_i, record.n_j, record.same, g.data_ptr(),
                             out.data_ptr(), stream)
            else:
                want64 = out_dtype == torch.complex128
                out = torch.empty(record.n_i, dtype=torch.complex128 if want64 else torch.complex64, device=device)
                o64, o32 = (out.data_ptr(), None) if want64 else (None, out.data_ptr())
                _native.call("qmbx_apply_within_adjoint_f32c_logged", table.h, table.d, record.buf.data_ptr(),
                             record.buf.numel(), record.cap, record.n_i, record.n_j, record.same,
                             int(record.include_diagonal), g.data_ptr(), o64, o32, stream)
            count = torch.empty(1, dtype=torch.int64, pin_memory=True)
            _native.call("qmbx_hitlog_count", record.buf.data_ptr(), count.data_ptr(), stream)
            done = torch.cuda.Event()
            done.record(torch.cuda.current_stream(device))
        record.count = (count, done)
        state = self._log_caps.get((device.index, record.n_i, record.n_j))
        if state is not None:
            state["pending"] = (count, done)
        return out

    def apply_within(self, configs_i: torch.Tensor, psi_i: torch.Tensor, configs_j: torch.Tensor) -> torch.Tensor:
        """H psi restricted to configs_j (qmb/hamiltonian.py:104-131); differentiable in psi_i.

        complex128 psi_i gives complex128 (FP64 path); complex64 psi_i gives
        complex64 computed with compensated FP32 accumulation.
        """
        if torch.is_grad_enabled() and psi_i.requires_grad:
            return _ApplyWithin.apply(self, configs_i, psi_i, configs_j, None)
        return self._apply(configs_i, psi_i, configs_j, adjoint=False)

    def apply_within_compensated(self, configs_i: torch.Tensor, psi_i: torch.Tensor, configs_j: torch.Tensor) -> torch.Tensor:
        """FP32-compensated H psi returned as complex128 (the compensated pair summed exactly); differentiable."""
        psi_i = psi_i.to(torch.complex64)
        if torch.is_grad_enabled() and psi_i.requires_grad:
            return _ApplyWithin.apply(self, configs_i, psi_i, configs_j, torch.complex128)
        return self._apply(configs_i, psi_i, configs_j, adjoint=False, out_dtype=torch.complex128)

    def apply_within_adjoint(self, configs_i: torch.Tensor, g_j: torch.Tensor, configs_j: torch.Tensor) -> torch.Tensor:
        """H^dagger applied to g_j on configs_j, restricted to configs_i (the adjoint of apply_within)."""
        return self._apply(configs_i, g_j, configs_j, adjoint=True)

    # -- sparse matrix on a fixed basis ------------------------------------------

    def matrix(self, configs: torch.Tensor, *, max_entries: int | None = None) -> HamiltonianMatrix | None:
        """H restricted to ``configs`` (distinct rows) as a ``HamiltonianMatrix``.

        Returns None when the matrix would have more than ``max_entries``
        entries (after the counting walk), so callers can fall back to
        ``apply_within``.
        """
        device = configs.device
        configs = self._configs(configs, "configs")
        n = configs.shape[0]
        table = self._table(device, configs.shape[1])
        lib = _native.library()
        need = ctypes.c_uint64(0)
        _native.check(lib.qmbx_matrix_workspace(table.h, n, ctypes.byref(need)))
        with torch.cuda.device(device):
            ws = _workspace(need.value, device)
            stream = _stream(device)
            row_ptr = torch.empty(n + 1, dtype=torch.int64, device=device)
            nnz = ctypes.c_int64(0)
            _native.call("qmbx_matrix_count", table.h, table.d, configs.data_ptr(), n, row_ptr.data_ptr(),
                         ctypes.byref(nnz), ws.data_ptr(), ws.numel(), stream)
            if max_entries is not None and nnz.value > max_entries:
                return None
            col = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=device)[:nnz.value]
            val = torch.empty(max(nnz.value, 1), dtype=torch.complex128, device=device)[:nnz.value]
            _native.call("qmbx_matrix_fill", table.h, table.d, configs.data_ptr(), n, row_ptr.data_ptr(),
                         col.data_ptr(), val.data_ptr(), ws.data_ptr(), ws.numel(), stream)
        return HamiltonianMatrix(row_ptr, col, val)

    # -- find_relative --------------------------------------------------------

    def find_relative(self, configs_i: torch.Tensor, psi_i: torch.Tensor, count_selected: int,
                      configs_exclude: torch.Tensor | None = None) -> torch.Tensor:
        """Heaviest connected configurations outside configs_exclude (qmb/hamiltonian.py:133-166)."""
        if configs_exclude is None:
            configs_exclude = configs_i
        device = configs_i.device
        configs_i = self._configs(configs_i, "configs_i")
        configs_exclude = self._configs(configs_exclude, "configs_exclude", device)
        nq = configs_i.shape[1]
        if configs_exclude.shape[1] != nq:
            raise RuntimeError("configs_exclude must have the same number of qubytes as configs_i.")
        psi = self._amplitudes(psi_i, configs_i.shape[0], "psi_i", device).to(torch.complex128)
        count_selected = int(count_selected)
        if count_selected < 0:
            raise RuntimeError("count_selected must not be negative.")
        table = self._table(device, nq)
        lib = _native.library()
        need = ctypes.c_uint64(0)
        _native.check(lib.qmbx_find_relative_workspace(table.h, configs_i.shape[0], count_selected,
                                                       configs_exclude.shape[0], ctypes.byref(need)))
        out = torch.empty((max(count_selected, 1), nq), dtype=torch.uint8, device=device)
        n_out = ctypes.c_int64(0)
        with torch.cuda.device(device):
            stream = _stream(device)
            for _ in range(4):
                ws = _workspace(need.value, device)
                want = ctypes.c_uint64(0)
                status = lib.qmbx_find_relative(table.h, table.d, configs_i.data_ptr(), psi.data_ptr(),
                                                configs_i.shape[0], count_selected, configs_exclude.data_ptr(),
                                                configs_exclude.shape[0], out.data_ptr(), ctypes.byref(n_out),
                                                ws.data_ptr(), ws.numel(), ctypes.byref(want), stream)
                if status == _native.QMBX_ERR_WORKSPACE and want.value > need.value:
                    need = want
                    del ws
                    continue
                _native.check(status)
                break
            else:
                raise RuntimeError("find_relative could not size its workspace")
        return out[:n_out.value]

    # -- PT2 step ----------------------------------------------------------------

    def pt2(self, configs: torch.Tensor, psi: torch.Tensor, count_selected: int) -> tuple[float, float, int]:
        """(E0, E2, rows selected) of the Epstein-Nesbet step of qmb/pert.py:37-61, in one engine call.

        E0 = Re<psi|H|psi>/<psi|psi> on ``configs`` (distinct rows); the
        connected rows are ``find_relative(configs, psi, count_selected,
        configs)``; E2 = sum |(H psi)_j|^2 / <psi|psi> / (E0 - Re H_jj) over them.
        """
        device = configs.device
        configs = self._configs(configs, "configs")
        n = configs.shape[0]
        psi = self._amplitudes(psi, n, "psi", device).to(torch.complex128)
        count_selected = int(count_selected)
        if count_selected <= 0:
            raise RuntimeError("count_selected must be positive.")
        table = self._table(device, configs.shape[1])
        lib = _native.library()
        need = ctypes.c_uint64(0)
        _native.check(lib.qmbx_pt2_workspace(table.h, n, count_selected, ctypes.byref(need)))
        energies = (ctypes.c_double * 2)()
        n_other = ctypes.c_int64(0)
        with torch.cuda.device(device):
            stream = _stream(device)
            for _ in range(4):
                ws = _workspace(need.value, device)
                want = ctypes.c_uint64(0)
                status = lib.qmbx_pt2(table.h, table.d, configs.data_ptr(), psi.data_ptr(), n, count_selected,
                                      energies, ctypes.byref(n_other), ws.data_ptr(), ws.numel(), ctypes.byref(want),
                                      stream)
                if status == _native.QMBX_ERR_WORKSPACE and want.value > need.value:
                    need = want
                    del ws
                    continue
                _native.check(status)
                break
            else:
                raise RuntimeError("pt2 could not size its workspace")
        return energies[0], energies[1], n_other.value

    # -- diagonal_term ----------------------------------------------------------

    def diagonal_term(self, configs: torch.Tensor) -> torch.Tensor:
        """<c|H|c> for every row (qmb/hamiltonian.py:168-186)."""
        device = configs.device
        configs = self._configs(configs, "configs")
        table = self._table(device, configs.shape[1])
        out = torch.empty(configs.shape[0], dtype=torch.complex128, device=device)
        with torch.cuda.device(device):
            _native.call("qmbx_diagonal_term", table.h, table.d, configs.data_ptr(), configs.shape[0], out.data_ptr(),
                         _stream(device))
        return out

    # -- single_relative --------------------------------------------------------

    def single_relative(self, configs: torch.Tensor) -> torch.Tensor:
        """One neighbour per row, drawn with probability proportional to |coef| (qmb/hamiltonian.py:188-206).

        The seed is drawn from torch's CPU generator, as the reference does
        (qmb/_hamiltonian_cuda.cu:963-964).
        """
        device = configs.device
        configs = self._configs(configs, "configs")
        table = self._table(device, configs.shape[1])
        seed = int(torch.randint(0, np.iinfo(np.int64).max, (), dtype=torch.int64))
        return self.single_relative_seeded(configs, seed)

    def single_relative_seeded(self, configs: torch.Tensor, seed: int) -> torch.Tensor:
        device = configs.device
        configs = self._configs(configs, "configs")
        table = self._table(device, configs.shape[1])
        lib = _native.library()
        need = ctypes.c_uint64(0)
        _native.check(lib.qmbx_single_relative_workspace(table.h, configs.shape[0], ctypes.byref(need)))
        out = torch.empty_like(configs)
        with torch.cuda.device(device):
            ws = _workspace(need.value, device)
            _native.call("qmbx_single_relative", table.h, table.d, configs.data_ptr(), configs.shape[0],
                         seed & (2**64 - 1), out.data_ptr(), ws.data_ptr(), ws.numel(), _stream(device))
        return out


class HamiltonianMatrix:
    """H restricted to one set of distinct rows, stored on the device as a sparse matrix (CSR).

    Built by ``Hamiltonian.matrix``: two term walks over the rows (count, then
    fill); ``apply(x)`` is then a sparse matrix-vector product, which is what
    an iterative eigensolver on a fixed basis (qmb/rldiag.py:19-52,
    qmb/haar.py:107-183) needs once per iteration.  Row j holds its diagonal
    entry first, then one entry per (term, row i) pair mapping row i onto row
    j.  ``row_ptr`` int64 [n + 1], ``col`` int32 [nnz], ``val`` complex128
    [nnz].
    """

    def __init__(self, row_ptr: torch.Tensor, col: torch.Tensor, val: torch.Tensor):
        self.row_ptr, self.col, self.val = row_ptr, col, val
        self.n = row_ptr.shape[0] - 1
        self.nnz = col.shape[0]

    def apply(self, x: torch.Tensor) -> torch.Tensor:
        """A x for complex128 x of shape [n], or of shape [n, m] (m vectors, one pass over the matrix);
        bit-identical on every call."""
        if x.dtype != torch.complex128 or x.dim() not in (1, 2) or x.shape[0] != self.n or \
                (x.dim() == 2 and x.shape[1] < 1):
            raise RuntimeError(f"x must be complex128 of shape [{self.n}] or [{self.n}, m].")
        if x.device != self.val.device:
            raise RuntimeError("x must be on the matrix's device.")
        x = x.contiguous()
        y = torch.empty_like(x)
        m = 1 if x.dim() == 1 else x.shape[1]
        with torch.cuda.device(x.device):
            _native.call("qmbx_matrix_apply_many", self.n, self.nnz, m, self.row_ptr.data_ptr(), self.col.data_ptr(),
                         self.val.data_ptr(), x.data_ptr(), y.data_ptr(), _stream(x.device))
        return y

    def to_dense(self) -> torch.Tensor:
        """The dense matrix (for checks on small row sets)."""
        rows = torch.repeat_interleave(torch.arange(self.n, device=self.val.device),
                                       self.row_ptr[1:] - self.row_ptr[:-1])
        dense = torch.zeros((self.n, self.n), dtype=torch.complex128, device=self.val.device)
        dense.index_put_((rows, self.col.to(torch.int64)), self.val, accumulate=True)
        return dense


class _HitRecord:
    """What a logged forward apply_within found (a device buffer), for its adjoint product."""

    def __init__(self, table: _Table, buf: torch.Tensor, cap: int, n_i: int, n_j: int, same: int,
                 dtype: torch.dtype, include_diagonal: bool):
        self.table, self.buf, self.cap, self.n_i, self.n_j, self.same = table, buf, cap, n_i, n_j, same
        self.dtype, self.include_diagonal = dtype, include_diagonal
        self.count = None  # (pinned host int64, event) once the adjoint is queued

    @property
    def hits(self) -> int | None:
        """Hits the forward found (waits for the copy queued with the adjoint)."""
        if self.count is None:
            return None
        self.count[1].synchronize()
        return int(self.count[0][0])


class _ApplyWithin(torch.autograd.Function):
    """y = H psi restricted to configs_j; backward applies H^dagger.

    The forward walk records its hits, and the backward replays that record
    (the adjoint needs exactly the (term, row) pairs the forward found); when
    the record could not hold them all, the library walks the adjoint
    instead, decided on the device, so the backward never waits for it.
    """

    @staticmethod
    def forward(ctx, ham: Hamiltonian, configs_i, psi_i, configs_j, out_dtype):
        ctx.ham = ham
        ctx.in_dtype = psi_i.dtype
        ctx.save_for_backward(configs_i, configs_j)
        deterministic = os.environ.get("QMBX_DETERMINISTIC", "")[:1] not in ("", "0")
        if not ham.hit_log or deterministic:  # the replay adds with atomics; the walk can be fixed-order
            ctx.record = None
            return ham._apply(configs_i, psi_i.detach(), configs_j, adjoint=False, out_dtype=out_dtype)
        out, ctx.record = ham._apply(configs_i, psi_i.detach(), configs_j, adjoint=False, out_dtype=out_dtype,
                                     log=True)
        return out

    @staticmethod
    def backward(ctx, grad):
        configs_i, configs_j = ctx.saved_tensors
        if grad is None:
            return None, None, None, None, None
        g = grad.to(ctx.in_dtype).contiguous()
        want = torch.complex128 if ctx.in_dtype == torch.complex128 else None
        if ctx.record is not None:
            gi = ctx.ham._adjoint_from_log(ctx.record, g, want)
        else:
            gi = ctx.ham._apply(configs_i, g, configs_j, adjoint=True, out_dtype=want)
        ctx.record = None
        return None, None, gi.to(ctx.in_dtype), None, None
