"""The C ABI library: it loads without a GPU, exports every declared symbol, and
its host-side term compiler reproduces the reference's operator walk."""

from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

import oracle
from conftest import REPO, golden

native = __import__("qmb_gb300._native", fromlist=["library"])


@pytest.fixture(scope="module")
def lib():
    import importlib

    importlib.import_module("qmb-public_gb300._build").build()
    return native.library()


def declared_symbols() -> list[str]:
    text = open(os.path.join(REPO, "include", "qmbx.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(qmbx_\w+)\s*\(", text, flags=re.M)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 14
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(native.SIGNATURES), "the ctypes binding must cover exactly the header"


def test_version_and_no_error(lib):
    assert lib.qmbx_version() >= 10000
    assert lib.qmbx_last_error() == b""


class Part(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("off_test", ctypes.c_uint64), ("off_apply", ctypes.c_uint64), ("off_coef", ctypes.c_uint64), ("off_coef32", ctypes.c_uint64), ("off_orig", ctypes.c_uint64),
                ("off_norm", ctypes.c_uint64), ("off_groups", ctypes.c_uint64), ("off_single_ne", ctypes.c_uint64),
                ("off_pair_ne", ctypes.c_uint64), ("off_nonempty", ctypes.c_uint64), ("off_narrow", ctypes.c_uint64),
                ("n_groups", ctypes.c_int64), ("n_nonempty", ctypes.c_int64),
                ("wide_groups", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Header(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_uint32), ("version", ctypes.c_uint32), ("n_qubytes", ctypes.c_int32),
                ("particle_cut", ctypes.c_int32), ("n_words", ctypes.c_int32), ("n_sites", ctypes.c_int32),
                ("n_terms", ctypes.c_int64), ("n_live", ctypes.c_int64), ("part", Part * 3),
                ("total_bytes", ctypes.c_uint64)]


def compile_table(lib, site, kind, coef, nq, pc):
    site = np.ascontiguousarray(site, dtype=np.int16)
    kind = np.ascontiguousarray(kind, dtype=np.uint8)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    nbytes = ctypes.c_uint64()
    native.check(lib.qmbx_table_bytes(site.ctypes.data, kind.ctypes.data, site.shape[0], nq, pc, ctypes.byref(nbytes)))
    blob = np.zeros(nbytes.value, dtype=np.uint8)
    native.check(lib.qmbx_table_build(site.ctypes.data, kind.ctypes.data, coef.ctypes.data, site.shape[0], nq, pc,
                                      blob.ctypes.data, blob.size))
    return blob


def read_part(blob, h, which):
    p = h.part[which]
    w = h.n_words
    n = p.n

    def arr(off, dtype, count):
        return np.frombuffer(blob, dtype=dtype, count=count, offset=off)

    # word-major: (mask, val) and (flip, par) of word q of term t at [q, t]
    test = arr(p.off_test, np.uint64, n * 2 * w).reshape(w, n, 2).transpose(1, 0, 2)
    apply = arr(p.off_apply, np.uint64, n * 2 * w).reshape(w, n, 2).transpose(1, 0, 2)
    coef = arr(p.off_coef, np.float64, n * 2).reshape(n, 2)
    orig = arr(p.off_orig, np.int32, n)
    return test, apply, coef, orig


def to_key(row: np.ndarray, w: int) -> list[int]:
    padded = np.zeros(8 * w, dtype=np.uint8)
    padded[:row.size] = row
    return [int.from_bytes(bytes(padded[8 * q:8 * q + 8]), "big") for q in range(w)]


def from_key(key: list[int], nq: int) -> np.ndarray:
    raw = b"".join(k.to_bytes(8, "big") for k in key)
    return np.frombuffer(raw[:nq], dtype=np.uint8).copy()


def check_groups(blob, h, which, part):
    """Terms sit in the group of their two lowest required-occupied key positions, stable in input order."""
    p = h.part[which]
    w = h.n_words
    groups = np.frombuffer(blob, dtype=np.int32, count=2 * p.n_groups, offset=p.off_groups).reshape(-1, 2)
    single_ne = np.frombuffer(blob, dtype=np.uint64, count=w, offset=p.off_single_ne)
    pair_ne = np.frombuffer(blob, dtype=np.uint64, count=64 * w * w, offset=p.off_pair_ne).reshape(64 * w, w)
    test, _, _, orig = part
    assert groups[0, 0] == 0 and groups[-1, 1] == p.n
    assert np.all(groups[1:, 0] == groups[:-1, 1])
    P = 64 * w
    listed = np.frombuffer(blob, dtype=np.int32, count=4 * p.n_nonempty, offset=p.off_nonempty).reshape(-1, 4)
    nonempty = np.nonzero(groups[:, 1] > groups[:, 0])[0]
    assert len(nonempty) == p.n_nonempty
    assert np.array_equal(listed[:, :2], groups[nonempty])
    for (lo, hi, a, b), g in zip(listed, nonempty):
        if g == 0:
            assert a == -1 and b == -1
        elif g <= P:
            assert a == g - 1 and b == -1
        else:
            assert g == 1 + P + b * (b - 1) // 2 + a and 0 <= a < b
    for g in nonempty:
        lo, hi = groups[g]
        assert list(orig[lo:hi]) == sorted(orig[lo:hi])
        for slot in range(lo, hi):
            req = [64 * q + b for q in range(w) for b in range(64)
                   if (int(test[slot, q, 0]) & int(test[slot, q, 1])) >> b & 1]
            if len(req) >= 2:
                a, b = req[0], req[1]
                assert g == 1 + P + b * (b - 1) // 2 + a
                assert int(pair_ne[a, b >> 6]) >> (b & 63) & 1
            elif len(req) == 1:
                assert g == 1 + req[0]
                assert int(single_ne[req[0] >> 6]) >> (req[0] & 63) & 1
            else:
                assert g == 0


def check_narrow(blob, h, which, part):
    """Tables of at most 32 sites hold (mask, val, flip, par) >> 32 of every term; the low halves are zero."""
    p = h.part[which]
    test, apply, _, _ = part
    if h.n_sites > 32:
        assert p.off_narrow == 0
        return
    assert p.off_narrow != 0 and p.off_narrow % 16 == 0
    narrow = np.frombuffer(blob, dtype=np.uint32, count=4 * p.n, offset=p.off_narrow).reshape(p.n, 4)
    full = np.stack([test[:, 0, 0], test[:, 0, 1], apply[:, 0, 0], apply[:, 0, 1]], axis=1)
    assert np.all(full & np.uint64(0xFFFFFFFF) == 0)
    assert np.array_equal((full >> np.uint64(32)).astype(np.uint32), narrow)


def closed_form(test, apply, key):
    for q, word in enumerate(key):
        mask, val = int(test[q, 0]), int(test[q, 1])
        if (word ^ val) & mask:
            return None
    image = [word ^ int(apply[q, 0]) for q, word in enumerate(key)]
    parity = sum(bin(word & int(apply[q, 1])).count("1") for q, word in enumerate(key)) & 1
    return image, parity


@pytest.mark.parametrize("case", ["random_terms_fermi", "random_terms_bose2", "ab_initio_6", "ising_4x4", "hubbard_3x2"])
def test_compiled_terms_reproduce_the_operator_walk(lib, case):
    g = golden(case)
    site, kind, coef = g["site"], g["kind"], g["coef"]
    pc = int(g["particle_cut"])
    rows = np.concatenate([g["configs_i"], g["configs_j"]])[:120]
    nq = rows.shape[1]
    blob = compile_table(lib, site, kind, coef, nq, pc)
    h = Header.from_buffer_copy(blob[:ctypes.sizeof(Header)].tobytes())
    assert h.n_words == (nq + 7) // 8
    fwd = read_part(blob, h, 0)
    adj = read_part(blob, h, 1)
    diag = read_part(blob, h, 2)
    assert fwd[0].shape[0] == adj[0].shape[0]
    # every live term appears exactly once; the adjoint part holds the same terms as the forward part
    live = []
    for part in (fwd, diag):
        live.extend(part[3].tolist())
    assert len(live) == len(set(live))
    assert sorted(fwd[3].tolist()) == sorted(adj[3].tolist())
    for which, part in ((0, fwd), (1, adj), (2, diag)):
        check_groups(blob, h, which, part)
        check_narrow(blob, h, which, part)
    # the same terms on rows of more than 32 sites carry no narrow records
    wide = compile_table(lib, site, kind, coef, 5, pc)
    hw = Header.from_buffer_copy(wide[:ctypes.sizeof(Header)].tobytes())
    assert all(hw.part[k].off_narrow == 0 for k in range(3))
    for t in range(site.shape[0]):
        ok_any = any(oracle.apply_term(site[t], kind[t], r, pc)[0] for r in rows[:40])
        if ok_any:
            assert t in live
    for part_name, (test, apply, cf, orig) in (("fwd", fwd), ("diag", diag)):
        for slot in range(len(orig)):
            t = int(orig[slot])
            for r in rows:
                ok, parity, out = oracle.apply_term(site[t], kind[t], r, pc)
                got = closed_form(test[slot], apply[slot], to_key(r, h.n_words))
                assert (got is not None) == ok, (part_name, t)
                if not ok:
                    continue
                image, par = got
                assert np.array_equal(from_key(image, nq), out)
                # the stored coefficient carries the constant part of the sign
                sign = -1.0 if parity else 1.0
                stored_sign = -1.0 if par else 1.0
                np.testing.assert_array_equal(cf[slot] * stored_sign, coef[t] * sign)
                if part_name == "diag":
                    assert np.array_equal(out, r)
    # the adjoint part maps every image back to its source with the same sign
    test_a, apply_a, cf_a, orig_a = adj
    for slot in range(len(orig_a)):
        t = int(orig_a[slot])
        for r in rows[:60]:
            ok, parity, out = oracle.apply_term(site[t], kind[t], r, pc)
            if not ok:
                continue
            back = closed_form(test_a[slot], apply_a[slot], to_key(out, h.n_words))
            assert back is not None
            image, par = back
            assert np.array_equal(from_key(image, nq), r)
            assert np.array_equal(cf_a[slot] * (-1.0 if par else 1.0), coef[t] * (-1.0 if parity else 1.0))


def test_table_rejects_bad_input(lib):
    site = np.array([[0, 1, 0, 0]], dtype=np.int16)
    kind = np.array([[1, 0, 2, 2]], dtype=np.uint8)
    nbytes = ctypes.c_uint64()
    assert lib.qmbx_table_bytes(site.ctypes.data, kind.ctypes.data, 1, 0, 1, ctypes.byref(nbytes)) == native.QMBX_ERR_ARGUMENT
    assert b"n_qubytes" in lib.qmbx_last_error()
    assert lib.qmbx_table_bytes(site.ctypes.data, kind.ctypes.data, 1, 1, 3, ctypes.byref(nbytes)) == native.QMBX_ERR_ARGUMENT
    bad_site = np.array([[8, 1, 0, 0]], dtype=np.int16)
    assert lib.qmbx_table_bytes(bad_site.ctypes.data, kind.ctypes.data, 1, 1, 1, ctypes.byref(nbytes)) == native.QMBX_ERR_ARGUMENT
    assert b"site 8" in lib.qmbx_last_error()
    bad_kind = np.array([[0, 1, 0, 0]], dtype=np.uint8) + 3
    assert lib.qmbx_table_bytes(site.ctypes.data, bad_kind.ctypes.data, 1, 1, 1, ctypes.byref(nbytes)) == native.QMBX_ERR_ARGUMENT
    # empty slots may hold any site value (the reference leaves them uninitialised)
    garbage = np.array([[3, 1, -77, 900]], dtype=np.int16)
    assert lib.qmbx_table_bytes(garbage.ctypes.data, kind.ctypes.data, 1, 1, 1, ctypes.byref(nbytes)) == native.QMBX_OK
    assert lib.qmbx_last_error() == b""


def test_dead_terms_are_dropped(lib):
    # a+_1 a+_1 can never apply; a+_2 a_2 is diagonal; a+_3 a_1 changes the row
    site = np.array([[1, 1, 0, 0], [2, 2, 0, 0], [3, 1, 0, 0]], dtype=np.int16)
    kind = np.array([[1, 1, 2, 2], [1, 0, 2, 2], [1, 0, 2, 2]], dtype=np.uint8)
    coef = np.ones((3, 2))
    blob = compile_table(lib, site, kind, coef, 1, 1)
    counts = (ctypes.c_int64 * 6)()
    native.check(lib.qmbx_table_counts(blob.ctypes.data, counts))
    assert list(counts) == [3, 2, 1, 1, 1, 1]


def hermitian_flag(lib, site, kind, coef, nq, pc):
    blob = compile_table(lib, site, kind, coef, nq, pc)
    flag = ctypes.c_int32()
    native.check(lib.qmbx_table_hermitian(blob.ctypes.data, ctypes.byref(flag)))
    return flag.value


@pytest.mark.parametrize("case", ["ab_initio_6", "ab_initio_10_complex", "random_terms_fermi", "random_terms_bose2",
                                  "ising_4x4", "hubbard_3x2"])
def test_hermitian_flag_agrees_with_the_dense_matrix(lib, case):
    g = golden(case)
    pc = int(g["particle_cut"])
    rows = np.concatenate([g["configs_i"], g["configs_j"]])[:150]
    rows = np.unique(rows, axis=0)
    flag = hermitian_flag(lib, g["site"], g["kind"], g["coef"], rows.shape[1], pc)
    h = oracle.dense_matrix(g["site"], g["kind"], g["coef"], rows, pc)
    gap = np.abs(h - h.conj().T).max()
    if flag:
        # a principal block of a Hermitian operator is Hermitian
        assert gap <= 1e-12 * max(1.0, np.abs(h).max())
    else:
        assert gap > 1e-6


def test_hermitian_flag_on_written_out_operators(lib):
    site = np.array([[0, 1, 0, 0], [1, 0, 0, 0], [2, 2, 0, 0]], dtype=np.int16)
    kind = np.array([[1, 0, 2, 2], [1, 0, 2, 2], [1, 0, 2, 2]], dtype=np.uint8)
    # a+_0 a_1 + a+_1 a_0 + 0.5 n_2 is Hermitian; with i and -i on the hops too
    assert hermitian_flag(lib, site, kind, np.array([[1.0, 0], [1.0, 0], [0.5, 0]]), 1, 1) == 1
    assert hermitian_flag(lib, site, kind, np.array([[0, 1.0], [0, -1.0], [0.5, 0]]), 1, 1) == 1
    # i on both hops, or a complex diagonal coefficient, is not
    assert hermitian_flag(lib, site, kind, np.array([[0, 1.0], [0, 1.0], [0.5, 0]]), 1, 1) == 0
    assert hermitian_flag(lib, site, kind, np.array([[1.0, 0], [1.0, 0], [0.5, 0.5]]), 1, 1) == 0
    # the second hop written in the other order: -a_0 a+_1 is the same operator as a+_1 a_0
    site2 = np.array([[0, 1, 0, 0], [0, 1, 0, 0], [2, 2, 0, 0]], dtype=np.int16)
    kind2 = np.array([[1, 0, 2, 2], [0, 1, 2, 2], [1, 0, 2, 2]], dtype=np.uint8)
    assert hermitian_flag(lib, site2, kind2, np.array([[1.0, 0], [-1.0, 0], [0.5, 0]]), 1, 1) == 1
    assert hermitian_flag(lib, site2, kind2, np.array([[1.0, 0], [1.0, 0], [0.5, 0]]), 1, 1) == 0
