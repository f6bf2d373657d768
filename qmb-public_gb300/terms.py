"""Term tables and configurations for the Hamiltonian engine.

``prepare`` turns the reference's Hamiltonian dictionary into its
``(site, kind, coef)`` table (qmb/_hamiltonian.cpp:29-64) and ``sort_terms``
orders that table as ``Hamiltonian.__init__`` does (qmb/hamiltonian.py:93-97).

The remaining functions build seeded synthetic Hamiltonians and determinant
sets with the shapes the engine is exercised on:

* ``integral_terms`` — an ab-initio-like Hamiltonian from random one- and
  two-electron integrals, mapped to spin orbitals with the interleaved
  convention of qmb/fcidump.py:97-114 (alpha = 2p, beta = 2p + 1; two-body
  tensor (ps|qr)/2 for a+_p a+_q a_r a_s) and brought to normal order the way
  openfermion's ``normal_ordered`` does (creation operators first, indices
  descending within each group, one sign flip per transposition, equal keys
  merged, coefficients below 1e-8 in magnitude dropped).
* ``hubbard_dict`` — the Fermi-Hubbard lattice of qmb/hubbard.py:63-86.
* ``random_determinants`` — unique, lexicographically sorted determinants with
  fixed alpha/beta electron counts.
"""

from __future__ import annotations

import numpy as np
import torch

EQ_TOLERANCE = 1e-8


def prepare(hamiltonian: dict) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Dictionary ``{((site, kind), ...): coef}`` to ``(site, kind, coef)``.

    Same layout as qmb/_hamiltonian.cpp:29-64: ``site`` int16[T, 4],
    ``kind`` uint8[T, 4] with 2 marking an empty slot, ``coef`` float64[T, 2]
    (real, imaginary), in dictionary order.  Empty slots hold site 0 (the
    reference leaves them uninitialised; the engine never reads them).
    """
    n = len(hamiltonian)
    site = np.zeros((n, 4), dtype=np.int16)
    kind = np.full((n, 4), 2, dtype=np.uint8)
    coef = np.zeros((n, 2), dtype=np.float64)
    for index, (key, value) in enumerate(hamiltonian.items()):
        if len(key) > 4:
            raise ValueError(f"a term has at most 4 operators, got {len(key)}")
        for slot, (s, k) in enumerate(key):
            site[index, slot] = s
            kind[index, slot] = k
        value = complex(value)
        coef[index, 0] = value.real
        coef[index, 1] = value.imag
    return torch.from_numpy(site), torch.from_numpy(kind), torch.from_numpy(coef)


def sort_terms(site: torch.Tensor, kind: torch.Tensor, coef: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Order terms by |coef| descending, with the same torch call as qmb/hamiltonian.py:93-97."""
    order = coef.norm(dim=1).argsort(descending=True)
    return site[order], kind[order], coef[order]


# ---------------------------------------------------------------------------
# synthetic ab-initio Hamiltonian
# ---------------------------------------------------------------------------


def random_integrals(n_orbit: int, seed: int, *, complex_valued: bool = False):
    """Seeded integrals: e0, h[p,q] and the chemist-notation tensor (pq|rs).

    h is symmetric (Hermitian when complex) with entries N(0,1)·exp(-|p-q|/2);
    (pq|rs) has the 8-fold permutational symmetry of real orbitals with
    entries N(0, 0.1) (standard deviation 0.1).
    """
    rng = np.random.default_rng(seed)
    e0 = float(rng.standard_normal())
    p = np.arange(n_orbit)
    decay = np.exp(-np.abs(p[:, None] - p[None, :]) / 2)
    upper = rng.standard_normal((n_orbit, n_orbit))
    h = np.triu(upper) + np.triu(upper, 1).T
    h = h * decay
    if complex_valued:
        im = rng.standard_normal((n_orbit, n_orbit)) * 0.3
        im = np.triu(im, 1)
        h = h + 1j * (im - im.T) * decay
    raw = rng.standard_normal((n_orbit,) * 4) * 0.1
    i, j, k, l = np.meshgrid(p, p, p, p, indexing="ij")
    a = np.maximum(i, j)
    b = np.minimum(i, j)
    c = np.maximum(k, l)
    d = np.minimum(k, l)
    first = (a > c) | ((a == c) & (b >= d))
    ia = np.where(first, a, c)
    ib = np.where(first, b, d)
    ic = np.where(first, c, a)
    id_ = np.where(first, d, b)
    eri = raw[ia, ib, ic, id_]
    return e0, h, eri


def integral_terms(n_orbit: int, seed: int, *, complex_valued: bool = False):
    """Normal-ordered fermion terms of the seeded synthetic integrals (see ``terms_from_integrals``)."""
    e0, h, eri = random_integrals(n_orbit, seed, complex_valued=complex_valued)
    return terms_from_integrals(e0, h, eri)


def terms_from_integrals(e0: float, h: np.ndarray, eri: np.ndarray):
    """Normal-ordered fermion terms of the integrals (e0, h[p,q], chemist (pq|rs)).

    Returns numpy ``(site, kind, coef)`` in a deterministic order: the
    constant, the one-body terms a+_P a_Q by (P, Q), the two-body terms
    a+_P a+_Q a_R a_S (P > Q, R > S) by key; spin orbitals interleaved
    (alpha 2p, beta 2p + 1).
    """
    n = h.shape[0]
    ns = 2 * n
    # one-body: a+_P a_Q, same spin
    p, q = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    p = p.ravel()
    q = q.ravel()
    one_keys = []
    one_vals = []
    for sigma in (0, 1):
        one_keys.append(np.stack([2 * p + sigma, 2 * q + sigma], axis=1))
        one_vals.append(h[p, q])
    one_keys = np.concatenate(one_keys)
    one_vals = np.concatenate(one_vals).astype(np.complex128)
    order = np.lexsort((one_keys[:, 1], one_keys[:, 0]))
    one_keys = one_keys[order]
    one_vals = one_vals[order]
    keep = np.abs(one_vals) >= EQ_TOLERANCE
    one_keys = one_keys[keep]
    one_vals = one_vals[keep]

    # two-body: coefficient of a+_P a+_Q a_R a_S is (ps|qr)/2 within the spin
    # blocks (P,Q,R,S) = (s1, s2, s2, s1) (qmb/fcidump.py:97-110)
    grid = np.arange(n)
    pp, qq, rr, ss = (x.ravel() for x in np.meshgrid(grid, grid, grid, grid, indexing="ij"))
    value = eri[pp, ss, qq, rr] / 2
    packed = []
    vals = []
    for s1 in (0, 1):
        for s2 in (0, 1):
            P = 2 * pp + s1
            Q = 2 * qq + s2
            R = 2 * rr + s2
            S = 2 * ss + s1
            live = (P != Q) & (R != S)
            P, Q, R, S, v = P[live], Q[live], R[live], S[live], value[live].astype(np.complex128)
            sign = np.ones(P.shape[0])
            swap = P < Q
            P, Q = np.where(swap, Q, P), np.where(swap, P, Q)
            sign = np.where(swap, -sign, sign)
            swap = R < S
            R, S = np.where(swap, S, R), np.where(swap, R, S)
            sign = np.where(swap, -sign, sign)
            packed.append(((P.astype(np.int64) * ns + Q) * ns + R) * ns + S)
            vals.append(v * sign)
    packed = np.concatenate(packed)
    vals = np.concatenate(vals)
    uniq, inverse = np.unique(packed, return_inverse=True)
    two_vals = np.zeros(uniq.shape[0], dtype=np.complex128)
    np.add.at(two_vals, inverse, vals)
    keep = np.abs(two_vals) >= EQ_TOLERANCE
    uniq = uniq[keep]
    two_vals = two_vals[keep]
    S = uniq % ns
    R = (uniq // ns) % ns
    Q = (uniq // ns // ns) % ns
    P = uniq // ns // ns // ns
    two_keys = np.stack([P, Q, R, S], axis=1)

    t_one = one_keys.shape[0]
    t_two = two_keys.shape[0]
    total = 1 + t_one + t_two
    site = np.zeros((total, 4), dtype=np.int16)
    kind = np.full((total, 4), 2, dtype=np.uint8)
    coef = np.zeros((total, 2), dtype=np.float64)
    coef[0] = (e0, 0.0)
    site[1:1 + t_one, :2] = one_keys
    kind[1:1 + t_one, :2] = (1, 0)
    coef[1:1 + t_one, 0] = one_vals.real
    coef[1:1 + t_one, 1] = one_vals.imag
    site[1 + t_one:] = two_keys
    kind[1 + t_one:] = (1, 1, 0, 0)
    coef[1 + t_one:, 0] = two_vals.real
    coef[1 + t_one:, 1] = two_vals.imag
    return site, kind, coef


def table_to_dict(site, kind, coef) -> dict:
    """Inverse of ``prepare`` for tables whose empty slots trail the operators."""
    site = np.asarray(site)
    kind = np.asarray(kind)
    coef = np.asarray(coef)
    out = {}
    for t in range(site.shape[0]):
        key = tuple((int(site[t, k]), int(kind[t, k])) for k in range(4) if kind[t, k] != 2)
        out[key] = complex(coef[t, 0], coef[t, 1])
    return out


def integral_hamiltonian_tables(n_orbit: int, seed: int, *, complex_valued: bool = False):
    """``(site, kind, coef)`` torch tensors ordered as ``Hamiltonian(dict)`` orders them."""
    site, kind, coef = integral_terms(n_orbit, seed, complex_valued=complex_valued)
    return sort_terms(torch.from_numpy(site), torch.from_numpy(kind), torch.from_numpy(coef))


def read_fcidump(path: str):
    """Read an FCIDUMP file (optionally gzip-compressed) into a term table.

    Restates the parsing of qmb/fcidump.py:50-95: the header's NORB, NELEC and
    MS2; integral lines ``value i j k l`` with 1-based orbitals, where
    (0,0,0,0) is the constant, (i,0,0,0) is skipped, (i,j,0,0) a symmetric
    one-body integral, (i,j,k,l) a chemist two-body integral (ij|kl) with its
    8-fold permutations, (i,j,k,0) an error.  The integrals then become
    normal-ordered terms as in ``terms_from_integrals`` (no openfermion
    needed) and are ordered as ``Hamiltonian(dict)`` orders them.
    Returns ``(n_orbit, n_electron, ms2, site, kind, coef)`` with torch tensors.
    """
    import gzip
    import re

    opener = gzip.open if str(path).endswith(".gz") else open
    with opener(path, "rt", encoding="utf-8") as f:
        n_orbit = n_electron = ms2 = None
        for line in f:
            low = line.lower()
            if (m := re.search(r"norb\s*=\s*(\d+)", low)) is not None:
                n_orbit = int(m.group(1))
            if (m := re.search(r"nelec\s*=\s*(\d+)", low)) is not None:
                n_electron = int(m.group(1))
            if (m := re.search(r"ms2\s*=\s*(\d+)", low)) is not None:
                ms2 = int(m.group(1))
            if "&end" in low or "/" == low.strip():
                break
        if n_orbit is None or n_electron is None or ms2 is None:
            raise ValueError("FCIDUMP header lacks NORB, NELEC or MS2")
        e0 = 0.0
        h = np.zeros((n_orbit, n_orbit))
        eri = np.zeros((n_orbit,) * 4)
        for line in f:
            parts = line.split()
            if not parts:
                continue
            value = float(parts[0].replace("D", "E").replace("d", "e"))
            i, j, k, l = (int(x) - 1 for x in parts[1:5])
            if (i, j, k, l) == (-1, -1, -1, -1):
                e0 = value
            elif j == -1 and k == -1 and l == -1:
                continue
            elif k == -1 and l == -1:
                h[i, j] = h[j, i] = value
            elif l == -1:
                raise ValueError(f"invalid FCIDUMP line: {line.strip()}")
            else:
                for a, b, c, d in ((i, j, k, l), (i, j, l, k), (j, i, k, l), (j, i, l, k), (l, k, j, i), (k, l, j, i),
                                   (l, k, i, j), (k, l, i, j)):
                    eri[a, b, c, d] = value
    site, kind, coef = terms_from_integrals(e0, h, eri)
    site, kind, coef = sort_terms(torch.from_numpy(site), torch.from_numpy(kind), torch.from_numpy(coef))
    return n_orbit, n_electron, ms2, site, kind, coef


def write_fcidump(path: str, e0: float, h: np.ndarray, eri: np.ndarray, n_electron: int, ms2: int = 0) -> None:
    """Write real integrals in FCIDUMP form (unique 8-fold two-body entries, i >= j, k >= l, ij >= kl)."""
    n = h.shape[0]
    with open(path, "w", encoding="utf-8") as f:
        f.write(f" &FCI NORB={n},NELEC={n_electron},MS2={ms2},\n  ORBSYM={','.join(['1'] * n)},\n  ISYM=1,\n &END\n")
        for i in range(n):
            for j in range(i + 1):
                for k in range(n):
                    for l in range(k + 1):
                        if i * (i + 1) // 2 + j >= k * (k + 1) // 2 + l and eri[i, j, k, l] != 0.0:
                            f.write(f"{eri[i, j, k, l]:.17e} {i + 1} {j + 1} {k + 1} {l + 1}\n")
        for i in range(n):
            for j in range(i + 1):
                if h[i, j] != 0.0:
                    f.write(f"{h[i, j]:.17e} {i + 1} {j + 1} 0 0\n")
        f.write(f"{e0:.17e} 0 0 0 0\n")


def n_integral_terms(n_orbit: int) -> int:
    """Term count of a dense-integral table: 2·C(n,2)² + n⁴ + 2n² + 1."""
    c2 = n_orbit * (n_orbit - 1) // 2
    return 2 * c2 * c2 + n_orbit**4 + 2 * n_orbit**2 + 1


# ---------------------------------------------------------------------------
# Fermi-Hubbard
# ---------------------------------------------------------------------------


def hubbard_dict(m: int, n: int, t: float, u: float) -> dict:
    """Open m×n Fermi-Hubbard lattice with spin, site index (i + j*m)*2 + o (qmb/hubbard.py:63-86)."""

    def index(i: int, j: int, o: int) -> int:
        return (i + j * m) * 2 + o

    out: dict = {}
    for i in range(m):
        for j in range(n):
            out[(index(i, j, 0), 1), (index(i, j, 0), 0), (index(i, j, 1), 1), (index(i, j, 1), 0)] = u
            if i != 0:
                for o in (0, 1):
                    out[(index(i, j, o), 1), (index(i - 1, j, o), 0)] = -t
                    out[(index(i - 1, j, o), 1), (index(i, j, o), 0)] = -t
            if j != 0:
                for o in (0, 1):
                    out[(index(i, j, o), 1), (index(i, j - 1, o), 0)] = -t
                    out[(index(i, j - 1, o), 1), (index(i, j, o), 0)] = -t
    return out


# ---------------------------------------------------------------------------
# configurations
# ---------------------------------------------------------------------------


def sort_rows(rows: np.ndarray) -> np.ndarray:
    """Lexicographic row order, unsigned bytes, byte 0 most significant."""
    rows = np.ascontiguousarray(rows, dtype=np.uint8)
    if rows.shape[0] == 0:
        return rows
    order = np.lexsort(tuple(rows[:, k] for k in range(rows.shape[1] - 1, -1, -1)))
    return rows[order]


def unique_rows(rows: np.ndarray) -> np.ndarray:
    rows = sort_rows(rows)
    if rows.shape[0] == 0:
        return rows
    keep = np.ones(rows.shape[0], dtype=bool)
    keep[1:] = np.any(rows[1:] != rows[:-1], axis=1)
    return rows[keep]


def pack_sites(bits: np.ndarray, n_qubytes: int) -> np.ndarray:
    """Occupation bits [N, n_sites] to rows [N, n_qubytes] (site s -> byte s/8, bit s%8)."""
    n, n_sites = bits.shape
    full = np.zeros((n, n_qubytes * 8), dtype=np.uint8)
    full[:, :n_sites] = bits
    return np.packbits(full, axis=1, bitorder="little")


def random_determinants(n_orbit: int, n_alpha: int, n_beta: int, count: int, seed: int, *,
                        n_qubytes: int | None = None) -> np.ndarray:
    """``count`` unique random determinants, sorted; alpha on even sites, beta on odd sites."""
    rng = np.random.default_rng(seed)
    n_sites = 2 * n_orbit
    nq = n_qubytes if n_qubytes is not None else (n_sites + 7) // 8
    have = np.zeros((0, nq), dtype=np.uint8)
    while have.shape[0] < count:
        batch = max(1024, int((count - have.shape[0]) * 1.1) + 16)
        bits = np.zeros((batch, n_sites), dtype=np.uint8)
        alpha = np.argsort(rng.random((batch, n_orbit)), axis=1)[:, :n_alpha]
        beta = np.argsort(rng.random((batch, n_orbit)), axis=1)[:, :n_beta]
        rows = np.arange(batch)[:, None]
        bits[rows, 2 * alpha] = 1
        bits[rows, 2 * beta + 1] = 1
        have = unique_rows(np.concatenate([have, pack_sites(bits, nq)]))
        space = _comb(n_orbit, n_alpha) * _comb(n_orbit, n_beta)
        if have.shape[0] >= space and have.shape[0] < count:
            raise ValueError(f"only {space} determinants exist, asked for {count}")
    pick = np.sort(rng.choice(have.shape[0], size=count, replace=False))
    return have[pick]


def all_determinants(n_orbit: int, n_alpha: int, n_beta: int, *, n_qubytes: int | None = None) -> np.ndarray:
    """Every determinant with the given electron counts, sorted."""
    from itertools import combinations

    n_sites = 2 * n_orbit
    nq = n_qubytes if n_qubytes is not None else (n_sites + 7) // 8
    alphas = list(combinations(range(n_orbit), n_alpha))
    betas = list(combinations(range(n_orbit), n_beta))
    bits = np.zeros((len(alphas) * len(betas), n_sites), dtype=np.uint8)
    r = 0
    for a in alphas:
        for b in betas:
            for x in a:
                bits[r, 2 * x] = 1
            for x in b:
                bits[r, 2 * x + 1] = 1
            r += 1
    return unique_rows(pack_sites(bits, nq))


def _comb(n: int, k: int) -> int:
    from math import comb

    return comb(n, k)


def random_psi(count: int, seed: int, dtype=np.complex128) -> np.ndarray:
    """Seeded complex N(0,1) amplitudes."""
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(count) + 1j * rng.standard_normal(count)).astype(dtype)
