"""Generate the golden fixtures of tests/golden/ by running the reference engine.

Run in a container that holds the reference source tree (qmb-public) and a
C++ toolchain:

    python tests/golden/make_golden.py --reference /path/to/qmb-public

It imports the reference's ``qmb.hamiltonian`` (its JIT-built CPU extension,
qmb/_hamiltonian_cpu.cpp, compiled by torch.utils.cpp_extension into a
temporary cache) and ``qmb.bitspack``, evaluates ``apply_within`` and
``find_relative`` on small seeded cases, and writes one compressed ``.npz``
per case holding the inputs and the reference's outputs.  The reference has
no CPU ``diagonal_term``; its value is taken as ``apply_within([c], [1], [c])``
per configuration, as the reference CPU engine computes it.

The fixtures are the only thing the tests read; the reference is not needed
to run the tests.
"""

from __future__ import annotations

import argparse
import os
import pathlib
import sys
import tempfile
import types

import numpy as np
import torch

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "qmb-public_gb300"))
import terms  # noqa: E402  (the package's generators, imported by path)


def load_reference(root: str):
    sys.dont_write_bytecode = True
    cache = pathlib.Path(tempfile.gettempdir()) / "qmb_reference_cache"
    stub = types.ModuleType("platformdirs")
    stub.user_cache_path = lambda appname=None, appauthor=None: cache  # type: ignore[attr-defined]
    sys.modules["platformdirs"] = stub
    sys.path.insert(0, root)
    import qmb.bitspack  # type: ignore
    import qmb.hamiltonian  # type: ignore

    return qmb.hamiltonian, qmb.bitspack


def ising_dict(m: int, n: int, x: float, z: float, zz: float, yy: float) -> dict:
    """Hard-core boson spin model in the form of qmb/ising.py:105-210 (X, Z fields, ZZ and YY bonds)."""
    from collections import defaultdict

    def idx(i, j):
        return i + j * m

    def X(i, j):
        return ((((idx(i, j), 1),), 1), (((idx(i, j), 0),), 1))

    def Y(i, j):
        return ((((idx(i, j), 1),), -1j), (((idx(i, j), 0),), 1j))

    def Z(i, j):
        return ((((idx(i, j), 1), (idx(i, j), 0)), 1), (((idx(i, j), 0), (idx(i, j), 1)), -1))

    h = defaultdict(complex)
    for i in range(m):
        for j in range(n):
            for k, v in X(i, j):
                h[k] += v * x
            for k, v in Z(i, j):
                h[k] += v * z
            if i != 0:
                for k1, v1 in Z(i, j):
                    for k2, v2 in Z(i - 1, j):
                        h[(*k1, *k2)] += v1 * v2 * zz
                for k1, v1 in Y(i, j):
                    for k2, v2 in Y(i - 1, j):
                        h[(*k1, *k2)] += v1 * v2 * yy
    return dict(h)


def random_terms_dict(n_sites: int, n_terms: int, seed: int) -> dict:
    """Arbitrary operator strings: repeated sites, any order, complex coefficients, an identity term."""
    rng = np.random.default_rng(seed)
    out = {(): complex(0.7, -0.2)}
    while len(out) < n_terms:
        n_ops = int(rng.integers(1, 5))
        key = tuple((int(rng.integers(0, n_sites)), int(rng.integers(0, 2))) for _ in range(n_ops))
        out[key] = complex(rng.standard_normal(), rng.standard_normal())
    return out


def random_rows(n_sites: int, count: int, seed: int, nq: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    bits = (rng.random((count, n_sites)) < 0.5).astype(np.uint8)
    return terms.unique_rows(terms.pack_sites(bits, nq))


def run_case(hmod, name, table_or_dict, kind, configs_i, psi_i, configs_j, counts, diag_configs, out_dir,
             exclude=None):
    if isinstance(table_or_dict, dict):
        ham = hmod.Hamiltonian(table_or_dict, kind=kind)
    else:
        ham = hmod.Hamiltonian(tuple(torch.as_tensor(x) for x in table_or_dict), kind=kind)
    ci = torch.from_numpy(configs_i)
    cj = torch.from_numpy(configs_j)
    pi = torch.from_numpy(psi_i)
    psi_j = ham.apply_within(ci, pi, cj).numpy()
    record = {
        "site": ham.site.numpy(), "kind": ham.kind.numpy(), "coef": ham.coef.numpy(),
        "particle_cut": np.int64(1 if kind == "fermi" else 2),
        "configs_i": configs_i, "psi_i": psi_i, "configs_j": configs_j, "psi_j": psi_j,
        "counts": np.asarray(counts, dtype=np.int64),
    }
    ex = None if exclude is None else torch.from_numpy(exclude)
    if exclude is not None:
        record["configs_exclude"] = exclude
    for k in counts:
        rel = ham.find_relative(ci, pi, int(k), ex).numpy()
        record[f"relative_{k}"] = rel
    diag = []
    one = torch.ones(1, dtype=torch.complex128)
    for r in range(diag_configs.shape[0]):
        c = torch.from_numpy(diag_configs[r:r + 1].copy())
        diag.append(ham.apply_within(c, one, c).numpy()[0])
    record["diag_configs"] = diag_configs
    record["diag"] = np.asarray(diag, dtype=np.complex128)
    path = out_dir / f"{name}.npz"
    np.savez_compressed(path, **record)
    print(f"{name}: T={record['site'].shape[0]} Ni={configs_i.shape[0]} Nj={configs_j.shape[0]} "
          f"relative={[record[f'relative_{k}'].shape[0] for k in counts]} -> {path.name}")


def make_bitspack(bmod, out_dir):
    rng = np.random.default_rng(5)
    record = {}
    for size, hi in ((1, 2), (2, 4), (4, 16), (8, 256)):
        for last in (16, 15, 14, 1000):
            x = rng.integers(0, hi, size=(3, last)).astype(np.uint8)
            packed = bmod.pack_int(torch.from_numpy(x), size).numpy()
            record[f"in_{size}_{last}"] = x
            record[f"packed_{size}_{last}"] = packed
    np.savez_compressed(out_dir / "bitspack.npz", **record)
    print("bitspack.npz")


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--reference", default=os.environ.get("QMB_REFERENCE", ""), required=False)
    args = parser.parse_args()
    if not args.reference:
        parser.error("--reference is required")
    hmod, bmod = load_reference(args.reference)
    out = HERE
    make_bitspack(bmod, out)

    # 1. 12 spin orbitals, 3 alpha + 3 beta: every determinant (400), real integrals
    s, k, c = terms.integral_terms(6, seed=11)
    dets = terms.all_determinants(6, 3, 3)
    psi = terms.random_psi(dets.shape[0], seed=12)
    sub = dets[np.random.default_rng(13).choice(dets.shape[0], 60, replace=False)]
    sub = terms.sort_rows(sub)
    psi_sub = terms.random_psi(sub.shape[0], seed=14)
    d = terms.table_to_dict(s, k, c)
    run_case(hmod, "ab_initio_6", d, "fermi", dets, psi, dets, [], dets[:64], out)
    run_case(hmod, "ab_initio_6_relative", d, "fermi", sub, psi_sub, dets, [1, 7, 50, 300, 100000], sub, out)

    # 2. 20 spin orbitals (n_qubytes 3), 4 alpha + 4 beta, rectangular sets, complex integrals
    s, k, c = terms.integral_terms(10, seed=21, complex_valued=True)
    dets_i = terms.random_determinants(10, 4, 4, 150, seed=22)
    dets_j = terms.unique_rows(np.concatenate([dets_i[::3], terms.random_determinants(10, 4, 4, 400, seed=23)]))
    psi_i = terms.random_psi(dets_i.shape[0], seed=24)
    run_case(hmod, "ab_initio_10_complex", (s, k, c), "fermi", dets_i, psi_i, dets_j, [1, 33, 500, 4000], dets_j[:40], out)

    # 3. arbitrary operator strings on 20 sites (n_qubytes 3), fermions and hard-core bosons
    rd = random_terms_dict(20, 400, seed=31)
    rows_i = random_rows(20, 300, seed=32, nq=3)
    rows_j = terms.unique_rows(np.concatenate([rows_i[::2], random_rows(20, 300, seed=33, nq=3)]))
    psi_r = terms.random_psi(rows_i.shape[0], seed=34)
    run_case(hmod, "random_terms_fermi", rd, "fermi", rows_i, psi_r, rows_j, [1, 10, 200, 5000], rows_j[:50], out)
    run_case(hmod, "random_terms_bose2", rd, "bose2", rows_i, psi_r, rows_j, [1, 10, 200, 5000], rows_j[:50], out)

    # 4. hard-core boson spin lattice 4x4 (16 sites, n_qubytes 2)
    isd = ising_dict(4, 4, x=0.7, z=-0.3, zz=1.1, yy=0.4)
    rows = random_rows(16, 500, seed=41, nq=2)
    psi_s = terms.random_psi(rows.shape[0], seed=42)
    run_case(hmod, "ising_4x4", isd, "bose2", rows, psi_s, rows, [], rows[:40], out)
    run_case(hmod, "ising_4x4_relative", isd, "bose2", rows[:60], psi_s[:60], rows, [5, 100, 1000], rows[:20], out,
             exclude=rows[30:200])

    # 5. Fermi-Hubbard 3x2 open lattice (12 sites), 3 alpha + 3 beta, every determinant
    hd = terms.hubbard_dict(3, 2, t=1.0, u=4.0)
    hdets = terms.all_determinants(6, 3, 3)
    hpsi = terms.random_psi(hdets.shape[0], seed=51)
    run_case(hmod, "hubbard_3x2", hd, "fermi", hdets, hpsi, hdets, [3, 40], hdets[:30], out)

    # 6. edge cases: duplicate target rows, empty sources
    dup_j = np.concatenate([dets[:20], dets[5:10], dets[30:40]])
    run_case(hmod, "edge_duplicates", d, "fermi", dets[:50], psi[:50], dup_j, [4], dets[:4], out)


if __name__ == "__main__":
    main()
