"""The host-side term builders: dictionary preparation, ordering and synthetic generators."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import golden
from qmb_gb300 import terms


def _fixture_dict(case):
    """The dictionary the fixture script handed to the reference, rebuilt in the same order."""
    import importlib.util
    import os

    from conftest import GOLDEN

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    if case == "ab_initio_6":
        return terms.table_to_dict(*terms.integral_terms(6, seed=11))
    if case == "random_terms_fermi":
        return mg.random_terms_dict(20, 400, seed=31)
    if case == "ising_4x4":
        return mg.ising_dict(4, 4, x=0.7, z=-0.3, zz=1.1, yy=0.4)
    return terms.hubbard_dict(3, 2, t=1.0, u=4.0)


@pytest.mark.parametrize("case", ["ab_initio_6", "random_terms_fermi", "ising_4x4", "hubbard_3x2"])
def test_prepare_and_sort_match_reference_order(case):
    """Hamiltonian(dict) tables equal the reference's (empty slots excepted: the reference leaves them uninitialised)."""
    g = golden(case)
    site, kind, coef = terms.prepare(_fixture_dict(case))
    site, kind, coef = terms.sort_terms(site, kind, coef)
    live = g["kind"] != 2
    assert np.array_equal(kind.numpy(), g["kind"])
    assert np.array_equal(site.numpy()[live], g["site"][live])
    assert np.array_equal(coef.numpy(), g["coef"])


def test_term_count_formula():
    for n in (2, 3, 6):
        site, kind, coef = terms.integral_terms(n, seed=1)
        assert site.shape[0] == terms.n_integral_terms(n)
    assert terms.n_integral_terms(6) == 1819
    assert terms.n_integral_terms(14) == 55371
    assert terms.n_integral_terms(26) == 669579
    assert terms.n_integral_terms(38) == 3076443


def test_normal_order_of_two_body_terms():
    site, kind, coef = terms.integral_terms(4, seed=3)
    two = np.all(kind == np.array([1, 1, 0, 0], dtype=np.uint8), axis=1)
    assert np.all(site[two, 0] > site[two, 1])
    assert np.all(site[two, 2] > site[two, 3])
    # spin is conserved: alpha count of created == alpha count of annihilated
    par = site[two] % 2
    assert np.array_equal(par[:, 0] + par[:, 1], par[:, 2] + par[:, 3])


def test_random_determinants_are_sorted_unique_with_fixed_counts():
    rows = terms.random_determinants(14, 5, 5, 5000, seed=7)
    assert rows.shape == (5000, 4)
    assert np.array_equal(terms.unique_rows(rows), rows)
    bits = np.unpackbits(rows, axis=1, bitorder="little")
    assert np.all(bits[:, 0::2].sum(axis=1) == 5)
    assert np.all(bits[:, 1::2].sum(axis=1) == 5)


def test_hubbard_term_count():
    d = terms.hubbard_dict(8, 8, 1.0, 4.0)
    # 64 on-site terms + 4 per bond per spin... 2 directions x 2 spins x 112 bonds
    assert len(d) == 64 + 4 * 112
    site, kind, coef = terms.prepare(d)
    assert site.dtype == torch.int16 and kind.dtype == torch.uint8 and coef.dtype == torch.float64


def test_fcidump_round_trip(tmp_path):
    e0, h, eri = terms.random_integrals(5, seed=9)
    path = tmp_path / "toy.FCIDUMP"
    terms.write_fcidump(str(path), e0, h, eri, n_electron=6)
    n_orbit, n_electron, ms2, site, kind, coef = terms.read_fcidump(str(path))
    assert (n_orbit, n_electron, ms2) == (5, 6, 0)
    ref = terms.sort_terms(*(torch.from_numpy(x) for x in terms.terms_from_integrals(e0, h, eri)))
    assert torch.equal(kind, ref[1])
    live = ref[1] != 2
    assert torch.equal(site[live], ref[0][live])
    torch.testing.assert_close(coef, ref[2], rtol=1e-15, atol=1e-15)


def test_fcidump_gzip_and_bad_line(tmp_path):
    import gzip

    e0, h, eri = terms.random_integrals(3, seed=4)
    plain = tmp_path / "a.FCIDUMP"
    terms.write_fcidump(str(plain), e0, h, eri, n_electron=2)
    gz = tmp_path / "a.FCIDUMP.gz"
    with open(plain, "rb") as src, gzip.open(gz, "wb") as dst:
        dst.write(src.read())
    assert terms.read_fcidump(str(gz))[0] == 3
    bad = tmp_path / "bad.FCIDUMP"
    bad.write_text(" &FCI NORB=2,NELEC=2,MS2=0,\n &END\n 1.0 1 2 1 0\n")
    with pytest.raises(ValueError):
        terms.read_fcidump(str(bad))


def test_hamiltonian_rejects_bad_inputs_on_the_host():
    from qmb_gb300 import Hamiltonian

    site, kind, coef = terms.integral_hamiltonian_tables(3, seed=1)
    ham = Hamiltonian((site, kind, coef), kind="fermi")
    rows = torch.from_numpy(terms.all_determinants(3, 1, 1))
    psi = torch.ones(rows.shape[0], dtype=torch.complex128)
    with pytest.raises(RuntimeError, match="uint8"):
        ham.apply_within(rows.to(torch.int32), psi, rows)
    with pytest.raises(RuntimeError, match="2D"):
        ham.diagonal_term(rows.flatten())
    # the engine has no CPU path: CPU tensors are refused, not computed some other way
    with pytest.raises(RuntimeError, match="CUDA"):
        ham.apply_within(rows, psi, rows)
    with pytest.raises(ValueError):
        Hamiltonian((site, kind, coef), kind="bose3")
