"""Pin the CPU oracle against golden vectors produced by the reference's own Python code.

The vectors come from ``tests/golden/make_golden.py``: the Krylov fixture generator of the
reference's ``tests/test_krylov_block.rs`` and its ``pyhessref`` twin (``krylov_block``,
``RHessSCF``, ``UHessSCF``, the naive RI-JK response) run on seeded synthetic systems.
"""

import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import cphf, krylov, rijk


@pytest.fixture(scope="module")
def kfix():
    z = load_golden("krylov_fixture.npz")
    # pyhessref stores RHS as rows; the col-major API takes [n, nset] (test_krylov_block.rs:14-16)
    return z["A"], z["b"].T.copy(), z["x_ref"].T.copy(), z


def test_krylov_small_deterministic(kfix):
    """tests/test_krylov_block.rs:7-47 on the oracle."""
    A, b, x_ref, z = kfix
    st = {}
    x = krylov.krylov_block(lambda v: A @ v, b, None, 1e-10, 30, 6, 1e-13, stats=st)
    assert np.allclose(x, x_ref, rtol=1e-6, atol=1e-8)
    assert np.abs(x + A @ x - b).max() < 1e-6
    # the reference Python twin on the same fixture
    assert np.abs(x - z["x_ms6"].T).max() < 1e-9
    assert st["aop_calls"] == int(z["calls_ms6"])


def test_krylov_with_restart(kfix):
    """tests/test_krylov_block.rs:49-81 (max_space = 3 forces hard restarts)."""
    A, b, x_ref, z = kfix
    st = {}
    x = krylov.krylov_block(lambda v: A @ v, b, None, 1e-10, 60, 3, 1e-13, stats=st)
    assert st["restarts"] >= 1
    assert np.allclose(x, x_ref, rtol=1e-5, atol=1e-6)
    assert np.abs(x + A @ x - b).max() < 1e-5


def test_krylov_panics_on_nonconvergence(kfix):
    """tests/test_krylov_block.rs:83-97: starving max_cycle must fail, not return silently."""
    A, b, _, _ = kfix
    with pytest.raises(krylov.KrylovNotConverged, match="failed to converge"):
        krylov.krylov_block(lambda v: A @ v, b, None, 1e-10, 2, 14, 1e-13)


def test_krylov_x0_already_solved(kfix):
    A, b, x_ref, _ = kfix
    x = krylov.krylov_block(lambda v: A @ v, b, x_ref, 1e-10, 30, 6, 1e-13)
    assert np.allclose(x, x_ref, rtol=1e-8, atol=1e-10)


@pytest.fixture(scope="module")
def rg():
    return load_golden("rhf_nao24_seed1.npz")


def test_rijk_separated_matches_reference_naive(rg):
    """hess_r.rs:82-186 restated vs the reference's naive RI-JK response (pyhessref)."""
    resp = rijk.rhf_response_bra(rg["cderi"], rg["mo_coeff"], rg["mo_occ"], rg["bra_probe"],
                                 float(rg["scale_j"]), float(rg["scale_k"]))
    assert rel_err(resp, rg["resp_probe"]) < 1e-12


def test_rijk_naive_restatement_matches_reference(rg):
    resp = rijk.rhf_response_bra_naive(rg["cderi"], rg["mo_coeff"], rg["mo_occ"], rg["bra_probe"],
                                       float(rg["scale_j"]), float(rg["scale_k"]))
    assert rel_err(resp, rg["resp_probe"]) < 1e-12


def _rhf_driver(g, tol):
    C, occ, e = g["mo_coeff"], g["mo_occ"], g["mo_energy"]
    sj, sk = float(g["scale_j"]), float(g["scale_k"])
    plug = lambda bra: rijk.rhf_response_bra(g["cderi"], C, occ, bra, sj, sk)  # noqa: E731
    return cphf.RHF(C, occ, e, [plug], int(g["natm"]),
                    config=dict(cphf_tol=tol, cphf_max_cycle=30, cphf_max_space=14))


def test_cphf_rhf_matches_reference_driver(rg):
    """RHessSCF solve/finalize/get_cphf_hess (pyhessref) vs the oracle's rscf.rs restatement."""
    drv = _rhf_driver(rg, 1e-10)
    mo1 = drv.solve_dimless_cphf(rg["rhs"])
    nocc = drv.nocc
    # vir block: both solve the same system to the same tolerance
    assert rel_err(mo1[nocc:], rg["mo1_solved"][nocc:]) < 1e-8
    # occ block: the Python twin pins mo1[oo] = rhs[oo] (hess_scf_restricted.py:239-245); Rust does not
    assert np.abs(mo1[:nocc] - rg["rhs"][:nocc]).max() < 1e-8
    mo1f, mo_e1 = drv.finalize_cphf(rg["f1mo"], rg["s1mo"], rg["mo1_solved"])
    assert rel_err(mo1f, rg["mo1"]) < 1e-11
    assert rel_err(mo_e1, rg["mo_e1"]) < 1e-11
    de = drv.get_cphf_hess(rg["f1mo"], rg["s1mo"], rg["mo1"], rg["mo_e1"])
    assert rel_err(de, rg["de_cphf"]) < 1e-12


def test_cphf_uhf_matches_reference_driver():
    ug = load_golden("uhf_nao20_seed2.npz")
    C = [ug["mo_coeff0"], ug["mo_coeff1"]]
    occ = [ug["mo_occ0"], ug["mo_occ1"]]
    e = [ug["mo_energy0"], ug["mo_energy1"]]
    sj, sk = float(ug["scale_j"]), float(ug["scale_k"])
    plug = lambda bra: rijk.uhf_response_bra(ug["cderi"], C, occ, bra, sj, sk)  # noqa: E731
    drv = cphf.UHF(C, occ, e, [plug], int(ug["natm"]), config=dict(cphf_tol=1e-10, cphf_max_cycle=30))
    mo1 = drv.solve_dimless_cphf([ug["rhs0"], ug["rhs1"]])
    for s in range(2):
        no = drv.nocc[s]
        assert rel_err(mo1[s][no:], ug[f"mo1_solved{s}"][no:]) < 1e-8
    f1 = [ug["f1mo0"], ug["f1mo1"]]
    s1 = [ug["s1mo0"], ug["s1mo1"]]
    mo1f, mo_e1 = drv.finalize_cphf(f1, s1, [ug["mo1_solved0"], ug["mo1_solved1"]])
    for s in range(2):
        assert rel_err(mo1f[s], ug[f"mo1{s}"]) < 1e-11
        assert rel_err(mo_e1[s], ug[f"mo_e1{s}"]) < 1e-11
    de = drv.get_cphf_hess(f1, s1, [ug["mo10"], ug["mo11"]], [ug["mo_e10"], ug["mo_e11"]])
    assert rel_err(de, ug["de_cphf"]) < 1e-12


def test_cphf_nonconvergence_raises(rg):
    drv = _rhf_driver(rg, 1e-10)
    drv.config["cphf_max_cycle"] = 1
    with pytest.raises(krylov.KrylovNotConverged):
        drv.solve_dimless_cphf(rg["rhs"])
