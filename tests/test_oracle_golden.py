"""Pin the CPU oracle against golden vectors produced by the reference's own Python code.

The vectors come from ``tests/golden/make_golden.py``: the Krylov fixture generator of the
reference's ``tests/test_krylov_block.rs`` and its ``pyhessref`` twin (``krylov_block``,
``RHessSCF``, ``UHessSCF``, the naive RI-JK response) run on seeded synthetic systems.
"""

import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import cphf, krylov, rijk, xc


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


# ---------------------------------------------------------------- XC response (bra form)
def _xc_golden(name):
    g = load_golden(name)
    nspin = int(g["nspin"])
    mocc = [g[f"mo_coeff{t}"][:, g[f"mo_occ{t}"] > 0] for t in range(nspin)]
    return g, nspin, mocc


def test_xc_rks_response_matches_reference_wrapper():
    """oracle/xc.py against pyhessref/nimatmul/rks.py:get_ks_response_bra_naive (its 2 bra mocc^T
    perturbed density, symmetrisation and v1 @ mocc; the stubbed NumInt gives the LDA fxc integral)."""
    g, _, mocc = _xc_golden("xc_rks_nao30_seed3.npz")
    got = xc.rks_response_bra(g["ao"], g["weights"], g["fxc"], g["bra0"], mocc[0])
    assert rel_err(got, g["resp0"]) < 1e-12
    got_b = xc.rks_response_bra(g["ao"], g["weights"], g["fxc"], g["bra0"], mocc[0], nbatch=3)
    assert rel_err(got_b, g["resp0"]) < 1e-12


def test_xc_uks_response_matches_reference_wrapper():
    """oracle/xc.py against pyhessref/nimatmul/uks.py:get_uks_response_bra_naive (per-spin bra mocc^T
    densities, spin-coupled fxc, v1_t @ mocc_t)."""
    g, _, mocc = _xc_golden("xc_uks_nao28_seed4.npz")
    got = xc.uks_response_bra(g["ao"], g["weights"], g["fxc"], [g["bra0"], g["bra1"]], mocc)
    for t in range(2):
        assert rel_err(got[t], g[f"resp{t}"]) < 1e-12


# ---------------------------------------------------------------- j2c decomposition
def test_j2c_recoverable_reference_case():
    """pure_decompose.rs:333-356 (test_check_recoverable): U^T U reproduces the 3 x 3 metric."""
    from oracle import decompose
    j2c = np.array([[10.0, 1.0, 2.0], [1.0, 20.0, 3.0], [2.0, 3.0, 30.0]])
    U, fallback = decompose.decomp_j2c_cd(j2c, None)
    assert not fallback and np.allclose(U.T @ U, j2c, rtol=1e-12, atol=1e-12)
    assert np.allclose(np.tril(U, -1), 0.0)
    U2, fallback2 = decompose.decomp_j2c_cd(j2c, 1e-14)
    assert not fallback2 and np.array_equal(U, U2)


def test_j2c_eigenvalue_fallback_and_solve():
    """The clamped-eigenvalue fallback (pure_decompose.rs:44-51) on an indefinite metric, and
    cderi = j3c U^-1 (pure_decompose.rs:205-252)."""
    from oracle import decompose
    rng = np.random.default_rng(5)
    q, _ = np.linalg.qr(rng.standard_normal((30, 30)))
    e = np.linspace(-0.2, 3.0, 30)
    j2c = (q * e) @ q.T
    U, fallback = decompose.decomp_j2c_cd(j2c, 1e-3)
    assert fallback
    assert np.allclose(U.T @ U, (q * np.maximum(e, 1e-3)) @ q.T, atol=1e-12)
    with pytest.raises(np.linalg.LinAlgError):
        decompose.decomp_j2c_cd(j2c, None)
    j3c = rng.standard_normal((50, 30))
    cd = decompose.solve_by_j2c_right(j3c, U)
    assert np.allclose(cd @ U, j3c, atol=1e-12)


# ---------------------------------------------------------------- CPHF right-hand side
@pytest.mark.parametrize("name", ["rhs_rhf_nao22_seed5.npz", "rhs_uhf_nao22_seed6.npz"])
def test_compute_dimless_cphf_rhs_matches_reference(name):
    """oracle/cphf.py:compute_dimless_cphf_rhs against pyhessref's RHessSCF / UHessSCF
    compute_dimensionless_cphf_rhs (rscf.rs:104-182, uscf.rs:78-173) on the same derivatives."""
    g = load_golden(name)
    for t in range(int(g["nspin"])):
        rhs, f1, s1 = cphf.compute_dimless_cphf_rhs(g[f"mo_coeff{t}"], g[f"mo_occ{t}"], g[f"mo_energy{t}"],
                                                    g["f1ao_core"], g[f"f1bra_el{t}"], g["s1ao"])
        assert rel_err(rhs, g[f"rhs{t}"]) < 1e-13
        assert rel_err(f1, g[f"f1mo{t}"]) < 1e-13
        assert rel_err(s1, g[f"s1mo{t}"]) < 1e-13
