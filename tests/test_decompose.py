"""FP64 two-centre metric decomposition and cderi build on the GPU against the oracle
(numpy / LAPACK restatement of src/ri_jk/pure_decompose.rs): Cholesky with the eigenvalue
fallback (decomp_j2c_cd, pure_decompose.rs:29-57) and cderi = j3c U^-1 (solve_by_j2c,
pure_decompose.rs:205-252; generate_cderi_with_decomp, src/ri_jk/hess_r.rs:1725-1735)."""

import numpy as np
import pytest

from conftest import rel_err
from cphf_gb300 import Context, CphfError, synth
from oracle import decompose, rijk

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("naux,seed", [(3, 0), (64, 1), (257, 2), (1000, 3)])
def test_j2c_cholesky_matches_lapack(naux, seed):
    if naux == 3:
        j2c = np.asfortranarray([[10.0, 1.0, 2.0], [1.0, 20.0, 3.0], [2.0, 3.0, 30.0]])
    else:
        j2c = decompose.synthetic_metric(naux, seed=seed, cond=1e6)
    ctx = Context()
    U, info = ctx.j2c_decompose(j2c, 1e-14)
    U_ref, fb = decompose.decomp_j2c_cd(j2c, 1e-14)
    assert not fb and info["eig_fallback"] == 0
    assert rel_err(U, U_ref) < 1e-12
    assert np.all(np.tril(U, -1) == 0.0)
    assert abs(info["min_diag"] - np.diag(U_ref).min()) <= 1e-12 * np.diag(U_ref).max()


def test_j2c_failure_without_threshold_is_an_error():
    q, _ = np.linalg.qr(np.random.default_rng(4).standard_normal((80, 80)))
    j2c = np.asfortranarray((q * np.linspace(-0.5, 2.0, 80)) @ q.T)
    with pytest.raises(CphfError) as e:
        Context().j2c_decompose(j2c, None)
    assert e.value.status == 3


@pytest.mark.parametrize("naux", [40, 129])
def test_j2c_eigenvalue_fallback(naux):
    """Indefinite metric: the eigenvalues are clamped at the threshold and the rebuilt matrix
    is factored (one-sided Jacobi eigensolver on the GPU)."""
    rng = np.random.default_rng(naux)
    q, _ = np.linalg.qr(rng.standard_normal((naux, naux)))
    e = np.concatenate([[-0.3, -0.05, 1e-9], np.geomspace(1e-2, 5.0, naux - 3)])
    j2c = np.asfortranarray((q * e) @ q.T)
    thr = 1e-3
    U, info = Context().j2c_decompose(j2c, thr)
    U_ref, fb = decompose.decomp_j2c_cd(j2c, thr)
    assert fb and info["eig_fallback"] == 1 and info["jacobi_sweeps"] >= 1
    target = (q * np.maximum(e, thr)) @ q.T
    assert rel_err(U.T @ U, target) < 1e-11
    assert rel_err(U, U_ref) < 1e-9


def test_j2c_small_diagonal_triggers_fallback():
    """Cholesky succeeds but min diag(U) <= threshold (pure_decompose.rs:36-41)."""
    j2c = decompose.synthetic_metric(50, seed=7, cond=1e12)
    U, info = Context().j2c_decompose(j2c, 1e-4)
    U_ref, fb = decompose.decomp_j2c_cd(j2c, 1e-4)
    assert fb and info["eig_fallback"] == 1
    assert rel_err(U.T @ U, U_ref.T @ U_ref) < 1e-11


@pytest.mark.parametrize("dims,seed", [(dict(nao=40, naux=130, nocc=(6,), natm=3, decay=8.0), 5),
                                       ("rhf_nao600", 0)])
def test_set_j3c_builds_cderi(dims, seed):
    """j3c = B U^T from a synthetic B and an SPD metric: the GPU recovers B = j3c U^-1 (1e-12
    relative to the oracle's triangular solve for a metric of condition number 1e3; two
    triangular solves in different operation orders differ by ~cond x 1e-16) and the plugin built
    from it answers like the one built from B.  The second case is the 180-RHS workload's size
    (nao 600, naux 2000)."""
    s = synth.make_system(dims, seed=seed)
    j2c = decompose.synthetic_metric(s.naux, seed=seed + 1, cond=1e3)
    U_ref, _ = decompose.decomp_j2c_cd(j2c, 1e-14)
    j3c = np.asfortranarray(s.cderi @ U_ref)
    cd_ref = decompose.solve_by_j2c_right(j3c, U_ref)
    ctx = Context()
    info = ctx.set_j3c(j3c, j2c, s.scale_j, s.scale_k)
    assert info["eig_fallback"] == 0
    cd = ctx.get_cderi()
    assert rel_err(cd, cd_ref) < 1e-12
    assert rel_err(cd, s.cderi) < 1e-9     # recovers the generating B (rounding of j3c, cond 1e5)
    if s.nao <= 100:
        ctx.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])
        bra = np.random.default_rng(9).standard_normal((s.nao, s.nocc[0], 3))
        ref = rijk.rhf_response_bra(cd_ref, s.mo_coeff[0], s.mo_occ[0], bra, s.scale_j, s.scale_k)
        assert rel_err(ctx.get_response_bra(bra), ref) < 1e-12


def test_set_j3c_ill_conditioned_metric():
    """Condition number 1e6: the GPU cderi and the oracle's agree to the triangular solve's
    forward-error scale (cond x 1e-16, with a factor 10 of margin)."""
    s = synth.make_system(dict(nao=36, naux=200, nocc=(5,), natm=3, decay=8.0), seed=11)
    cond = 1e6
    j2c = decompose.synthetic_metric(s.naux, seed=12, cond=cond)
    U_ref, _ = decompose.decomp_j2c_cd(j2c, 1e-14)
    j3c = np.asfortranarray(s.cderi @ U_ref)
    cd_ref = decompose.solve_by_j2c_right(j3c, U_ref)
    ctx = Context()
    ctx.set_j3c(j3c, j2c, s.scale_j, s.scale_k)
    assert rel_err(ctx.get_cderi(), cd_ref) < 10 * cond * 1e-16
