"""Synthetic workload generator: layouts, the closure of rhs/f1mo/s1mo, and the operator scale."""

import numpy as np

from cphf_gb300 import synth
from oracle import cphf, rijk


def test_layouts_and_closure():
    s = synth.make_system("rhf_nao24", seed=3)
    nao, naux = s.nao, s.naux
    assert s.cderi.shape == (nao * (nao + 1) // 2, naux) and s.cderi.flags.f_contiguous
    C = s.mo_coeff[0]
    assert np.allclose(C.T @ C, np.eye(nao), atol=1e-12)
    e = s.mo_energy[0]
    no = s.nocc[0]
    assert np.all(e[:no] < -0.29) and np.all(e[no:] > 0.049)
    e_ai = e[no:, None] - e[None, :no]
    b1 = s.f1mo[0] - s.s1mo[0] * e[None, :no, None, None]
    # rhs = -(f1mo - s1mo eocc)[vir] / e_ai ; rhs[occ] = -0.5 s1mo[occ]   (rscf.rs:174-177)
    assert np.allclose(s.rhs[0][no:], -b1[no:] / e_ai[:, :, None, None], atol=1e-14)
    assert np.allclose(s.rhs[0][:no], -0.5 * s.s1mo[0][:no])


def test_operator_scale_is_bounded():
    """The dimensionless operator's spectral radius is about 0.5 by construction."""
    s = synth.make_system("rhf_nao24", seed=5)
    C, occ, e = s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0]
    plug = lambda bra: rijk.rhf_response_bra(s.cderi, C, occ, bra, s.scale_j, s.scale_k)  # noqa: E731
    drv = cphf.RHF(C, occ, e, [plug], s.natm)
    no, nmo = drv.nocc, drv.nmo
    n = nmo * no
    # dense dimensionless operator restricted to the vir-occ block
    cols = []
    for k in range(n):
        v = np.zeros(n)
        v[k] = 1.0
        cols.append(drv.response_dimless_cphf(v.reshape(nmo, no, 1, order="F")).reshape(n, order="F"))
    A = np.array(cols).T
    vo = np.array([p >= no for i in range(no) for p in range(nmo)])
    rho = np.abs(np.linalg.eigvals(A[np.ix_(vo, vo)])).max()
    assert 0.2 < rho <= 0.55


def test_seed_determinism():
    a = synth.make_system("rhf_nao24", seed=11)
    b = synth.make_system("rhf_nao24", seed=11)
    assert np.array_equal(a.cderi, b.cderi) and np.array_equal(a.rhs[0], b.rhs[0])
