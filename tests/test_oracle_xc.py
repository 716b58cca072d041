"""The XC oracle (bra form of the reference's numint response) against the density-matrix form."""

import numpy as np

from conftest import rel_err
from cphf_gb300 import synth
from oracle import xc


def _small_grid(nspin, seed=0):
    dims = dict(nao=30, naux=60, nocc=(6,) if nspin == 1 else (6, 5), natm=3, decay=6.0, grid=True,
                points=(150, 260), window=12)
    return synth.make_system(dims, seed=seed)


def test_rks_bra_form_equals_dm_form():
    s = _small_grid(1)
    g = s.grid
    mocc = s.mo_coeff[0][:, :s.nocc[0]]
    bra = np.random.default_rng(1).standard_normal((s.nao, s.nocc[0], 4))
    r1 = xc.rks_response_bra(g.ao, g.weights, g.fxc, bra, mocc)
    r2 = xc.rks_response_bra_dm_form(g.ao, g.weights, g.fxc, bra, mocc)
    assert rel_err(r1, r2) < 1e-12


def test_rks_grid_batching_is_a_sum():
    s = _small_grid(1)
    g = s.grid
    mocc = s.mo_coeff[0][:, :s.nocc[0]]
    bra = np.random.default_rng(2).standard_normal((s.nao, s.nocc[0], 3))
    r1 = xc.rks_response_bra(g.ao, g.weights, g.fxc, bra, mocc)
    r2 = xc.rks_response_bra(g.ao, g.weights, g.fxc, bra, mocc, nbatch=97)
    assert rel_err(r1, r2) < 1e-13


def test_uks_reduces_to_rks_for_equal_spins():
    """Equal spins with fxc_ss' = f/2 everywhere give RKS/2 per spin (closed-shell factor 4 vs 2)."""
    s = _small_grid(1)
    g = s.grid
    mocc = s.mo_coeff[0][:, :s.nocc[0]]
    bra = np.random.default_rng(3).standard_normal((s.nao, s.nocc[0], 2))
    f2 = np.zeros((len(g.weights), 2, 2), order="F")
    f2[:] = 0.5 * g.fxc[:, None, None]
    ru = xc.uks_response_bra(g.ao, g.weights, f2, [bra, bra], [mocc, mocc])
    rr = xc.rks_response_bra(g.ao, g.weights, g.fxc, bra, mocc)
    assert rel_err(ru[0], 0.5 * rr) < 1e-12
    assert rel_err(ru[1], 0.5 * rr) < 1e-12


def test_grid_generator_block_sparsity():
    s = _small_grid(2)
    g = s.grid
    assert g.fxc.shape == (len(g.weights), 2, 2)
    assert np.all(g.weights > 0) and np.all(g.weights <= 1e-2)
    ao_per_atm = s.nao // s.natm
    for A in range(s.natm):
        blk = g.ao[g.atom_offsets[A]:g.atom_offsets[A + 1]]
        nz = np.nonzero(np.abs(blk).sum(axis=0))[0]
        lo, hi = A * ao_per_atm, (A + 1) * ao_per_atm - 1
        assert nz.min() >= max(0, lo - g.window) and nz.max() <= min(s.nao - 1, hi + g.window)


def test_mgga_bra_form_equals_dm_form_and_lda():
    """SIGMA / TAU branches (pure_eval_rho.rs:289-316, pure_xcpot.rs:335-351) of the bra form
    against the independent density-matrix form; the RHO case of the general function against
    the LDA one."""
    s = _small_grid(1)
    g = s.grid
    mocc = s.mo_coeff[0][:, :s.nocc[0]]
    bra = np.random.default_rng(5).standard_normal((s.nao, s.nocc[0], 3))
    for den in ("sigma", "tau"):
        ao, fxc = synth.make_mgga_grid(g, den, seed=6)
        r1 = xc.rks_response_bra_mgga(ao, g.weights, fxc, bra, mocc, den, nbatch=97)
        r2 = xc.rks_response_bra_mgga_dm_form(ao, g.weights, fxc, bra, mocc, den)
        assert rel_err(r1, r2) < 1e-12
    r0 = xc.rks_response_bra_mgga(g.ao[:, :, None], g.weights, g.fxc, bra, mocc, "rho")
    assert rel_err(r0, xc.rks_response_bra(g.ao, g.weights, g.fxc, bra, mocc)) < 1e-13


def test_mgga_uks_reduces_to_rks_for_equal_spins():
    """UKS with identical spins and the kernel f[x,s,y,t] = f_RKS[x,y] for every spin pair: each
    output spin sees wv = 2 f rho1, so x2 (hess_uks) reproduces the RKS response (x4, hess_rks)."""
    s = _small_grid(1)
    g = s.grid
    mocc = s.mo_coeff[0][:, :s.nocc[0]]
    bra = np.random.default_rng(7).standard_normal((s.nao, s.nocc[0], 2))
    ao, fr = synth.make_mgga_grid(g, "sigma", seed=8)
    ng, nv = fr.shape[0], fr.shape[1]
    fu = np.zeros((ng, nv, 2, nv, 2))
    for si in range(2):
        for so in range(2):
            fu[:, :, si, :, so] = fr
    ru = xc.uks_response_bra_mgga(ao, g.weights, fu, [bra, bra], [mocc, mocc], "sigma")
    rr = xc.rks_response_bra_mgga(ao, g.weights, fr, bra, mocc, "sigma")
    assert rel_err(ru[0], rr) < 1e-12 and rel_err(ru[1], rr) < 1e-12
