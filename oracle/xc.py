"""XC (fxc) response in bra form, RHO (LDA) branch -- oracle restatement (test infrastructure only).

Restates the reference's matrix-multiply numerical integration for the CPKS
response:

* :func:`rks_response_bra` -- ``get_rks_response_bra_batched`` /
  ``get_rks_response_bra`` (``src/numint_matmul/hess_rks.rs:570-605, 752-797``):
  ``rho1`` from ``get_rho_from_one_bra_mult_ket_with_output``
  (``pure_eval_rho.rs:216-334``, RHO terms 283-287), the weighted kernel and
  ``contract_ao_wv_bra`` (``pure_xcpot.rs:285-352, 370-465``), times 4.0
  (``hess_rks.rs:603``).
* :func:`uks_response_bra` -- ``get_uks_response_bra`` (``hess_uks.rs:390-441``)
  with ``uks_fxc_pot_with_eff_bra_trans_with_output`` (``pure_xcpot.rs:921-1028``),
  times 2.0 (``hess_uks.rs:438-439``).
* :func:`rks_response_bra_dm_form` -- the density-matrix form of the same
  kernel (``rho1 = phi D1 phi``, ``V = phi^T (w f rho1) phi``, the PySCF-based
  naive twin ``pyhessref/nimatmul/rks.py:713-782``), an independent cross-check.

Grid data: ``ao [ngrids, nao]`` (AO values, derivative order 0), ``weights
[ngrids]``, ``fxc_eff [ngrids, 1, 1]`` (RKS) or ``[ngrids, 1, 2, 1, 2]`` (UKS).
Grid batches of ``nbatch`` points are summed as in ``hess_rks.rs:766-776``.
"""

import numpy as np


def _batches(ngrids, nbatch):
    nbatch = ngrids if not nbatch else nbatch
    for start in range(0, ngrids, nbatch):
        yield start, min(start + nbatch, ngrids)


def rks_response_bra(ao, weights, fxc_eff, bra, mocc, nbatch=None):
    """RKS XC response, bra ``[nao, nocc, nprop]`` -> same shape."""
    bra = np.asarray(bra)
    shape = bra.shape
    nao, nocc = mocc.shape
    bra = bra.reshape(nao, nocc, -1)
    nprop = bra.shape[2]
    resp = np.zeros((nao, nocc, nprop))
    fxc = np.asarray(fxc_eff).reshape(len(weights), 1, 1)
    for g0, g1 in _batches(len(weights), nbatch):
        phi = ao[g0:g1]
        ao_bra = phi @ mocc                                       # pure_xcpot.rs:403-406
        # rho1[g, a] = sum_i (phi mocc)[g,i] (phi bra_a)[g,i]      pure_eval_rho.rs:283-287
        ket = (phi @ bra.reshape(nao, nocc * nprop)).reshape(g1 - g0, nocc, nprop)
        rho1 = np.einsum("gi,gia->ga", ao_bra, ket)
        # wv[g, a] = w_g sum_x fxc[g,x,y] rho1[g,x,a]             pure_xcpot.rs:409, 443
        wv = weights[g0:g1, None] * fxc[g0:g1, 0, 0][:, None] * rho1
        # out[:, :, a] += phi^T (wv[:, a] * ao_bra)                pure_xcpot.rs:331-333
        for a in range(nprop):
            resp[:, :, a] += phi.T @ (wv[:, a:a + 1] * ao_bra)
    return (4.0 * resp).reshape(shape)


def uks_response_bra(ao, weights, fxc_eff, bra, mocc, nbatch=None):
    """UKS XC response; ``bra`` and ``mocc`` are two-spin lists."""
    nao = mocc[0].shape[0]
    shapes = [np.asarray(b).shape for b in bra]
    bra = [np.asarray(bra[s]).reshape(nao, mocc[s].shape[1], -1) for s in range(2)]
    nprop = bra[0].shape[2]
    ng = len(weights)
    fxc = np.asarray(fxc_eff).reshape(ng, 1, 2, 1, 2)
    resp = [np.zeros((nao, mocc[s].shape[1], nprop)) for s in range(2)]
    for g0, g1 in _batches(ng, nbatch):
        phi = ao[g0:g1]
        ao_bra = [phi @ mocc[s] for s in range(2)]
        rho1 = np.zeros((g1 - g0, 2, nprop))
        for s in range(2):
            no = mocc[s].shape[1]
            ket = (phi @ bra[s].reshape(nao, no * nprop)).reshape(g1 - g0, no, nprop)
            rho1[:, s, :] = np.einsum("gi,gia->ga", ao_bra[s], ket)
        for s in range(2):
            # pure_xcpot.rs:1006 -- contract the inner (var, spin) pair for output spin s
            wv = weights[g0:g1, None] * np.einsum("gt,gta->ga", fxc[g0:g1, 0, :, 0, s], rho1)
            for a in range(nprop):
                resp[s][:, :, a] += phi.T @ (wv[:, a:a + 1] * ao_bra[s])
    return [(2.0 * resp[s]).reshape(shapes[s]) for s in range(2)]


def rks_response_bra_dm_form(ao, weights, fxc_eff, bra, mocc):
    """Density-matrix form: ``dm1 = 2 (bra mocc^T + h.c.)``, ``v1 = phi^T (w f rho[dm1]) phi``, ``v1 mocc``."""
    bra = np.asarray(bra)
    shape = bra.shape
    nao, nocc = mocc.shape
    bra = bra.reshape(nao, nocc, -1)
    fxc = np.asarray(fxc_eff).reshape(-1)
    out = np.zeros_like(bra)
    for a in range(bra.shape[2]):
        dm1 = 2.0 * bra[:, :, a] @ mocc.T
        dm1 = dm1 + dm1.T
        rho = np.einsum("gu,uv,gv->g", ao, dm1, ao, optimize=True)
        v1 = ao.T @ ((weights * fxc * rho)[:, None] * ao)
        out[:, :, a] = v1 @ mocc
    return out.reshape(shape)
