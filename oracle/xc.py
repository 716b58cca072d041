"""XC (fxc) response in bra form, RHO (LDA), SIGMA (GGA) and TAU (meta-GGA) branches -- oracle
restatement (test infrastructure only).

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

* :func:`rks_response_bra_mgga` / :func:`uks_response_bra_mgga` -- the same for every density
  type: rho1's SIGMA and TAU terms (``pure_eval_rho.rs:289-316``) and ``contract_ao_wv_bra``'s
  (``pure_xcpot.rs:335-351``), with ``ao [ngrids, nao, ncomp]`` (value and gradient) and
  ``fxc_eff [ngrids, nvar, nvar]`` / ``[ngrids, nvar, 2, nvar, 2]``;
  :func:`rks_response_bra_mgga_dm_form` is its independent density-matrix cross-check.

Grid data (LDA functions): ``ao [ngrids, nao]`` (AO values, derivative order 0), ``weights
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


# ---------------------------------------------------------------- GGA / meta-GGA (SIGMA, TAU)
NVAR = {"rho": 1, "sigma": 4, "tau": 5}   # XCDenType::num_nvar (src/xceff/flags.rs:33-40)


def _rho1_mgga(aob, ket, den):
    """rho1[g, x, a] of ``get_rho_from_one_bra_mult_ket_with_output`` (pure_eval_rho.rs:283-316):
    aob[c] = ao_c mocc [g, i], ket[c] = ao_c bra_a [g, i, a], c = 0 (value), 1-3 (gradient)."""
    ng, nprop = ket[0].shape[0], ket[0].shape[2]
    rho = np.zeros((ng, NVAR[den], nprop))
    rho[:, 0] = np.einsum("gi,gia->ga", aob[0], ket[0])                       # 283-287
    if den in ("sigma", "tau"):
        for t in range(1, 4):                                                 # 289-296
            rho[:, t] = np.einsum("gi,gia->ga", aob[0], ket[t]) + np.einsum("gi,gia->ga", aob[t], ket[0])
    if den == "tau":
        for t in range(1, 4):                                                 # 309-315
            rho[:, 4] += 0.5 * np.einsum("gi,gia->ga", aob[t], ket[t])
    return rho


def _contract_ao_wv_bra(phi, aob, wv, den):
    """``contract_ao_wv_bra`` (pure_xcpot.rs:285-352) for every column a: phi [ncomp][g, mu],
    aob [ncomp][g, i], wv [g, nvar, a] -> out [mu, i, a]."""
    out = np.einsum("gu,ga,gi->uia", phi[0], wv[:, 0], aob[0], optimize=True)        # 331-333
    if den in ("sigma", "tau"):
        for t in range(1, 4):                                                 # 336-343
            out += np.einsum("gu,ga,gi->uia", phi[0], wv[:, t], aob[t], optimize=True)
            out += np.einsum("gu,ga,gi->uia", phi[t], wv[:, t], aob[0], optimize=True)
    if den == "tau":
        for t in range(1, 4):                                                 # 346-350
            out += 0.5 * np.einsum("gu,ga,gi->uia", phi[t], wv[:, 4], aob[t], optimize=True)
    return out


def rks_response_bra_mgga(ao, weights, fxc_eff, bra, mocc, den, nbatch=None):
    """RKS XC response for den = "rho" / "sigma" / "tau": ao [ngrids, nao, ncomp] (value and
    first derivatives), fxc_eff [ngrids, nvar, nvar]; hess_rks.rs:570-605 with
    rks_fxc_pot_with_eff_bra_trans_with_output (pure_xcpot.rs:370-465; wv[g, y] = w_g sum_x
    fxc_eff[g, x, y] rho1[g, x], 443-444), times 4.0."""
    bra = np.asarray(bra)
    shape = bra.shape
    nao, nocc = mocc.shape
    bra = bra.reshape(nao, nocc, -1)
    nprop = bra.shape[2]
    nc = 1 if den == "rho" else 4
    ng = len(weights)
    nv = NVAR[den]
    fxc = np.asarray(fxc_eff).reshape(ng, nv, nv)
    resp = np.zeros((nao, nocc, nprop))
    for g0, g1 in _batches(ng, nbatch):
        phi = [ao[g0:g1, :, c] for c in range(nc)]
        aob = [p @ mocc for p in phi]
        ket = [(p @ bra.reshape(nao, nocc * nprop)).reshape(g1 - g0, nocc, nprop) for p in phi]
        rho1 = _rho1_mgga(aob, ket, den)
        wv = weights[g0:g1, None, None] * np.einsum("gxy,gxa->gya", fxc[g0:g1], rho1)
        resp += _contract_ao_wv_bra(phi, aob, wv, den)
    return (4.0 * resp).reshape(shape)


def uks_response_bra_mgga(ao, weights, fxc_eff, bra, mocc, den, nbatch=None):
    """UKS XC response for den = "rho" / "sigma" / "tau": fxc_eff [ngrids, nvar, 2, nvar, 2]
    (hess_uks.rs:390-441, pure_xcpot.rs:921-1028: wv_t[g, y] = w_g sum_{x,s} fxc_eff[g, x, s, y, t]
    rho1_s[g, x], 1006), times 2.0."""
    nao = mocc[0].shape[0]
    shapes = [np.asarray(b).shape for b in bra]
    bra = [np.asarray(bra[s]).reshape(nao, mocc[s].shape[1], -1) for s in range(2)]
    nprop = bra[0].shape[2]
    nc = 1 if den == "rho" else 4
    ng = len(weights)
    nv = NVAR[den]
    fxc = np.asarray(fxc_eff).reshape(ng, nv, 2, nv, 2)
    resp = [np.zeros((nao, mocc[s].shape[1], nprop)) for s in range(2)]
    for g0, g1 in _batches(ng, nbatch):
        phi = [ao[g0:g1, :, c] for c in range(nc)]
        aob = [[p @ mocc[s] for p in phi] for s in range(2)]
        rho1 = []
        for s in range(2):
            no = mocc[s].shape[1]
            ket = [(p @ bra[s].reshape(nao, no * nprop)).reshape(g1 - g0, no, nprop) for p in phi]
            rho1.append(_rho1_mgga(aob[s], ket, den))
        rho1 = np.stack(rho1, axis=2)                                # [g, x, s, a]
        for t in range(2):
            wv = weights[g0:g1, None, None] * np.einsum("gxsy,gxsa->gya", fxc[g0:g1, :, :, :, t], rho1)
            resp[t] += _contract_ao_wv_bra(phi, aob[t], wv, den)
    return [(2.0 * resp[s]).reshape(shapes[s]) for s in range(2)]


def rks_response_bra_mgga_dm_form(ao, weights, fxc_eff, bra, mocc, den):
    """Independent density-matrix form of the same kernel: dm1 = 2 (bra mocc^T + h.c.);
    rho1 = phi dm phi, grad rho1 = d_t phi dm phi + phi dm d_t phi, tau1 = 1/2 sum_t d_t phi dm d_t phi;
    v1 = sum_g [wv0 phi phi + wv_t (d_t phi phi + phi d_t phi) + 1/2 wv4 sum_t d_t phi d_t phi];
    resp = v1 mocc (the symmetric dm makes the 2 x 2 factor of the bra form's 4.0)."""
    bra = np.asarray(bra)
    shape = bra.shape
    nao, nocc = mocc.shape
    bra = bra.reshape(nao, nocc, -1)
    ng = len(weights)
    nv = NVAR[den]
    fxc = np.asarray(fxc_eff).reshape(ng, nv, nv)
    out = np.zeros_like(bra)
    phi = [ao[:, :, c] for c in range(1 if den == "rho" else 4)]
    for a in range(bra.shape[2]):
        dm1 = 2.0 * bra[:, :, a] @ mocc.T
        dm1 = dm1 + dm1.T
        rho = np.zeros((ng, nv))
        rho[:, 0] = np.einsum("gu,uv,gv->g", phi[0], dm1, phi[0], optimize=True)
        if den in ("sigma", "tau"):
            for t in range(1, 4):
                rho[:, t] = 2.0 * np.einsum("gu,uv,gv->g", phi[t], dm1, phi[0], optimize=True)
        if den == "tau":
            for t in range(1, 4):
                rho[:, 4] += 0.5 * np.einsum("gu,uv,gv->g", phi[t], dm1, phi[t], optimize=True)
        wv = weights[:, None] * np.einsum("gxy,gx->gy", fxc, rho)
        v1 = phi[0].T @ (wv[:, 0:1] * phi[0])
        if den in ("sigma", "tau"):
            for t in range(1, 4):
                m = phi[t].T @ (wv[:, t:t + 1] * phi[0])
                v1 += m + m.T
        if den == "tau":
            for t in range(1, 4):
                v1 += 0.5 * phi[t].T @ (wv[:, 4:5] * phi[t])
        out[:, :, a] = v1 @ mocc
    return out.reshape(shape)
