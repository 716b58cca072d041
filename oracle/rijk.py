"""RI-J / RI-K response (bra form) -- oracle restatement (test infrastructure only).

Restates ``src/ri_jk/hess_r.rs`` of the reference:

* :func:`rijk_response_bra_separated` -- ``get_rijk_response_bra_separated``
  (``hess_r.rs:82-186``): J from the total density response through the packed
  upper triangle of ``cderi`` (``hess_r.rs:128-140``), K per spin over aux
  batches of 72 (``hess_r.rs:144-183``).
* :func:`rhf_response_bra` -- ``RHessRIJK::get_response_bra`` (``hess_r.rs:1916-1953``).
* :func:`uhf_response_bra` -- ``UHessRIJK::get_response_bra`` (``src/ri_jk/hess_u.rs:270-313``).
* :func:`rhf_response_bra_naive` -- the einsum form
  ``get_rijk_response_bra_naive`` (``src/ri_jk/hess_r_naive.rs:861-903``) with
  the RI factor ``(uv|P)(P|Q)^-1(Q|kl)`` replaced by ``sum_P B_P,uv B_P,kl``.
* :func:`pack_triu_tilde` / :func:`unpack_tri_sym` -- ``src/util/density_matrices.rs:48-77``
  and rstsr's ``unpack_tri(Upper, Sy)``: col-major packed upper triangle,
  element ``(mu <= nu)`` at ``nu*(nu+1)/2 + mu``.

Shapes follow the reference (col-major semantics, numpy indexing):
``cderi [nao_tp, naux]``, ``mo_coeff [nao, nmo]``, ``mo_occ [nmo]``,
``bra [nao, nocc, nprop]``.  The per-RHS loop of ``hess_r.rs:164-176`` is
evaluated as one GEMM over all RHS of an aux batch (same products and sums,
only the loop order of independent RHS differs).  Every contraction that the reference
performs as a matrix product runs through BLAS here too (``tensordot``), so
that the timed CPU baseline reflects the reference's arithmetic and not numpy's generic
einsum loop.
"""

import numpy as np


def triu_index(nao):
    """Return (mu, nu) index arrays of the packed upper triangle in storage order."""
    mu = np.concatenate([np.arange(nu + 1) for nu in range(nao)])
    nu = np.concatenate([np.full(nu + 1, nu) for nu in range(nao)])
    return mu, nu


def pack_triu_tilde(dm):
    """``[nao, nao, ...] -> [nao_tp, ...]``, off-diagonal elements doubled (density_matrices.rs:48-57)."""
    nao = dm.shape[0]
    mu, nu = triu_index(nao)
    out = 2.0 * dm[mu, nu]
    out[mu == nu] *= 0.5
    return out


def unpack_tri_sym(tp, nao):
    """``[nao_tp, ...] -> [nao, nao, ...]`` symmetric unpack of the packed upper triangle."""
    mu, nu = triu_index(nao)
    out = np.zeros((nao, nao) + tp.shape[1:])
    out[mu, nu] = tp
    out[nu, mu] = tp
    return out


def _mocc(mo_coeff, mo_occ):
    return mo_coeff[:, np.asarray(mo_occ) > 0]


def rijk_response_bra_separated(cderi, mo_coeff, mo_occ, bra, do_j=True, do_k=True, nbatch_aux=72):
    """``get_rijk_response_bra_separated`` (hess_r.rs:82-186).

    ``mo_coeff``, ``mo_occ``, ``bra`` are lists with one entry per spin.
    Returns ``(j_ao [nao, nao, nprop] or None, [k_bra_s [nao, nocc_s, nprop]])``.
    """
    nset = len(mo_coeff)
    nao = mo_coeff[0].shape[0]
    nao_tp, naux = cderi.shape
    assert nao_tp == nao * (nao + 1) // 2
    mocc = [_mocc(mo_coeff[s], mo_occ[s]) for s in range(nset)]
    nocc = [m.shape[1] for m in mocc]
    bra = [np.asarray(bra[s]).reshape(nao, nocc[s], -1) for s in range(nset)]
    nprop = bra[0].shape[2]

    j_ao = None
    if do_j:
        # hess_r.rs:131-139
        dm1 = np.zeros((nao, nao, nprop))
        for s in range(nset):
            dm1 += np.tensordot(bra[s], mocc[s], axes=([1], [1])).transpose(0, 2, 1)  # uin,vi->uvn
        dm1 = dm1 + dm1.transpose(1, 0, 2)
        dm1_tp = pack_triu_tilde(dm1)
        itm_j_aux = cderi.T @ dm1_tp
        resp_tp_j = 2.0 * (cderi @ itm_j_aux)
        j_ao = unpack_tri_sym(resp_tp_j, nao)

    k_bras = []
    if do_k:
        for s in range(nset):
            mocc_s = mocc[s]
            no = nocc[s]
            bra_s = bra[s]
            resp_k = np.zeros_like(bra_s)
            bra_mat = bra_s.reshape(nao, no * nprop)
            for p0 in range(0, naux, nbatch_aux):
                p1 = min(p0 + nbatch_aux, naux)
                nb = p1 - p0
                cd = unpack_tri_sym(cderi[:, p0:p1], nao)            # [mu, nu, P]
                # hess_r.rs:160-162: bxo[nu,P,i] = sum_mu B[mu,nu,P] C[mu,i]; oxo[k,P,i]
                bxo = np.tensordot(cd, mocc_s, axes=([0], [0]))            # uvP,ui->vPi
                oxo = np.tensordot(mocc_s, bxo, axes=([0], [0]))           # vk,vPi->kPi
                # hess_r.rs:168: bxo1[nu,P,j,a] = sum_mu B[mu,nu,P] bra[mu,j,a]
                bxo1 = (cd.reshape(nao, nao * nb).T @ bra_mat).reshape(nao, nb, no, nprop)
                # hess_r.rs:169-170: resp[nu,k,a] -= sum_{P,j} bxo1[nu,P,j,a] oxo[k,P,j]
                resp_k -= np.einsum("vPja,kPj->vka", bxo1, oxo, optimize=True)
                # hess_r.rs:172-175: oxo1[k,P,j,a] = sum_nu C[nu,k] bxo1[nu,P,j,a];
                #                    resp[nu,k,a] -= sum_{P,j} bxo[nu,P,j] oxo1[k,P,j,a]
                oxo1 = np.einsum("vk,vPja->kPja", mocc_s, bxo1, optimize=True)
                resp_k -= np.einsum("vPj,kPja->vka", bxo, oxo1, optimize=True)
            k_bras.append(resp_k)
    return j_ao, k_bras


def rhf_response_bra(cderi, mo_coeff, mo_occ, bra, scale_j, scale_k):
    """``RHessRIJK::get_response_bra`` (hess_r.rs:1916-1953); bra ``[nao, nocc, ...]``."""
    bra = np.asarray(bra)
    shape = bra.shape
    nao = mo_coeff.shape[0]
    mocc = _mocc(mo_coeff, mo_occ)
    nocc = mocc.shape[1]
    j_ao, k_bras = rijk_response_bra_separated(
        cderi, [mo_coeff], [mo_occ], [bra], scale_j != 0.0, scale_k != 0.0)
    nprop = int(np.prod(shape[2:])) if len(shape) > 2 else 1
    resp = np.zeros((nao, nocc, nprop))
    if j_ao is not None:
        resp += scale_j * np.tensordot(j_ao, mocc, axes=([1], [0])).transpose(0, 2, 1)  # uvn,vi->uin
    if k_bras:
        resp += scale_k * k_bras[0].reshape(nao, nocc, nprop)
    return resp.reshape(shape)


def uhf_response_bra(cderi, mo_coeff, mo_occ, bra, scale_j, scale_k):
    """``UHessRIJK::get_response_bra`` (hess_u.rs:270-313); lists of two spins."""
    nao = mo_coeff[0].shape[0]
    j_ao, k_bras = rijk_response_bra_separated(
        cderi, list(mo_coeff), list(mo_occ), list(bra), scale_j != 0.0, scale_k != 0.0)
    out = []
    for s in range(2):
        mocc = _mocc(mo_coeff[s], mo_occ[s])
        shape = np.asarray(bra[s]).shape
        nprop = int(np.prod(shape[2:])) if len(shape) > 2 else 1
        r = np.zeros((nao, mocc.shape[1], nprop))
        if j_ao is not None:
            r += 0.5 * scale_j * np.tensordot(j_ao, mocc, axes=([1], [0])).transpose(0, 2, 1)  # uvn,vi->uin
        if k_bras:
            r += scale_k * k_bras[s].reshape(r.shape)
        out.append(r.reshape(shape))
    return out


def rhf_response_bra_naive(cderi, mo_coeff, mo_occ, bra, scale_j, scale_k):
    """Einsum cross-check (hess_r_naive.rs:861-903) with ``eri[uv,kl] = sum_P B_P,uv B_P,kl``."""
    nao = mo_coeff.shape[0]
    mocc = _mocc(mo_coeff, mo_occ)
    bra = np.asarray(bra)
    shape = bra.shape
    bra = bra.reshape(nao, mocc.shape[1], -1)
    cd = unpack_tri_sym(cderi, nao)
    eri = np.einsum("uvP,klP->uvkl", cd, cd, optimize=True)
    rj = np.einsum("uvkl,kjA,lj,vi->uiA", eri, bra, mocc, mocc, optimize=True)
    rk0 = np.einsum("uvkl,vjA,lj,ki->uiA", eri, bra, mocc, mocc, optimize=True)
    rk1 = np.einsum("uvkl,kjA,vj,li->uiA", eri, bra, mocc, mocc, optimize=True)
    return (4.0 * scale_j * rj - scale_k * (rk0 + rk1)).reshape(shape)
