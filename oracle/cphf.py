"""CPHF driver (RHF and UHF) -- oracle restatement (test infrastructure only).

Restates the CPHF part of ``src/hessian/rscf.rs`` and ``src/hessian/uscf.rs``:

* ``RHF.response_mo``            -- ``rscf.rs:210-220``
* ``RHF.response_dimless_cphf``  -- ``rscf.rs:237-263``
* ``RHF.solve_dimless_cphf``     -- ``rscf.rs:278-300`` (Rust semantics: no
  pinning of ``mo1[occ, occ]``, unlike ``pyhessref/hess_scf_restricted.py:239-245``)
* ``RHF.finalize_cphf``          -- ``rscf.rs:328-353``
* ``RHF.get_cphf_hess``          -- ``rscf.rs:371-399``
* ``UHF.*``                      -- ``uscf.rs:203-446`` (both spins concatenated
  into one Krylov vector per column, ``uscf.rs:292-334``)
* :func:`compute_dimless_cphf_rhs` -- ``rscf.rs:104-182`` (RHF) and ``uscf.rs:78-173``
  (UHF, per spin with the shared core and overlap derivatives), from the summed skeleton
  derivatives the core / electron-interaction / overlap providers return

Electron-interaction plugins are callables ``get_response_bra(bra) -> resp``
(RHF: ``[nao, nocc, nprop]``; UHF: two-spin lists), mirroring
``RHessElecInteractAPI::get_response_bra`` (``src/hessian/trait_rhess.rs:664``).
Orbitals are ordered occupied first, as ``rscf.rs:253-254`` assumes.
"""

import numpy as np

from .krylov import krylov_block

DEFAULT_CONFIG = dict(level_shift=0.0, cphf_tol=1e-8, cphf_max_cycle=42, cphf_max_space=14,
                      cphf_lindep=1e-14)   # HessSCFConfig::default, rscf.rs:14-18


class RHF:
    def __init__(self, mo_coeff, mo_occ, mo_energy, plugins, natm, config=None):
        self.mo_coeff = np.asarray(mo_coeff, dtype=np.float64)
        self.mo_occ = np.asarray(mo_occ, dtype=np.float64)
        self.mo_energy = np.asarray(mo_energy, dtype=np.float64)
        self.plugins = list(plugins)
        self.natm = natm
        self.config = dict(DEFAULT_CONFIG, **(config or {}))
        occ = self.mo_occ > 0
        self.nocc = int(occ.sum())
        self.nmo = len(self.mo_occ)
        self.eocc = self.mo_energy[occ]
        self.evir = self.mo_energy[~occ]
        self.e_ai = self.evir[:, None] - self.eocc[None, :]
        self.e_ij = self.eocc[:, None] - self.eocc[None, :]
        self.krylov_stats = {}

    # rscf.rs:210-220
    def response_mo(self, mo1):
        mo1 = np.asarray(mo1)
        shape = mo1.shape
        C = self.mo_coeff
        x = mo1.reshape(self.nmo, self.nocc, -1)
        ubra = np.einsum("up,pia->uia", C, x, optimize=True)
        resp = np.zeros_like(x)
        for get_response_bra in self.plugins:
            resp += np.einsum("up,uia->pia", C, get_response_bra(ubra), optimize=True)
        return resp.reshape(shape)

    # rscf.rs:237-263
    def response_dimless_cphf(self, mo1):
        mo1 = np.asarray(mo1)
        shape = mo1.shape
        x = mo1.reshape(self.nmo, self.nocc, -1)
        shift = self.config["level_shift"]
        resp = self.response_mo(x)
        if shift != 0.0:
            resp -= shift * x
        resp[self.nocc:] /= (self.e_ai + shift)[:, :, None]
        resp[:self.nocc] = 0.0
        return resp.reshape(shape)

    # rscf.rs:278-300
    def solve_dimless_cphf(self, rhs, x0=None):
        rhs = np.asarray(rhs)
        shape = rhs.shape
        n = self.nmo * self.nocc
        b = rhs.reshape(self.nmo, self.nocc, -1).reshape(n, -1, order="F")

        def aop(x):
            y = self.response_dimless_cphf(x.reshape(self.nmo, self.nocc, -1, order="F"))
            return y.reshape(n, -1, order="F")

        c = self.config
        self.krylov_stats = {}
        x = krylov_block(aop, b, x0, c["cphf_tol"], c["cphf_max_cycle"], c["cphf_max_space"],
                         c["cphf_lindep"], stats=self.krylov_stats)
        return x.reshape(self.nmo, self.nocc, -1, order="F").reshape(shape)

    # rscf.rs:328-353
    def finalize_cphf(self, f1mo, s1mo, mo1):
        no = self.nocc
        b1mo = f1mo - s1mo * self.eocc[None, :, None, None] + self.response_mo(mo1)
        mo1 = np.array(mo1, copy=True)
        mo1[no:] = -b1mo[no:] / self.e_ai[:, :, None, None]
        mo_e1 = b1mo[:no] + mo1[:no] * self.e_ij[:, :, None, None]
        return mo1, mo_e1

    # rscf.rs:371-399; f1mo, s1mo, mo1: [nmo, nocc, 3, natm]; mo_e1: [nocc, nocc, 3, natm]
    def get_cphf_hess(self, f1mo, s1mo, mo1, mo_e1):
        return _cphf_hess([(f1mo, s1mo, mo1, mo_e1, self.eocc)], (4.0, 4.0, 2.0), self.natm)


class UHF:
    def __init__(self, mo_coeff, mo_occ, mo_energy, plugins, natm, config=None):
        self.mo_coeff = [np.asarray(m, dtype=np.float64) for m in mo_coeff]
        self.mo_occ = [np.asarray(m, dtype=np.float64) for m in mo_occ]
        self.mo_energy = [np.asarray(m, dtype=np.float64) for m in mo_energy]
        self.plugins = list(plugins)
        self.natm = natm
        self.config = dict(DEFAULT_CONFIG, **(config or {}))
        occ = [m > 0 for m in self.mo_occ]
        self.nocc = [int(o.sum()) for o in occ]
        self.nmo = [len(m) for m in self.mo_occ]
        self.eocc = [self.mo_energy[s][occ[s]] for s in range(2)]
        self.evir = [self.mo_energy[s][~occ[s]] for s in range(2)]
        self.e_ai = [self.evir[s][:, None] - self.eocc[s][None, :] for s in range(2)]
        self.e_ij = [self.eocc[s][:, None] - self.eocc[s][None, :] for s in range(2)]
        self.krylov_stats = {}

    # uscf.rs:203-218
    def response_mo(self, mo1):
        x = [np.asarray(mo1[s]).reshape(self.nmo[s], self.nocc[s], -1) for s in range(2)]
        ubra = [np.einsum("up,pia->uia", self.mo_coeff[s], x[s], optimize=True) for s in range(2)]
        resp = [np.zeros((self.nmo[s],) + ubra[s].shape[1:]) for s in range(2)]
        for get_response_bra in self.plugins:
            r = get_response_bra(ubra)
            for s in range(2):
                resp[s] += np.einsum("up,uia->pia", self.mo_coeff[s], r[s], optimize=True)
        return [resp[s].reshape(np.asarray(mo1[s]).shape) for s in range(2)]

    # uscf.rs:230-265
    def response_dimless_cphf(self, mo1):
        shift = self.config["level_shift"]
        x = [np.asarray(mo1[s]).reshape(self.nmo[s], self.nocc[s], -1) for s in range(2)]
        resp = self.response_mo(x)
        for s in range(2):
            if shift != 0.0:
                resp[s] -= shift * x[s]
            resp[s][self.nocc[s]:] /= (self.e_ai[s] + shift)[:, :, None]
            resp[s][:self.nocc[s]] = 0.0
        return resp

    def _pack(self, x):   # uscf.rs:292-304
        return np.concatenate([x[s].reshape(self.nmo[s], self.nocc[s], -1).reshape(
            self.nmo[s] * self.nocc[s], -1, order="F") for s in range(2)], axis=0)

    def _unpack(self, v):  # uscf.rs:306-319
        na = self.nmo[0] * self.nocc[0]
        parts = [v[:na], v[na:]]
        return [parts[s].reshape(self.nmo[s], self.nocc[s], -1, order="F") for s in range(2)]

    # uscf.rs:278-341
    def solve_dimless_cphf(self, rhs, x0=None):
        shapes = [np.asarray(r).shape for r in rhs]
        b = self._pack([np.asarray(r) for r in rhs])

        def aop(v):
            return self._pack(self.response_dimless_cphf(self._unpack(v)))

        c = self.config
        self.krylov_stats = {}
        x = krylov_block(aop, b, x0, c["cphf_tol"], c["cphf_max_cycle"], c["cphf_max_space"],
                         c["cphf_lindep"], stats=self.krylov_stats)
        out = self._unpack(x)
        return [out[s].reshape(shapes[s]) for s in range(2)]

    # uscf.rs:365-406
    def finalize_cphf(self, f1mo, s1mo, mo1):
        resp = self.response_mo(mo1)
        mo1_out, mo_e1 = [], []
        for s in range(2):
            no = self.nocc[s]
            b1mo = f1mo[s] - s1mo[s] * self.eocc[s][None, :, None, None] + resp[s]
            m = np.array(mo1[s], copy=True)
            m[no:] = -b1mo[no:] / self.e_ai[s][:, :, None, None]
            mo1_out.append(m)
            mo_e1.append(b1mo[:no] + m[:no] * self.e_ij[s][:, :, None, None])
        return mo1_out, mo_e1

    # uscf.rs:408-446
    def get_cphf_hess(self, f1mo, s1mo, mo1, mo_e1):
        return _cphf_hess([(f1mo[s], s1mo[s], mo1[s], mo_e1[s], self.eocc[s]) for s in range(2)],
                          (2.0, 2.0, 1.0), self.natm)


def _cphf_hess(spins, factors, natm):
    """``de[x, y, B, A]`` assembly of rscf.rs:378-397 / uscf.rs:423-443.

    For ``B <= A``: ``de[:, :, B, A] = sum_spin f0 <mo1_B, f1mo_A> - f1 <mo1_B, s1mo_A eocc>
    - f2 <mo_e1_B, s1oo_A>`` (contracting the two MO indices); then for ``B < A``
    ``de[:, :, A, B] += de[:, :, B, A]^T``.
    """
    f0, f1, f2 = factors
    de = np.zeros((3, 3, natm, natm))
    for A in range(natm):
        for B in range(A + 1):
            acc = np.zeros((3, 3))
            for (f1mo, s1mo, mo1, mo_e1, eocc) in spins:
                no = len(eocc)
                acc += f0 * np.einsum("pix,piy->xy", mo1[..., B], f1mo[..., A])
                acc -= f1 * np.einsum("pix,piy->xy", mo1[..., B], s1mo[..., A] * eocc[None, :, None])
                acc -= f2 * np.einsum("pix,piy->xy", mo_e1[..., B], s1mo[:no, :, :, A])
            de[:, :, B, A] += acc
        for B in range(A):
            de[:, :, A, B] += de[:, :, B, A].T
    return de


def compute_dimless_cphf_rhs(mo_coeff, mo_occ, mo_energy, f1ao_core, f1bra_el, s1ao, level_shift=0.0):
    """``compute_dimless_cphf_rhs`` (rscf.rs:104-182; uscf.rs:78-173 per spin).

    ``f1ao_core``, ``s1ao``: ``[nao, nao, 3, natm]`` (``f1ao_core`` may be None = 0);
    ``f1bra_el``: ``[nao, nocc, 3, natm]`` (None = 0).  Returns ``(rhs, f1mo, s1mo)``, each
    ``[nmo, nocc, 3, natm]``."""
    C = np.asarray(mo_coeff, dtype=np.float64)
    occ = np.asarray(mo_occ) > 0
    no = int(occ.sum())
    mocc = C[:, occ]
    e = np.asarray(mo_energy, dtype=np.float64)
    eocc, evir = e[occ], e[~occ]
    e_ai_shift = evir[:, None] - eocc[None, :] + level_shift
    s1ao = np.asarray(s1ao)
    nao = C.shape[0]
    tail = s1ao.shape[2:]
    f1bra = np.zeros((nao, no) + tail)
    if f1ao_core is not None:
        f1bra += np.einsum("uvxA,vi->uixA", f1ao_core, mocc, optimize=True)     # f1ao_core % mocc
    if f1bra_el is not None:
        f1bra += f1bra_el
    f1mo = np.einsum("up,uixA->pixA", C, f1bra, optimize=True)                 # mo_coeff^T % f1bra
    s1mo = np.einsum("up,uvxA,vi->pixA", C, s1ao, mocc, optimize=True)          # C^T (s1ao % mocc)
    b1mo = f1mo - s1mo * eocc[None, :, None, None]
    rhs = np.zeros_like(f1mo)
    rhs[no:] = -b1mo[no:] / e_ai_shift[:, :, None, None]
    rhs[:no] = -0.5 * s1mo[:no]
    return rhs, f1mo, s1mo
