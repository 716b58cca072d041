"""Generate the golden vectors under tests/golden/ from the reference's own Python code.

Run where the reference project is available and name its root in the ``CPHF_REFERENCE``
environment variable.  Nothing at test time reads the reference: the tests only load the
``.npz`` files written here.

What runs, all from the reference's sources:

* ``prototype/02-7-krylov_testing_setup.py`` -- ``build_test_system(n=40, nrhs=12)``, the
  fixture generator of ``tests/test_krylov_block.rs`` -- and ``pyhessref/krylov_block.py``
  on it with the Rust tests' parameters (``tol=1e-10``; ``max_space`` 6 and 3).
* ``pyhessref/rijk/hess_restricted_naive.get_rijk_response_bra_naive`` and
  ``pyhessref/rijk/hess_unrestricted_naive.get_uijk_response_bra_naive`` on seeded
  synthetic systems: PySCF is absent, so a stub ``pyscf`` package is installed whose
  integral hooks return the synthetic factor -- ``int3c2e`` -> dense ``B[mu, nu, P]`` and
  ``int2c2e`` -> identity -- making ``(uv|P)(P|Q)^-1(Q|kl) = sum_P B_P,uv B_P,kl``.
* ``pyhessref/hess_scf_restricted.RHessSCF`` and ``hess_scf_unrestricted.UHessSCF``
  (``response_dimless_cphf``, ``solve_dimless_cphf``, ``finalize_cphf``,
  ``get_cphf_hess``) driven by those naive plugins.
* ``pyhessref/nimatmul/rks.get_ks_response_bra_naive`` and
  ``pyhessref/nimatmul/uks.get_uks_response_bra_naive`` (the XC response in bra form) on seeded
  synthetic grids: the stub ``pyscf.dft.numint.NumInt`` supplies the LDA fxc integral PySCF
  would compute, ``nr_rks_fxc`` -> ``v1 = phi^T diag(w f rho1[dm1]) phi`` and ``nr_uks_fxc`` ->
  ``v1_t = phi^T diag(w sum_s f[., s, t] rho1[dm1_s]) phi``, with ``rho1[dm] = sum phi dm phi``.
  What runs from the reference is its wrapper: the perturbed density built from the bra
  (``2 bra mocc^T`` for RKS, ``bra mocc^T`` per spin for UKS), its symmetrisation and the
  projection ``v1 @ mocc``; the fxc integral itself is the stub's.

Usage: ``CPHF_REFERENCE=<reference root> python tests/golden/make_golden.py``
"""

import importlib.util
import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
REF = Path(os.environ["CPHF_REFERENCE"]) if os.environ.get("CPHF_REFERENCE") else None
sys.path.insert(0, str(REPO / "rstsr-showcase-hessian_gb300"))

from cphf_gb300 import synth  # noqa: E402


class _FakeMol:
    def __init__(self, nao, natm):
        self.nao = nao
        self.natm = natm

    def nao_nr(self):
        return self.nao


_CURRENT = {}


def _install_stub_pyscf():
    """A minimal ``pyscf`` so that pyhessref imports; integrals come from ``_CURRENT``."""
    pyscf = types.ModuleType("pyscf")
    gto = types.ModuleType("pyscf.gto")
    gto.Mole = _FakeMol
    df = types.ModuleType("pyscf.df")
    grad = types.ModuleType("pyscf.df.grad")
    rhf = types.ModuleType("pyscf.df.grad.rhf")

    def _int3c_wrapper(mol, aux, intor, aosym):
        assert intor == "int3c2e" and aosym == "s1"
        return lambda: _CURRENT["int3c2e"]

    rhf._int3c_wrapper = _int3c_wrapper
    dft = types.ModuleType("pyscf.dft")
    numint = types.ModuleType("pyscf.dft.numint")
    numint.NumInt = _StubNumInt
    dft.numint = numint
    pyscf.gto, pyscf.df, df.grad, grad.rhf, pyscf.dft = gto, df, grad, rhf, dft
    for name, mod in {"pyscf": pyscf, "pyscf.gto": gto, "pyscf.df": df, "pyscf.df.grad": grad,
                      "pyscf.df.grad.rhf": rhf, "pyscf.dft": dft, "pyscf.dft.numint": numint}.items():
        sys.modules[name] = mod


def _rho1(ao, dm):
    """rho1[p, g] = sum_{mu nu} ao[g, mu] dm[p, mu, nu] ao[g, nu] for dm [nprop, nao, nao]."""
    return np.einsum("gu,puv,gv->pg", ao, dm, ao, optimize=True)


def _fxc_mat(ao, wv):
    """v[p] = ao^T diag(wv[p]) ao."""
    return np.einsum("gu,pg,gv->puv", ao, wv, ao, optimize=True)


class _StubNumInt:
    """LDA fxc integrals on the synthetic grid of ``_CURRENT["grid"]`` (ao, weights, fxc)."""

    def nr_rks_fxc(self, mol, grids, xc, dm0, dm1, hermi=1, rho0=None, vxc=None, fxc=None):
        g = _CURRENT["grid"]
        dm1 = np.asarray(dm1)
        shape = dm1.shape
        dm = dm1.reshape(-1, shape[-2], shape[-1])
        wv = g.weights[None, :] * g.fxc[None, :] * _rho1(g.ao, dm)
        return _fxc_mat(g.ao, wv).reshape(shape)

    def nr_uks_fxc(self, mol, grids, xc, dm0, dm1, hermi=1, rho0=None, vxc=None, fxc=None):
        g = _CURRENT["grid"]
        dms = [np.asarray(d) for d in dm1]
        rho = [_rho1(g.ao, d.reshape(-1, d.shape[-2], d.shape[-1])) for d in dms]
        out = []
        for t in range(2):
            wv = g.weights[None, :] * (g.fxc[None, :, 0, t] * rho[0] + g.fxc[None, :, 1, t] * rho[1])
            out.append(_fxc_mat(g.ao, wv).reshape(dms[t].shape))
        return out


class _FakeAux:
    def __init__(self, naux):
        self.naux = naux

    def intor(self, name):
        assert name == "int2c2e"
        return np.eye(self.naux)


def _load_file(path, name):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _dense_b(s):
    nao = s.nao
    mu = np.concatenate([np.arange(nu + 1) for nu in range(nao)])
    nu = np.concatenate([np.full(nu + 1, nu) for nu in range(nao)])
    cd = np.zeros((nao, nao, s.naux))
    cd[mu, nu] = s.cderi
    cd[nu, mu] = s.cderi
    return cd


def _to_py(a):
    """[nmo, nocc, 3, natm] (col-major meaning) -> pyhessref's [natm, 3, nmo, nocc]."""
    return np.ascontiguousarray(np.transpose(a, (3, 2, 0, 1)))


def _from_py(a):
    return np.asfortranarray(np.transpose(a, (2, 3, 1, 0)))


def krylov_golden():
    # The setup script imports `krylov_block` from its own directory; load it with that on the path.
    sys.path.insert(0, str(REF / "prototype"))
    try:
        setup = _load_file(REF / "prototype" / "02-7-krylov_testing_setup.py", "krylov_testing_setup")
    finally:
        sys.path.pop(0)
    kb = _load_file(REF / "pyhessref" / "krylov_block.py", "pyhessref_krylov_block")
    A, b, eigs = setup.build_test_system(n=40, nrhs=12)
    x_ref = np.linalg.solve(np.eye(40) + A, b.T).T
    out = dict(A=A, b=b, x_ref=x_ref, eigs=eigs)
    for ms, mc in [(6, 30), (3, 60)]:
        calls = [0]

        def aop(x):
            calls[0] += 1
            return (A @ x.T).T

        x = kb.krylov_block(aop, b, tol=1e-10, max_cycle=mc, max_space=ms, lindep=1e-13)
        out[f"x_ms{ms}"] = x
        out[f"calls_ms{ms}"] = np.array(calls[0])
    np.savez(HERE / "krylov_fixture.npz", **out)


def rhf_golden(name, seed):
    from pyhessref.hess_scf_restricted import RHessSCF
    from pyhessref.rijk.hess_restricted_naive import get_rijk_response_bra_naive

    s = synth.make_system(name, seed=seed)
    C, occ, e = s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0]
    mol, aux = _FakeMol(s.nao, s.natm), _FakeAux(s.naux)
    _CURRENT["int3c2e"] = _dense_b(s)

    class Plugin:
        def make_response_preparation(self, mo_coeff, mo_occ):
            self.mo_coeff, self.mo_occ = mo_coeff, mo_occ

        def get_response_bra(self, bra):
            return get_rijk_response_bra_naive(mol, aux, self.mo_coeff, self.mo_occ, bra,
                                               scale_j=s.scale_j, scale_k=s.scale_k)

    plug = Plugin()
    drv = RHessSCF(mol, C, occ, e, None, [], [plug])
    drv.make_response_preparation(C, occ)
    rng = np.random.default_rng(seed + 100)
    bra_probe = rng.standard_normal((s.nao, s.nocc[0], 5))
    resp_probe = plug.get_response_bra(np.ascontiguousarray(np.transpose(bra_probe, (2, 0, 1))))
    rhs_py = _to_py(s.rhs[0])
    mo1_py = drv.solve_dimless_cphf(rhs_py.copy())
    pre = {"f1mo": _to_py(s.f1mo[0]), "s1mo": _to_py(s.s1mo[0]), "rhs": rhs_py}
    fin = drv.finalize_cphf(mo1_py.copy(), pre)
    de_py = drv.get_cphf_hess(pre["f1mo"], pre["s1mo"], fin["mo1"], fin["mo_e1"])
    np.savez(HERE / f"{name}_seed{seed}.npz",
             cderi=s.cderi, mo_coeff=C, mo_occ=occ, mo_energy=e, rhs=s.rhs[0], f1mo=s.f1mo[0],
             s1mo=s.s1mo[0], scale_j=s.scale_j, scale_k=s.scale_k, natm=s.natm,
             bra_probe=bra_probe, resp_probe=np.asfortranarray(np.transpose(resp_probe, (1, 2, 0))),
             mo1_solved=_from_py(mo1_py), mo1=_from_py(fin["mo1"]),
             mo_e1=_from_py(fin["mo_e1"]), de_cphf=np.asfortranarray(np.transpose(de_py, (3, 2, 1, 0))))


def uhf_golden(dims, tag, seed):
    from pyhessref.hess_scf_unrestricted import UHessSCF
    from pyhessref.rijk.hess_unrestricted_naive import get_uijk_response_bra_naive

    s = synth.make_system(dims, seed=seed)
    mol, aux = _FakeMol(s.nao, s.natm), _FakeAux(s.naux)
    _CURRENT["int3c2e"] = _dense_b(s)
    C = np.stack(s.mo_coeff)
    occ = np.stack(s.mo_occ)
    e = np.stack(s.mo_energy)

    class Plugin:
        def make_response_preparation(self, mo_coeff, mo_occ):
            self.mo_coeff, self.mo_occ = mo_coeff, mo_occ

        def get_response_bra(self, bra):
            return get_uijk_response_bra_naive(mol, aux, self.mo_coeff, self.mo_occ, bra,
                                               scale_j=s.scale_j, scale_k=s.scale_k)

    plug = Plugin()
    drv = UHessSCF(mol, C, occ, e, None, [], [plug])
    drv.make_response_preparation(C, occ)
    rhs_py = [_to_py(r) for r in s.rhs]
    mo1_py = drv.solve_dimless_cphf([r.copy() for r in rhs_py])
    pre = {"f1mo": [_to_py(f) for f in s.f1mo], "s1mo": [_to_py(x) for x in s.s1mo], "rhs": rhs_py}
    fin = drv.finalize_cphf([m.copy() for m in mo1_py], pre)
    de_py = drv.get_cphf_hess(pre["f1mo"], pre["s1mo"], fin["mo1"], fin["mo_e1"])
    out = dict(cderi=s.cderi, scale_j=s.scale_j, scale_k=s.scale_k, natm=s.natm,
               de_cphf=np.asfortranarray(np.transpose(de_py, (3, 2, 1, 0))))
    for sp in range(2):
        out.update({f"mo_coeff{sp}": s.mo_coeff[sp], f"mo_occ{sp}": s.mo_occ[sp],
                    f"mo_energy{sp}": s.mo_energy[sp], f"rhs{sp}": s.rhs[sp], f"f1mo{sp}": s.f1mo[sp],
                    f"s1mo{sp}": s.s1mo[sp], f"mo1_solved{sp}": _from_py(mo1_py[sp]),
                    f"mo1{sp}": _from_py(fin["mo1"][sp]), f"mo_e1{sp}": _from_py(fin["mo_e1"][sp])})
    np.savez(HERE / f"{tag}_seed{seed}.npz", **out)


XC_RKS = dict(nao=30, naux=90, nocc=(6,), natm=3, decay=6.0, grid=True, points=(150, 260), window=12)
XC_UKS = dict(nao=28, naux=84, nocc=(6, 5), natm=3, decay=6.0, grid=True, points=(140, 240), window=12)


def xc_golden(dims, tag, seed):
    """The reference's XC response wrappers (bra form) on a seeded synthetic grid."""
    from pyhessref.nimatmul.rks import get_ks_response_bra_naive
    from pyhessref.nimatmul.uks import get_uks_response_bra_naive

    s = synth.make_system(dims, seed=seed)
    g = s.grid
    _CURRENT["grid"] = g
    mol = _FakeMol(s.nao, s.natm)
    rng = np.random.default_rng(seed + 300)
    nprop = 4
    out = dict(ao=g.ao, weights=g.weights, fxc=g.fxc, atom_offsets=g.atom_offsets, cderi=s.cderi,
               scale_j=s.scale_j, scale_k=s.scale_k, nspin=s.nspin)
    # bra [nao, nocc, nprop] (col-major meaning) <-> pyhessref's [nprop, nao, nocc]
    if s.nspin == 1:
        C, occ = s.mo_coeff[0], s.mo_occ[0]
        bra = rng.standard_normal((s.nao, s.nocc[0], nprop))
        resp = get_ks_response_bra_naive(mol, None, "lda", C, occ, None,
                                         np.ascontiguousarray(np.transpose(bra, (2, 0, 1))))
        out.update(mo_coeff0=C, mo_occ0=occ, mo_energy0=s.mo_energy[0], bra0=bra,
                   resp0=np.asfortranarray(np.transpose(resp, (1, 2, 0))))
    else:
        bra = [rng.standard_normal((s.nao, s.nocc[t], nprop)) for t in range(2)]
        resp = get_uks_response_bra_naive(mol, None, "lda", [c for c in s.mo_coeff], [o for o in s.mo_occ],
                                          None, None,
                                          [np.ascontiguousarray(np.transpose(b, (2, 0, 1))) for b in bra])
        for t in range(2):
            out.update({f"mo_coeff{t}": s.mo_coeff[t], f"mo_occ{t}": s.mo_occ[t],
                        f"mo_energy{t}": s.mo_energy[t], f"bra{t}": bra[t],
                        f"resp{t}": np.asfortranarray(np.transpose(resp[t], (1, 2, 0)))})
    np.savez(HERE / f"{tag}_seed{seed}.npz", **out)


def rhs_golden(tag, seed, nspin):
    """compute_dimensionless_cphf_rhs of pyhessref's RHessSCF / UHessSCF with stub derivative
    providers returning seeded synthetic skeleton derivatives (core and overlap AO matrices per
    atom, the electron-interaction bra)."""
    dims = dict(nao=22, naux=60, nocc=(5,) if nspin == 1 else (5, 4), natm=3, decay=6.0)
    s = synth.make_system(dims, seed=seed)
    nao, natm = s.nao, s.natm
    rng = np.random.default_rng(seed + 500)
    sym = lambda a: a + np.swapaxes(a, -1, -2)  # noqa: E731
    f1core = 0.1 * rng.standard_normal((natm, 3, nao, nao))
    s1ao = 0.1 * sym(rng.standard_normal((natm, 3, nao, nao)))
    f1el = [0.1 * rng.standard_normal((natm, 3, nao, s.nocc[t])) for t in range(nspin)]
    mol = _FakeMol(nao, natm)

    class Gen:
        def __init__(self, arr):
            self.arr = arr

        def generator_deriv1(self):
            return lambda A: self.arr[A]

    class El:
        def get_deriv1_bra(self, mo_coeff, mo_occ):
            return f1el[0] if nspin == 1 else [f1el[0], f1el[1]]

    out = dict(f1ao_core=np.asfortranarray(np.transpose(f1core, (2, 3, 1, 0))),
               s1ao=np.asfortranarray(np.transpose(s1ao, (2, 3, 1, 0))), natm=natm, nspin=nspin)
    if nspin == 1:
        from pyhessref.hess_scf_restricted import RHessSCF
        drv = RHessSCF(mol, s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0], Gen(s1ao), [Gen(f1core)], [El()])
        res = drv.compute_dimensionless_cphf_rhs()
        res = {k: [v] for k, v in res.items()}
    else:
        from pyhessref.hess_scf_unrestricted import UHessSCF
        drv = UHessSCF(mol, np.stack(s.mo_coeff), np.stack(s.mo_occ), np.stack(s.mo_energy), Gen(s1ao),
                       [Gen(f1core)], [El()])
        res = drv.compute_dimensionless_cphf_rhs()
    for t in range(nspin):
        out.update({f"mo_coeff{t}": s.mo_coeff[t], f"mo_occ{t}": s.mo_occ[t], f"mo_energy{t}": s.mo_energy[t],
                    f"f1bra_el{t}": np.asfortranarray(np.transpose(f1el[t], (2, 3, 1, 0))),
                    f"rhs{t}": _from_py(res["rhs"][t]), f"f1mo{t}": _from_py(res["f1mo"][t]),
                    f"s1mo{t}": _from_py(res["s1mo"][t])})
    np.savez(HERE / f"{tag}_seed{seed}.npz", **out)


def main():
    if REF is None or not (REF / "pyhessref").is_dir():
        raise SystemExit("set CPHF_REFERENCE to the reference project's root (the directory holding pyhessref/)")
    _install_stub_pyscf()
    sys.path.insert(0, str(REF))
    krylov_golden()
    rhf_golden("rhf_nao24", seed=1)
    uhf_golden(dict(nao=20, naux=70, nocc=(5, 4), natm=3, decay=6.0), "uhf_nao20", seed=2)
    xc_golden(XC_RKS, "xc_rks_nao30", seed=3)
    xc_golden(XC_UKS, "xc_uks_nao28", seed=4)
    rhs_golden("rhs_rhf_nao22", seed=5, nspin=1)
    rhs_golden("rhs_uhf_nao22", seed=6, nspin=2)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
