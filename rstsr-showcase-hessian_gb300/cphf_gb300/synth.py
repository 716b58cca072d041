"""Seeded synthetic CPHF systems (the workloads of the benchmark and the parity tests).

The reference computes ``cderi`` (B), MO coefficients, orbital energies and
the CPHF right-hand side from real molecules through libcint/libxc.  Those
are inputs to the response path, not part of it, so this module draws them
from seeded distributions with the shapes and value ranges of a molecule:

* ``B[mu nu, P]`` symmetric in ``mu nu``, stored as the col-major packed upper
  triangle ``[nao_tp, naux]`` (element ``mu <= nu`` at ``nu (nu+1)/2 + mu``,
  the layout of ``generate_cderi_with_decomp``, ``src/ri_jk/hess_r.rs:1725-1735``),
  entries ``N(0, sigma^2)`` with ``sigma = 0.3 exp(-|mu - nu| / L)``;
* ``C`` orthogonal (Q of the QR of a Gaussian matrix, so ``S = I``);
* occupied energies sorted uniform on ``[-20, -0.3]``, virtual uniform on ``[0.05, 5]``;
* ``s1mo`` Gaussian x 0.1; the right-hand side is Gaussian x 0.1 in the
  virtual block and ``-0.5 s1mo`` in the occupied block
  (``src/hessian/rscf.rs:176-177``); ``f1mo`` is chosen so that
  ``rhs[vir] = -(f1mo - s1mo eocc)[vir] / e_ai`` holds exactly, and its
  occupied block is Gaussian x 0.1;
* the scale of B (and of the XC kernel) is fixed so that the spectral norm of
  the induced response operator on the vir-occ block is ``0.5 x`` the smallest
  orbital-energy gap, estimated by ``npower`` power iterations with a
  self-contained numpy matvec in the Z-factored form.

XC grids (RKS/UKS): per-atom point counts uniform on ``[8000, 14000]`` (or as
given), weights uniform on ``(0, 1e-2]``, AO values Gaussian times an
envelope ``exp(-(d/40)^2)`` of the index distance ``d`` between the AO and the
point's atom block, exactly zero for ``d > window`` AO indices;
``f_xc = -c rho^{-2/3}`` with ``rho`` log-uniform on ``[1e-6, 10]``; ``c`` is
chosen so that the XC operator's norm matches the RI-JK operator's before the
common rescaling.

All arrays are float64 and Fortran-ordered, so that their raw buffers are the
col-major layouts of the C ABI in ``include/cphf.h``.
"""

from dataclasses import dataclass, field

import numpy as np

# The workloads, named by their sizes.
CONFIGS = {
    # nao=24, naux=84, nocc=5, nrhs=12 (4 atoms), sigma decay length 6
    "rhf_nao24": dict(nao=24, naux=84, nocc=(5,), natm=4, decay=6.0),
    # nao=600, naux=2000, nocc=60, nrhs=180 (60 atoms), decay 20
    "rhf_nao600": dict(nao=600, naux=2000, nocc=(60,), natm=60, decay=20.0),
    # half-size case for profiler captures: nao=300, naux=1000, nocc=30, nrhs=90
    "rhf_nao300": dict(nao=300, naux=1000, nocc=(30,), natm=30, decay=20.0),
    # profiler captures at the evaluation size's nocc (120 = the width of one T tile):
    # nao=384, naux=1280, nocc=120, nrhs=36 (12 atoms)
    "rhf_nao384_occ120": dict(nao=384, naux=1280, nocc=(120,), natm=12, decay=20.0),
    # config above plus a ~660k-point LDA grid (60 atoms x 10 AOs)
    "rks_nao600": dict(nao=600, naux=2000, nocc=(60,), natm=60, decay=20.0, grid=True),
    # UHF/UKS: nao=800, naux=2700, nocc 80/78, 240 RHS (80 atoms)
    "uks_nao800": dict(nao=800, naux=2700, nocc=(80, 78), natm=80, decay=20.0, grid=True),
    # evaluation size: nao=1200, naux=4000, nocc=120, 360 RHS (120 atoms)
    "rhf_nao1200": dict(nao=1200, naux=4000, nocc=(120,), natm=120, decay=20.0),
}


@dataclass
class Grid:
    ao: np.ndarray            # [ngrids, nao], F-order (grid index fastest)
    weights: np.ndarray       # [ngrids]
    fxc: np.ndarray           # RKS: [ngrids]; UKS: [ngrids, 2, 2] (F-order), f[g, s_in, s_out]
    atom_offsets: np.ndarray  # int64 [natm + 1], grid points of atom A are [off[A], off[A+1])
    window: int = 80


@dataclass
class System:
    nao: int
    naux: int
    natm: int
    nspin: int
    cderi: np.ndarray                   # [nao_tp, naux] F-order
    mo_coeff: list                      # per spin [nao, nmo] F-order
    mo_occ: list                        # per spin [nmo]
    mo_energy: list                     # per spin [nmo]
    rhs: list                           # per spin [nmo, nocc, 3, natm] F-order
    f1mo: list
    s1mo: list
    scale_j: float = 1.0
    scale_k: float = 0.5
    grid: Grid = None
    scale_b: float = 1.0                # factor applied to the raw Gaussian B
    info: dict = field(default_factory=dict)

    @property
    def nocc(self):
        return [int((o > 0).sum()) for o in self.mo_occ]

    @property
    def nmo(self):
        return [len(o) for o in self.mo_occ]

    @property
    def nrhs(self):
        return 3 * self.natm


def _fortran(a):
    return np.asfortranarray(a, dtype=np.float64)


def make_cderi(rng, nao, naux, decay):
    """Packed upper-triangle B ``[nao_tp, naux]`` (F-order), sigma = 0.3 exp(-|mu-nu|/decay)."""
    nao_tp = nao * (nao + 1) // 2
    mu = np.concatenate([np.arange(nu + 1) for nu in range(nao)])
    nu = np.concatenate([np.full(nu + 1, nu) for nu in range(nao)])
    sigma = 0.3 * np.exp(-np.abs(mu - nu) / decay)
    out = np.empty((nao_tp, naux), order="F")
    chunk = max(1, (1 << 24) // nao_tp)
    for p0 in range(0, naux, chunk):
        p1 = min(naux, p0 + chunk)
        out[:, p0:p1] = (rng.standard_normal((p1 - p0, nao_tp)) * sigma[None, :]).T
    return out


def make_grid(rng, nao, natm, points_range=(8000, 14000), window=80, nspin=1):
    """Per-atom grid batches with block-sparse Gaussian-envelope AO values."""
    npts = rng.integers(points_range[0], points_range[1] + 1, size=natm)
    offsets = np.zeros(natm + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(npts)
    ng = int(offsets[-1])
    ao_per_atm = nao // natm
    ao = np.zeros((ng, nao), order="F")
    mu = np.arange(nao)
    for A in range(natm):
        lo, hi = A * ao_per_atm, (A + 1) * ao_per_atm if A < natm - 1 else nao
        d = np.maximum(np.maximum(lo - mu, mu - (hi - 1)), 0)
        env = np.where(d <= window, np.exp(-(d / 40.0) ** 2), 0.0)
        cols = np.nonzero(env)[0]
        g0, g1 = offsets[A], offsets[A + 1]
        ao[g0:g1, cols] = rng.standard_normal((g1 - g0, len(cols))) * env[cols][None, :]
    weights = rng.uniform(0.0, 1e-2, size=ng)
    weights = np.where(weights == 0.0, 1e-2, weights)
    rho = np.exp(rng.uniform(np.log(1e-6), np.log(10.0), size=ng))
    if nspin == 1:
        fxc = -rho ** (-2.0 / 3.0)
    else:
        # spin-resolved LDA-form kernel: same-spin -c rho_s^{-2/3}, weak opposite-spin coupling
        rho_s = np.stack([rho, np.exp(rng.uniform(np.log(1e-6), np.log(10.0), size=ng))], axis=1)
        fxc = np.zeros((ng, 2, 2), order="F")
        fxc[:, 0, 0] = -rho_s[:, 0] ** (-2.0 / 3.0)
        fxc[:, 1, 1] = -rho_s[:, 1] ** (-2.0 / 3.0)
        cross = -0.1 * (rho_s[:, 0] * rho_s[:, 1]) ** (-1.0 / 3.0)
        fxc[:, 0, 1] = cross
        fxc[:, 1, 0] = cross
    return Grid(ao=ao, weights=weights, fxc=_fortran(fxc), atom_offsets=offsets, window=window)


def make_mgga_grid(grid, den, seed=0, nspin=1, coupling=0.1):
    """Gradient-dependent XC data on an LDA grid: ``ao [ngrids, nao, 4]`` (the grid's values plus
    three seeded derivative components with the same AO windows) and ``fxc_eff`` of density type
    ``den`` ("sigma": nvar 4, "tau": nvar 5) -- ``[ngrids, nvar, nvar]`` (RKS) or
    ``[ngrids, nvar, 2, nvar, 2]`` (UKS), symmetric under ``(x, s_in) <-> (y, s_out)``, with the
    grid's LDA kernel in the density-density block and seeded couplings of relative size
    ``coupling`` elsewhere (the shapes of the reference's ``get_cached_ao(1)`` and
    ``intmd["cpks_fxc"]``)."""
    rng = np.random.default_rng(seed)
    ng, nao = grid.ao.shape
    nvar = {"sigma": 4, "tau": 5}[den]
    ao = np.zeros((ng, nao, 4), order="F")
    ao[:, :, 0] = grid.ao
    mask = grid.ao != 0.0
    for t in range(1, 4):
        ao[:, :, t] = np.where(mask, rng.standard_normal((ng, nao)) * np.abs(grid.ao).max(axis=0, keepdims=True), 0.0)
    if nspin == 1:
        f00 = np.asarray(grid.fxc).reshape(ng)
        x = rng.standard_normal((ng, nvar, nvar)) * coupling * np.abs(f00)[:, None, None]
        fxc = 0.5 * (x + x.transpose(0, 2, 1))
        fxc[:, 0, 0] = f00
    else:
        fl = np.asarray(grid.fxc).reshape(ng, 2, 2)
        x = rng.standard_normal((ng, nvar * 2, nvar * 2)) * coupling * np.abs(fl).max(axis=(1, 2))[:, None, None]
        x = 0.5 * (x + x.transpose(0, 2, 1))               # index (x, s) -> x + nvar s
        for si in range(2):
            for so in range(2):
                x[:, nvar * si, nvar * so] = fl[:, si, so]
        # [g, (x, s_in), (y, s_out)] -> [g, x, s_in, y, s_out]
        fxc = x.reshape(ng, 2, nvar, 2, nvar).transpose(0, 2, 1, 4, 3)
    return ao, np.asfortranarray(fxc)


class _PowerOperator:
    """Response on the vir-occ block, used only to set the synthetic scale (float32).

    Z-factored form: ``Z_P = B_P Cocc``, ``O_P = Cocc^T Z_P``;
    ``J C1 = 2 sum_P Z_P (2 <Z_P, C1>)``; ``K = -sum_P [B_P C1 O_P + Z_P (Z_P^T C1)^T]``.
    """

    def __init__(self, sysm):
        self.s = sysm
        nao, naux = sysm.nao, sysm.naux
        mu = np.concatenate([np.arange(nu + 1) for nu in range(nao)])
        nu = np.concatenate([np.full(nu + 1, nu) for nu in range(nao)])
        dense = np.zeros((naux, nao, nao), dtype=np.float32)
        chunk = max(1, (1 << 26) // (nao * nao))
        for p0 in range(0, naux, chunk):
            p1 = min(naux, p0 + chunk)
            blk = sysm.cderi[:, p0:p1].T.astype(np.float32)
            dense[p0:p1, mu, nu] = blk
            dense[p0:p1, nu, mu] = blk
        self.dense = dense                                   # [P, mu, nu]
        self.mocc = [sysm.mo_coeff[s][:, :sysm.nocc[s]].astype(np.float32) for s in range(sysm.nspin)]
        self.z = [(dense.reshape(naux * nao, nao) @ m).reshape(naux, nao, -1) for m in self.mocc]
        self.o = [np.einsum("ui,Puj->Pij", m, z, optimize=True) for m, z in zip(self.mocc, self.z)]

    def jk(self, c1):
        s = self.s
        ns = s.nspin
        naux, nao = s.naux, s.nao
        jfac = s.scale_j * (1.0 if ns == 1 else 0.5)
        d = sum(2.0 * np.einsum("Pui,ui->P", self.z[t], c1[t], optimize=True) for t in range(ns))
        out = []
        for t in range(ns):
            r = jfac * 2.0 * np.einsum("Pui,P->ui", self.z[t], d, optimize=True)
            y = (self.dense.reshape(naux * nao, nao) @ c1[t]).reshape(naux, nao, -1)
            r -= s.scale_k * np.einsum("Puj,Pij->ui", y, self.o[t], optimize=True)
            w = np.einsum("Pvi,vj->Pij", self.z[t], c1[t], optimize=True)
            r -= s.scale_k * np.einsum("Puj,Pij->ui", self.z[t], w, optimize=True)
            out.append(r)
        return out

    def xc(self, c1):
        s = self.s
        g = s.grid
        ns = s.nspin
        ao = g.ao.astype(np.float32)
        rho, aob = [], []
        for t in range(ns):
            ab = ao @ self.mocc[t]
            aob.append(ab)
            rho.append(np.einsum("gi,gi->g", ab, ao @ c1[t]))
        out = []
        for t in range(ns):
            if ns == 1:
                wv = g.weights * g.fxc * rho[0]
                fac = 4.0
            else:
                wv = g.weights * (g.fxc[:, 0, t] * rho[0] + g.fxc[:, 1, t] * rho[1])
                fac = 2.0
            out.append(fac * (ao.T @ (wv.astype(np.float32)[:, None] * aob[t])))
        return out

    def apply(self, parts, xvo):
        """xvo: per-spin [nvir, nocc] -> per-spin vir-occ response (not divided by gaps)."""
        s = self.s
        cv = [s.mo_coeff[t][:, s.nocc[t]:].astype(np.float32) for t in range(s.nspin)]
        c1 = [cv[t] @ xvo[t].astype(np.float32) for t in range(s.nspin)]
        acc = [np.zeros_like(c) for c in c1]
        if "jk" in parts:
            acc = [a + b for a, b in zip(acc, self.jk(c1))]
        if "xc" in parts:
            acc = [a + b for a, b in zip(acc, self.xc(c1))]
        return [(cv[t].T @ acc[t]).astype(np.float64) for t in range(s.nspin)]

    def norm(self, parts, rng, npower):
        s = self.s
        x = [rng.standard_normal((s.nmo[t] - s.nocc[t], s.nocc[t])) for t in range(s.nspin)]
        lam = 0.0
        for _ in range(npower):
            nrm = np.sqrt(sum(float((v * v).sum()) for v in x))
            x = [v / nrm for v in x]
            y = self.apply(parts, x)
            lam = np.sqrt(sum(float((v * v).sum()) for v in y))
            x = y
        return lam


def make_system(name_or_dims, seed=0, npower=8, scale_j=1.0, scale_k=None, grid_points=(8000, 14000)):
    """Build a seeded synthetic system from a workload name in :data:`CONFIGS` or a dims dict."""
    dims = dict(CONFIGS[name_or_dims]) if isinstance(name_or_dims, str) else dict(name_or_dims)
    nao, naux, natm = dims["nao"], dims["naux"], dims["natm"]
    nocc = tuple(dims["nocc"])
    nspin = len(nocc)
    if scale_k is None:
        scale_k = 0.5 if nspin == 1 else 1.0    # RHF exchange prefactor folded into scale_k
    rng = np.random.default_rng(seed)

    mo_coeff, mo_occ, mo_energy = [], [], []
    for s in range(nspin):
        q, _ = np.linalg.qr(rng.standard_normal((nao, nao)))
        mo_coeff.append(_fortran(q))
        eo = np.sort(rng.uniform(-20.0, -0.3, size=nocc[s]))
        ev = np.sort(rng.uniform(0.05, 5.0, size=nao - nocc[s]))
        mo_energy.append(np.concatenate([eo, ev]))
        occ = np.zeros(nao)
        occ[:nocc[s]] = 2.0 if nspin == 1 else 1.0
        mo_occ.append(occ)

    cderi = make_cderi(rng, nao, naux, dims.get("decay", 20.0))
    grid = None
    if dims.get("grid"):
        grid = make_grid(rng, nao, natm, dims.get("points", grid_points), dims.get("window", 80), nspin)

    rhs, f1mo, s1mo = [], [], []
    for s in range(nspin):
        no = nocc[s]
        eo = mo_energy[s][:no]
        e_ai = mo_energy[s][no:, None] - eo[None, :]
        s1 = 0.1 * rng.standard_normal((nao, no, 3, natm))
        r = np.empty((nao, no, 3, natm))
        r[no:] = 0.1 * rng.standard_normal((nao - no, no, 3, natm))
        r[:no] = -0.5 * s1[:no]
        f1 = np.empty_like(r)
        f1[no:] = -r[no:] * e_ai[:, :, None, None] + s1[no:] * eo[None, :, None, None]
        f1[:no] = 0.1 * rng.standard_normal((no, no, 3, natm))
        rhs.append(_fortran(r))
        f1mo.append(_fortran(f1))
        s1mo.append(_fortran(s1))

    sysm = System(nao=nao, naux=naux, natm=natm, nspin=nspin, cderi=cderi, mo_coeff=mo_coeff,
                  mo_occ=mo_occ, mo_energy=mo_energy, rhs=rhs, f1mo=f1mo, s1mo=s1mo,
                  scale_j=scale_j, scale_k=scale_k, grid=grid)

    gap = min(float(mo_energy[s][nocc[s]] - mo_energy[s][nocc[s] - 1]) for s in range(nspin))
    op = _PowerOperator(sysm)
    prng = np.random.default_rng(seed + 7919)
    norm_jk = op.norm(("jk",), prng, npower)
    norm_total = norm_jk
    if grid is not None:
        norm_xc = op.norm(("xc",), prng, npower)
        c = norm_jk / norm_xc
        grid.fxc *= c
        norm_total = 2.0 * norm_jk
    s2 = min(1.0, 0.5 * gap / norm_total)
    sysm.cderi *= np.sqrt(s2)
    sysm.scale_b = float(np.sqrt(s2))
    if grid is not None:
        grid.fxc *= s2
    sysm.info = dict(gap=gap, norm_jk=norm_jk, norm_total=norm_total, s2=s2, seed=seed)
    del op
    return sysm
