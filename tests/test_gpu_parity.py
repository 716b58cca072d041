"""GPU parity: every libcphf entry point against the CPU oracle on the same seeded inputs.

Bars: FP64 plugin responses and driver steps agree with the oracle to 1e-12 relative
(max |diff| / max |ref|); FP64 solves to 1e-10 relative; the mixed-precision solve reaches
max_j ||b - (I+A)x||_2 < 1e-8 and its U1 and Hessian agree with FP64 within 1e-7.
"""

import numpy as np
import pytest

from conftest import load_golden, rel_err
from cphf_gb300 import Context, CphfError, KrylovNotConverged, synth
from oracle import cphf, krylov, rijk, xc

pytestmark = pytest.mark.gpu

MEDIUM = dict(nao=96, naux=300, nocc=(12,), natm=8, decay=12.0)
MEDIUM_U = dict(nao=80, naux=260, nocc=(11, 9), natm=6, decay=12.0)
GRID_R = dict(nao=64, naux=200, nocc=(9,), natm=4, decay=10.0, grid=True, points=(700, 1300), window=20)
GRID_U = dict(nao=60, naux=180, nocc=(8, 7), natm=4, decay=10.0, grid=True, points=(600, 1100), window=20)
# Split-FP16 operator of the inner solves (22-bit planes scaled per operand row, FP32
# accumulation, T and W re-split between contractions): ~1e-6 relative to FP64; its error is
# removed by the defect correction, whose final accuracy the mixed-solve tests check.
LOWP_TOL = 1e-5


def make_ctx(s, precision="fp64", **cfg):
    ctx = Context(precision=precision, **cfg)
    ctx.set_cderi(s.cderi, s.scale_j, s.scale_k)
    if s.grid is not None:
        ctx.set_grid(s.grid.ao, s.grid.weights, s.grid.fxc, s.nspin, s.grid.atom_offsets)
    if s.nspin == 1:
        ctx.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])
    else:
        ctx.make_response_preparation(s.mo_coeff, s.mo_occ, s.mo_energy)
    return ctx


def oracle_plugins(s):
    mocc = [s.mo_coeff[t][:, :s.nocc[t]] for t in range(s.nspin)]
    plugs = []
    if s.nspin == 1:
        plugs.append(lambda b: rijk.rhf_response_bra(s.cderi, s.mo_coeff[0], s.mo_occ[0], b, s.scale_j, s.scale_k))
        if s.grid is not None:
            g = s.grid
            plugs.append(lambda b: xc.rks_response_bra(g.ao, g.weights, g.fxc, b, mocc[0]))
    else:
        plugs.append(lambda b: rijk.uhf_response_bra(s.cderi, s.mo_coeff, s.mo_occ, b, s.scale_j, s.scale_k))
        if s.grid is not None:
            g = s.grid
            plugs.append(lambda b: xc.uks_response_bra(g.ao, g.weights, g.fxc, b, mocc))
    return plugs


def oracle_driver(s, **cfg):
    if s.nspin == 1:
        return cphf.RHF(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0], oracle_plugins(s), s.natm, config=cfg)
    return cphf.UHF(s.mo_coeff, s.mo_occ, s.mo_energy, oracle_plugins(s), s.natm, config=cfg)


@pytest.fixture(scope="module")
def med():
    s = synth.make_system(MEDIUM, seed=7)
    return s, make_ctx(s)


@pytest.mark.parametrize("dims,seed", [("rhf_nao24", 1), (MEDIUM, 7)])
def test_rijk_response_bra_rhf(dims, seed):
    s = synth.make_system(dims, seed=seed)
    ctx = make_ctx(s)
    bra = np.random.default_rng(seed).standard_normal((s.nao, s.nocc[0], 7))
    got = ctx.get_response_bra(bra)
    ref = rijk.rhf_response_bra(s.cderi, s.mo_coeff[0], s.mo_occ[0], bra, s.scale_j, s.scale_k)
    assert rel_err(got, ref) < 1e-12


def test_rijk_response_matches_reference_golden():
    g = load_golden("rhf_nao24_seed1.npz")
    ctx = Context()
    ctx.set_cderi(g["cderi"], float(g["scale_j"]), float(g["scale_k"]))
    ctx.make_response_preparation(g["mo_coeff"], g["mo_occ"], g["mo_energy"])
    assert rel_err(ctx.get_response_bra(g["bra_probe"]), g["resp_probe"]) < 1e-12


@pytest.mark.parametrize("sj,sk", [(1.0, 0.0), (0.0, 0.7), (1.3, 0.25)])
def test_rijk_scales_and_j_or_k_only(sj, sk):
    s = synth.make_system(MEDIUM, seed=8, scale_j=sj, scale_k=sk)
    ctx = make_ctx(s)
    bra = np.random.default_rng(2).standard_normal((s.nao, s.nocc[0], 3))
    ref = rijk.rhf_response_bra(s.cderi, s.mo_coeff[0], s.mo_occ[0], bra, sj, sk)
    assert rel_err(ctx.get_response_bra(bra), ref) < 1e-12


def test_rijk_k_term_aux_chunking():
    s = synth.make_system(MEDIUM, seed=9)
    ctx = make_ctx(s, aux_chunk=37)   # ragged last chunk
    bra = np.random.default_rng(3).standard_normal((s.nao, s.nocc[0], 5))
    ref = rijk.rhf_response_bra(s.cderi, s.mo_coeff[0], s.mo_occ[0], bra, s.scale_j, s.scale_k)
    assert rel_err(ctx.get_response_bra(bra), ref) < 1e-12


def test_rijk_response_bra_uhf():
    s = synth.make_system(MEDIUM_U, seed=4)
    ctx = make_ctx(s)
    rng = np.random.default_rng(4)
    bra = [rng.standard_normal((s.nao, s.nocc[t], 6)) for t in range(2)]
    got = ctx.get_response_bra(bra)
    ref = rijk.uhf_response_bra(s.cderi, s.mo_coeff, s.mo_occ, bra, s.scale_j, s.scale_k)
    for t in range(2):
        assert rel_err(got[t], ref[t]) < 1e-12


def test_xc_response_rks():
    s = synth.make_system(GRID_R, seed=5)
    ctx = make_ctx(s)
    bra = np.random.default_rng(5).standard_normal((s.nao, s.nocc[0], 4))
    g = s.grid
    ref = xc.rks_response_bra(g.ao, g.weights, g.fxc, bra, s.mo_coeff[0][:, :s.nocc[0]])
    assert rel_err(ctx.get_response_bra(bra, plugin="xc"), ref) < 1e-12
    both = ref + rijk.rhf_response_bra(s.cderi, s.mo_coeff[0], s.mo_occ[0], bra, s.scale_j, s.scale_k)
    assert rel_err(ctx.get_response_bra(bra), both) < 1e-12


@pytest.mark.parametrize("chunk", [900, 2500])
def test_xc_response_chunked_grouped(chunk):
    """Uneven per-atom batches split over several chunks of the grouped XC kernels."""
    s = synth.make_system(GRID_R, seed=15)
    ctx = make_ctx(s, xc_chunk_points=chunk)
    bra = np.random.default_rng(15).standard_normal((s.nao, s.nocc[0], 3))
    g = s.grid
    ref = xc.rks_response_bra(g.ao, g.weights, g.fxc, bra, s.mo_coeff[0][:, :s.nocc[0]])
    assert rel_err(ctx.get_response_bra(bra, plugin="xc"), ref) < 1e-12
    lp = make_ctx(s, precision="mixed", xc_chunk_points=chunk)
    mo1 = np.random.default_rng(16).standard_normal((s.nao, s.nocc[0], 3))
    assert rel_err(lp.response_dimless_cphf_lowp(mo1), ctx.response_dimless_cphf(mo1)) < LOWP_TOL


def test_xc_response_uks():
    s = synth.make_system(GRID_U, seed=6)
    ctx = make_ctx(s)
    rng = np.random.default_rng(6)
    bra = [rng.standard_normal((s.nao, s.nocc[t], 3)) for t in range(2)]
    g = s.grid
    ref = xc.uks_response_bra(g.ao, g.weights, g.fxc, bra, [s.mo_coeff[t][:, :s.nocc[t]] for t in range(2)])
    got = ctx.get_response_bra(bra, plugin="xc")
    for t in range(2):
        assert rel_err(got[t], ref[t]) < 1e-12


@pytest.mark.parametrize("dims", [MEDIUM, MEDIUM_U, GRID_R])
def test_response_mo_and_dimless(dims):
    s = synth.make_system(dims, seed=10)
    ctx = make_ctx(s)
    drv = oracle_driver(s)
    rng = np.random.default_rng(10)
    if s.nspin == 1:
        mo1 = rng.standard_normal((s.nao, s.nocc[0], 4))
        assert rel_err(ctx.response_mo(mo1), drv.response_mo(mo1)) < 1e-12
        assert rel_err(ctx.response_dimless_cphf(mo1), drv.response_dimless_cphf(mo1)) < 1e-12
    else:
        mo1 = [rng.standard_normal((s.nao, s.nocc[t], 4)) for t in range(2)]
        for a, b in zip(ctx.response_dimless_cphf(mo1), drv.response_dimless_cphf(mo1)):
            assert rel_err(a, b) < 1e-12


def test_solve_finalize_hess_rhf_golden():
    """The whole CPHF chain against the reference Python driver's golden vectors."""
    g = load_golden("rhf_nao24_seed1.npz")
    ctx = Context(cphf_tol=1e-10, cphf_max_cycle=30)
    ctx.set_cderi(g["cderi"], float(g["scale_j"]), float(g["scale_k"]))
    ctx.make_response_preparation(g["mo_coeff"], g["mo_occ"], g["mo_energy"])
    mo1 = ctx.solve_dimless_cphf(g["rhs"])
    nocc = int((g["mo_occ"] > 0).sum())
    assert rel_err(mo1[nocc:], g["mo1_solved"][nocc:]) < 1e-8
    mo1f, mo_e1 = ctx.finalize_cphf(g["f1mo"], g["s1mo"], g["mo1_solved"])
    assert rel_err(mo1f, g["mo1"]) < 1e-11
    assert rel_err(mo_e1, g["mo_e1"]) < 1e-11
    de = ctx.get_cphf_hess(g["f1mo"], g["s1mo"], g["mo1"], g["mo_e1"])
    assert rel_err(de, g["de_cphf"]) < 1e-12


@pytest.mark.parametrize("dims", [MEDIUM, MEDIUM_U, GRID_R, GRID_U])
def test_solve_dimless_cphf_fp64_matches_oracle(dims):
    s = synth.make_system(dims, seed=12)
    ctx = make_ctx(s, cphf_tol=1e-10)
    drv = oracle_driver(s, cphf_tol=1e-10)
    rhs = s.rhs[0] if s.nspin == 1 else s.rhs
    got = ctx.solve_dimless_cphf(rhs)
    ref = drv.solve_dimless_cphf(rhs)
    st = ctx.last_stats
    assert st["aop_calls"] == drv.krylov_stats["aop_calls"]
    if s.nspin == 1:
        got, ref = [got], [ref]
    for a, b in zip(got, ref):
        assert rel_err(a, b) < 1e-10
    f1 = s.f1mo[0] if s.nspin == 1 else s.f1mo
    s1 = s.s1mo[0] if s.nspin == 1 else s.s1mo
    m1 = got[0] if s.nspin == 1 else got
    mf, me = ctx.finalize_cphf(f1, s1, m1)
    rf, re_ = drv.finalize_cphf(f1, s1, m1)
    if s.nspin == 1:
        mf, me, rf, re_ = [mf], [me], [rf], [re_]
    for a, b in zip(mf, rf):
        assert rel_err(a, b) < 1e-11
    for a, b in zip(me, re_):
        assert rel_err(a, b) < 1e-11
    de = ctx.get_cphf_hess(f1, s1, mf[0] if s.nspin == 1 else mf, me[0] if s.nspin == 1 else me)
    ref_de = drv.get_cphf_hess(f1, s1, rf[0] if s.nspin == 1 else rf, re_[0] if s.nspin == 1 else re_)
    assert rel_err(de, ref_de) < 1e-11


TC_RAGGED = dict(nao=150, naux=70, nocc=(13,), natm=9, decay=12.0)
# more than 128 occupied orbitals: the inner T generation leaves the bra-resident kernel for the
# batched one (K = nocc over more than four blocks of 32)
TC_WIDE_OCC = dict(nao=176, naux=60, nocc=(136,), natm=2, decay=12.0)


@pytest.mark.parametrize("tc", [1, 0])
@pytest.mark.parametrize("dims", [MEDIUM, TC_RAGGED, TC_WIDE_OCC, MEDIUM_U, GRID_R, GRID_U])
def test_lowp_operator_accuracy(dims, tc):
    """The split-precision operator of the mixed solve agrees with FP64 to LOWP_TOL."""
    s = synth.make_system(dims, seed=14)
    c64 = make_ctx(s)
    clp = make_ctx(s, precision="mixed", tensor_cores=tc)
    clp.profile(True)
    rng = np.random.default_rng(14)
    if s.nspin == 1:
        mo1 = rng.standard_normal((s.nao, s.nocc[0], 5))
        ref, got = [c64.response_dimless_cphf(mo1)], [clp.response_dimless_cphf_lowp(mo1)]
    else:
        mo1 = [rng.standard_normal((s.nao, s.nocc[t], 5)) for t in range(2)]
        ref, got = c64.response_dimless_cphf(mo1), clp.response_dimless_cphf_lowp(mo1)
    for a, b in zip(got, ref):
        assert rel_err(a, b) < LOWP_TOL
    if tc:
        classes = ["kterm_tcgen05_f16x3", "tgen_tcgen05_f16x3", "wgen_tcgen05_f16x3", "term2_tcgen05_f16x3"]
        if s.grid is not None:
            classes.append("xc_tcgen05_f16x3")
        assert_tensor_core_classes(clp, classes)
    else:
        assert not clp.tensor_cores_active
        assert "kterm_tcgen05_f16x3" not in clp.profile_report()


def assert_correction_classes(ctx):
    """Some residual update ran on the exact-slice operator in correction precision (3 or 4
    slices), all four of its contractions on tcgen05."""
    rep = ctx.profile_report()
    assert any(rep.get(f"kterm_tcgen05_bf16x{k}c_exact", {}).get("launches", 0) > 0 for k in (3, 4)), sorted(rep)
    for part in ("kterm", "tgen", "wgen", "term2"):
        assert sum(rep.get(f"{part}_tcgen05_bf16x{k}c_exact", {}).get("launches", 0) for k in (3, 4)) > 0, part


def assert_tensor_core_classes(ctx, classes):
    """The context ran its split-precision / exact-slice contractions on tcgen05: the tensor
    cores are active and each named kernel class of the CUDA-event profiler has launches."""
    assert ctx.tensor_cores_active
    rep = ctx.profile_report()
    for name in classes:
        assert rep.get(name, {}).get("launches", 0) > 0, (name, sorted(rep))


def _max_col_residual(c64, s, x):
    """max_j ||b_j - (I + A) x_j||_2 with the native FP64 operator."""
    rhs = [s.rhs[0]] if s.nspin == 1 else s.rhs
    xs = [x] if s.nspin == 1 else x
    y = c64.response_dimless_cphf(x)
    y = [y] if s.nspin == 1 else y
    r = np.concatenate([(b - a - yy).reshape(-1, b.shape[2] * b.shape[3], order="F")
                        for b, a, yy in zip(rhs, xs, y)], axis=0)
    return float(np.linalg.norm(r, axis=0).max()), float(max(np.abs(a).max() for a in xs))


@pytest.mark.parametrize("dims", [MEDIUM, TC_RAGGED, MEDIUM_U, GRID_R])
@pytest.mark.parametrize("mode", [1, 2])
def test_emulated_fp64_residual(dims, mode):
    """The residual of the mixed solve's first correction, computed with the emulated FP64
    operator (mode 1: double-float GEMMs, XC included; mode 2: plus the K term on the tensor
    cores with exact BF16 slices, chunked over aux functions), matches the native FP64 residual of the
    same x to 1e-9 relative to max |x| (the split-FP16 operator of the inner solves is ~1e-6)."""
    s = synth.make_system(dims, seed=15)
    rhs = s.rhs[0] if s.nspin == 1 else s.rhs
    c64 = make_ctx(s)
    cmx = make_ctx(s, precision="mixed", residual_dfloat=mode, max_refine=1, residual_tol=1.0, verify_residual=0,
                   aux_chunk=16)
    cmx.profile(True)
    x = cmx.solve_dimless_cphf(rhs)
    res_emul = cmx.last_stats["residual_max"]
    assert cmx.last_stats["residual_mode"] == mode
    if mode == 2:
        classes = ["kterm_tcgen05_bf16x6_exact", "tgen_tcgen05_bf16x6_exact", "wgen_tcgen05_bf16x6_exact",
                   "term2_tcgen05_bf16x6_exact"]
        if s.grid is not None:
            classes.append("xc_tcgen05_bf16x6_exact")
        assert_tensor_core_classes(cmx, classes)
    res_64, xmax = _max_col_residual(c64, s, x)
    assert 1e-9 < res_64 < 1e-3            # a real, unconverged residual of the low-precision step
    assert abs(res_emul - res_64) < 1e-9 * max(1.0, xmax), (res_emul, res_64, xmax)


@pytest.mark.parametrize("dims,dfloat", [(MEDIUM, 1), (MEDIUM, 0), (GRID_U, 1), (TC_RAGGED, 1), (MEDIUM, 2),
                                         (TC_RAGGED, 2), (GRID_U, 2)])
def test_mixed_precision_solve(dims, dfloat):
    s = synth.make_system(dims, seed=13)
    rhs = s.rhs[0] if s.nspin == 1 else s.rhs
    c64 = make_ctx(s, cphf_tol=1e-10, cphf_lindep=1e-20)
    x64 = c64.solve_dimless_cphf(rhs)
    cmx = make_ctx(s, precision="mixed", residual_dfloat=dfloat)
    cmx.profile(dfloat == 2)
    xmx = cmx.solve_dimless_cphf(rhs)
    st = cmx.last_stats
    assert st["residual_max"] < 1e-8
    assert st["refine_steps"] >= 1 and st["lowp_matvec_columns"] > 0
    nset = 3 * s.natm
    # every correction's residual is recomputed with the FP64-accurate operator (the solve's own
    # final check, verify_residual = 2); convergence is decided on that recomputed residual
    assert st["fp64_matvec_columns"] == st["refine_steps"] * nset
    # exact slices: the first correction's residual recomputed in full, later corrections
    # subtracted with the exact-slice operator in correction precision (residual mode 4)
    assert st["residual_mode"] == (4 if dfloat == 2 and st["refine_steps"] > 1 else dfloat)
    if dfloat == 2:
        assert_tensor_core_classes(cmx, ["kterm_tcgen05_f16x3", "kterm_tcgen05_bf16x6_exact"])
        if st["refine_steps"] > 1:
            assert_correction_classes(cmx)
    res64, xmax = _max_col_residual(c64, s, xmx)
    assert res64 < 1e-8
    # the solve's own final residual agrees with the native FP64 residual of its answer
    assert abs(st["residual_max"] - res64) < 1e-9 * max(1.0, xmax), (st["residual_max"], res64)
    if s.nspin == 1:
        x64, xmx = [x64], [xmx]
    for a, b in zip(xmx, x64):
        assert np.abs(a - b).max() < 1e-7
    f1 = s.f1mo[0] if s.nspin == 1 else s.f1mo
    s1 = s.s1mo[0] if s.nspin == 1 else s.s1mo
    h = []
    for ctx, x in [(c64, x64), (cmx, xmx)]:
        m1, me = ctx.finalize_cphf(f1, s1, x[0] if s.nspin == 1 else x)
        h.append(ctx.get_cphf_hess(f1, s1, m1, me))
    assert np.abs(h[0] - h[1]).max() < 1e-7


@pytest.mark.parametrize("dims", [MEDIUM, TC_RAGGED, MEDIUM_U, GRID_R, GRID_U])
def test_correction_precision_residual(dims):
    """Loose inner solves force several defect-correction steps: every later residual is the
    previous one minus (I + A) d on the exact-slice operator in correction precision (residual
    mode 4), and the solve's own final residual still agrees with the native FP64 residual."""
    s = synth.make_system(dims, seed=21)
    rhs = s.rhs[0] if s.nspin == 1 else s.rhs
    c64 = make_ctx(s)
    cmx = make_ctx(s, precision="mixed", residual_dfloat=2, inner_tol=1e-3)
    cmx.profile(True)
    x = cmx.solve_dimless_cphf(rhs)
    st = cmx.last_stats
    assert st["refine_steps"] >= 2 and st["residual_mode"] == 4
    assert st["residual_max"] < 1e-8
    assert_tensor_core_classes(cmx, ["kterm_tcgen05_bf16x6_exact"])
    assert_correction_classes(cmx)
    if s.grid is not None:  # the XC grid contractions of the corrections in correction precision too
        assert_tensor_core_classes(cmx, ["xc_tcgen05_bf16x6_exact", "xc_tcgen05_bf16c_exact"])
    res64, xmax = _max_col_residual(c64, s, x)
    assert res64 < 1e-8
    assert abs(st["residual_max"] - res64) < 1e-9 * max(1.0, xmax), (st["residual_max"], res64)


@pytest.mark.parametrize("dims", [MEDIUM, GRID_U])
def test_mixed_solve_cuda_graphs(dims):
    """Inner operator replayed from captured CUDA graphs (one per block width, two solves so
    the second replays every width) gives the eager operator's solution."""
    s = synth.make_system(dims, seed=17)
    rhs = s.rhs[0] if s.nspin == 1 else s.rhs
    eager = make_ctx(s, precision="mixed", cuda_graphs=0)
    graph = make_ctx(s, precision="mixed", cuda_graphs=1)
    x0 = eager.solve_dimless_cphf(rhs)
    for _ in range(2):
        x1 = graph.solve_dimless_cphf(rhs)
        assert graph.last_stats["residual_max"] < 1e-8
        for a, b in zip([x1] if s.nspin == 1 else x1, [x0] if s.nspin == 1 else x0):
            assert np.abs(a - b).max() < 1e-9


def test_gpu_krylov_reference_fixture():
    """tests/test_krylov_block.rs:7-97 through the device solver (dense operator on the GPU)."""
    z = load_golden("krylov_fixture.npz")
    A, b, x_ref = z["A"], z["b"].T.copy(), z["x_ref"].T.copy()
    ctx = Context()
    x = ctx.krylov_block(A, b, None, 1e-10, 30, 6, 1e-13)
    assert np.allclose(x, x_ref, rtol=1e-6, atol=1e-8)
    assert np.abs(x + A @ x - b).max() < 1e-6
    assert ctx.last_stats["aop_calls"] == int(z["calls_ms6"])
    xr = ctx.krylov_block(A, b, None, 1e-10, 60, 3, 1e-13)
    assert ctx.last_stats["restarts"] >= 1
    assert np.allclose(xr, x_ref, rtol=1e-5, atol=1e-6)
    ox = krylov.krylov_block(lambda v: A @ v, b, None, 1e-10, 60, 3, 1e-13)
    assert np.abs(xr - ox).max() < 1e-8
    with pytest.raises(KrylovNotConverged):
        ctx.krylov_block(A, b, None, 1e-10, 2, 14, 1e-13)


def test_gpu_krylov_host_callback_operator():
    z = load_golden("krylov_fixture.npz")
    A, b = z["A"], z["b"].T.copy()
    ctx = Context()
    x = ctx.krylov_block(lambda v: A @ v, b, None, 1e-10, 30, 6, 1e-13)
    ox = krylov.krylov_block(lambda v: A @ v, b, None, 1e-10, 30, 6, 1e-13)
    assert np.abs(x - ox).max() < 1e-8


def test_errors_are_status_codes(med):
    s, ctx = med
    bad = s.rhs[0].copy()
    bad[3, 1, 0, 0] = np.nan
    with pytest.raises(CphfError) as e:
        ctx.solve_dimless_cphf(bad)
    assert e.value.status == 3
    with pytest.raises(KrylovNotConverged):
        c2 = make_ctx(s, cphf_max_cycle=1)
        c2.solve_dimless_cphf(s.rhs[0])
    with pytest.raises(CphfError) as e:
        Context().get_response_bra(np.zeros((4, 2, 1)))
    assert e.value.status in (7, 8)


def test_empty_and_single_column(med):
    s, ctx = med
    one = ctx.get_response_bra(np.ones((s.nao, s.nocc[0], 1)))
    ref = rijk.rhf_response_bra(s.cderi, s.mo_coeff[0], s.mo_occ[0], np.ones((s.nao, s.nocc[0], 1)),
                                s.scale_j, s.scale_k)
    assert rel_err(one, ref) < 1e-12
    zero = ctx.get_response_bra(np.zeros((s.nao, s.nocc[0], 0)))
    assert zero.shape == (s.nao, s.nocc[0], 0)
    x = ctx.solve_dimless_cphf(np.zeros((s.nao, s.nocc[0], 2)))
    assert np.all(x == 0.0)


@pytest.mark.parametrize("name", ["xc_rks_nao30_seed3.npz", "xc_uks_nao28_seed4.npz"])
def test_xc_plugin_matches_reference_wrapper_golden(name):
    """The XC plugin (FP64 grouped kernels, and the mixed context's split-precision operator)
    against the reference's own XC response wrappers (get_ks_response_bra_naive /
    get_uks_response_bra_naive, tests/golden/make_golden.py)."""
    g = load_golden(name)
    nspin = int(g["nspin"])
    C = [g[f"mo_coeff{t}"] for t in range(nspin)]
    occ = [g[f"mo_occ{t}"] for t in range(nspin)]
    e = [g[f"mo_energy{t}"] for t in range(nspin)]
    bra = [g[f"bra{t}"] for t in range(nspin)]
    ref = [g[f"resp{t}"] for t in range(nspin)]
    arg = (lambda v: v[0]) if nspin == 1 else (lambda v: v)
    for with_rijk in (False, True):
        ctx = Context()
        if with_rijk:
            ctx.set_cderi(g["cderi"], float(g["scale_j"]), float(g["scale_k"]))
        else:
            ctx.set_nao(C[0].shape[0])
        ctx.set_grid(g["ao"], g["weights"], g["fxc"], nspin, g["atom_offsets"])
        ctx.make_response_preparation(arg(C), arg(occ), arg(e))
        got = ctx.get_response_bra(arg(bra), plugin="xc")
        got = [got] if nspin == 1 else got
        for a, b in zip(got, ref):
            assert rel_err(a, b) < 1e-12


def test_fp64_operator_matches_oracle_at_nao600():
    """The FP64 dimensionless operator at nao=600 / naux=2000 / nocc=60 (the 180-RHS workload),
    on a few columns, against the CPU oracle's response_dimless_cphf: 1e-12 relative."""
    s = synth.make_system("rhf_nao600", seed=0)
    ctx = make_ctx(s)
    drv = oracle_driver(s)
    mo1 = np.random.default_rng(600).standard_normal((s.nao, s.nocc[0], 3))
    assert rel_err(ctx.response_dimless_cphf(mo1), drv.response_dimless_cphf(mo1)) < 1e-12
    bra = np.random.default_rng(601).standard_normal((s.nao, s.nocc[0], 2))
    ref = rijk.rhf_response_bra(s.cderi, s.mo_coeff[0], s.mo_occ[0], bra, s.scale_j, s.scale_k)
    assert rel_err(ctx.get_response_bra(bra), ref) < 1e-12


def _bad_weights():
    """MLP weights whose outputs are far off: a guess x0 = b (1 + o1) several times too large and
    preconditioner entries m = 1 / (1 + o2) spread over two orders of magnitude."""
    from oracle import mlp as omlp
    d = omlp.unpack(omlp.init_weights(3).astype(np.float64))
    d["W3"] = 3.0 * np.random.default_rng(33).standard_normal(d["W3"].shape)
    d["b3"] = np.array([5.0, 30.0])
    return omlp.pack(d).astype(np.float32)


@pytest.mark.parametrize("dims,mode", [(MEDIUM, 1), (MEDIUM, 2), (MEDIUM_U, 1), (MEDIUM_U, 2)])
def test_mixed_solve_with_bad_learned_preconditioner(dims, mode):
    """A deliberately bad network costs iterations, never accuracy: the mixed solve's outer
    FP64-accurate residual still decides convergence to ||b - (I+A)x|| < 1e-8 (one- and
    two-spin solves; uscf.rs:278-341 goes through the same x0 hook)."""
    s = synth.make_system(dims, seed=31)
    c64 = make_ctx(s)
    cmx = make_ctx(s, precision="mixed", use_learned_guess=mode)
    cmx.set_mlp_weights(_bad_weights())
    x = cmx.solve_dimless_cphf(s.rhs[0] if s.nspin == 1 else s.rhs)
    assert cmx.last_stats["residual_max"] < 1e-8
    res64, _ = _max_col_residual(c64, s, x)
    assert res64 < 1e-8


def test_fp64_solve_with_bad_learned_guess():
    """On an FP64 context the network only supplies x0; the Krylov iteration and its stopping test
    are the reference's, so a bad guess still converges to the plain solution."""
    s = synth.make_system(MEDIUM, seed=32)
    # lindep below tol^2, so that the trial-norm stopping test (max(lindep, tol^2)) is tol's
    base = make_ctx(s, cphf_tol=1e-11, cphf_lindep=1e-24)
    x_ref = base.solve_dimless_cphf(s.rhs[0])
    bad = make_ctx(s, cphf_tol=1e-11, cphf_lindep=1e-24, use_learned_guess=1)
    bad.set_mlp_weights(_bad_weights())
    x = bad.solve_dimless_cphf(s.rhs[0])
    assert np.abs(x[s.nocc[0]:] - x_ref[s.nocc[0]:]).max() < 1e-8
    res64, _ = _max_col_residual(base, s, x)
    assert res64 < 1e-8


@pytest.mark.parametrize("name", ["rhs_rhf_nao22_seed5.npz", "rhs_uhf_nao22_seed6.npz"])
def test_compute_dimless_cphf_rhs_golden(name):
    """The GPU right-hand-side assembly against pyhessref's compute_dimensionless_cphf_rhs."""
    g = load_golden(name)
    nspin = int(g["nspin"])
    arg = (lambda v: v[0]) if nspin == 1 else (lambda v: v)
    ctx = Context()
    ctx.set_nao(g["mo_coeff0"].shape[0])
    ctx.make_response_preparation(arg([g[f"mo_coeff{t}"] for t in range(nspin)]),
                                  arg([g[f"mo_occ{t}"] for t in range(nspin)]),
                                  arg([g[f"mo_energy{t}"] for t in range(nspin)]))
    rhs, f1, s1 = ctx.compute_dimless_cphf_rhs(g["f1ao_core"], arg([g[f"f1bra_el{t}"] for t in range(nspin)]),
                                               g["s1ao"])
    if nspin == 1:
        rhs, f1, s1 = [rhs], [f1], [s1]
    for t in range(nspin):
        assert rel_err(rhs[t], g[f"rhs{t}"]) < 1e-12
        assert rel_err(f1[t], g[f"f1mo{t}"]) < 1e-12
        assert rel_err(s1[t], g[f"s1mo{t}"]) < 1e-12
    # without the electron-interaction part (f1bra_el = NULL)
    rhs0, f10, s10 = ctx.compute_dimless_cphf_rhs(g["f1ao_core"], None, g["s1ao"])
    r_ref, f_ref, s_ref = cphf.compute_dimless_cphf_rhs(g["mo_coeff0"], g["mo_occ0"], g["mo_energy0"], g["f1ao_core"],
                                                        None, g["s1ao"])
    assert rel_err(rhs0 if nspin == 1 else rhs0[0], r_ref) < 1e-12
    assert rel_err(f10 if nspin == 1 else f10[0], f_ref) < 1e-12


GRID_MG = dict(nao=56, naux=170, nocc=(8,), natm=4, decay=10.0, grid=True, points=(500, 900), window=18)
GRID_MG_U = dict(nao=52, naux=160, nocc=(7, 6), natm=4, decay=10.0, grid=True, points=(500, 900), window=18)


def _mgga_ctx(s, den, precision="fp64", coupling=0.1, fxc_scale=1.0, **cfg):
    ao, fxc = synth.make_mgga_grid(s.grid, den, seed=41, nspin=s.nspin, coupling=coupling)
    fxc = fxc * fxc_scale
    ctx = Context(precision=precision, **cfg)
    ctx.set_cderi(s.cderi, s.scale_j, s.scale_k)
    ctx.set_grid_ex(den, ao, s.grid.weights, fxc, s.nspin)
    if s.nspin == 1:
        ctx.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])
    else:
        ctx.make_response_preparation(s.mo_coeff, s.mo_occ, s.mo_energy)
    return ctx, ao, fxc


@pytest.mark.parametrize("dims,den", [(GRID_MG, "sigma"), (GRID_MG, "tau"), (GRID_MG_U, "sigma"), (GRID_MG_U, "tau")])
def test_xc_gga_mgga_response(dims, den):
    """SIGMA (GGA) and TAU (meta-GGA) XC response of the plugin against the oracle's restatement
    of pure_eval_rho.rs:289-316 / pure_xcpot.rs:335-351 (1e-12), and the split-precision form."""
    s = synth.make_system(dims, seed=40)
    ctx, ao, fxc = _mgga_ctx(s, den, xc_chunk_points=777)   # ragged point chunks
    rng = np.random.default_rng(42)
    g = s.grid
    if s.nspin == 1:
        bra = rng.standard_normal((s.nao, s.nocc[0], 5))
        ref = [xc.rks_response_bra_mgga(ao, g.weights, fxc, bra, s.mo_coeff[0][:, :s.nocc[0]], den)]
        got = [ctx.get_response_bra(bra, plugin="xc")]
    else:
        bra = [rng.standard_normal((s.nao, s.nocc[t], 5)) for t in range(2)]
        ref = xc.uks_response_bra_mgga(ao, g.weights, fxc, bra, [s.mo_coeff[t][:, :s.nocc[t]] for t in range(2)], den)
        got = ctx.get_response_bra(bra, plugin="xc")
    for a, b in zip(got, ref):
        assert rel_err(a, b) < 1e-12
    lp, _, _ = _mgga_ctx(s, den, precision="mixed")
    mo1 = [rng.standard_normal((s.nao, s.nocc[t], 4)) for t in range(s.nspin)]
    arg = (lambda v: v[0]) if s.nspin == 1 else (lambda v: v)
    r64 = ctx.response_dimless_cphf(arg(mo1))
    rlp = lp.response_dimless_cphf_lowp(arg(mo1))
    for a, b in zip([rlp] if s.nspin == 1 else rlp, [r64] if s.nspin == 1 else r64):
        assert rel_err(a, b) < LOWP_TOL


def test_xc_set_grid_ex_rho_is_lda():
    """den_type RHO through the general entry point is the LDA plugin on component 0."""
    s = synth.make_system(GRID_R, seed=43)
    g = s.grid
    ctx = make_ctx(s)
    ex = Context()
    ex.set_cderi(s.cderi, s.scale_j, s.scale_k)
    ao4 = np.asfortranarray(np.stack([g.ao] * 4, axis=2))
    ex.set_grid_ex("rho", ao4, g.weights, g.fxc, 1, g.atom_offsets)
    ex.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])
    bra = np.random.default_rng(44).standard_normal((s.nao, s.nocc[0], 3))
    assert rel_err(ex.get_response_bra(bra, plugin="xc"), ctx.get_response_bra(bra, plugin="xc")) < 1e-13


@pytest.mark.parametrize("dims", [GRID_MG, GRID_MG_U])
def test_mixed_solve_gga(dims):
    """Mixed-precision CPKS solve with a GGA kernel: the solve's own residual and the native FP64
    residual both below 1e-8, U1 within 1e-7 of the plain FP64 solve."""
    s = synth.make_system(dims, seed=45)
    rhs = s.rhs[0] if s.nspin == 1 else s.rhs
    c64, _, _ = _mgga_ctx(s, "sigma", fxc_scale=0.5, cphf_tol=1e-10, cphf_lindep=1e-22)
    x64 = c64.solve_dimless_cphf(rhs)
    cmx, _, _ = _mgga_ctx(s, "sigma", precision="mixed", fxc_scale=0.5)
    xmx = cmx.solve_dimless_cphf(rhs)
    assert cmx.last_stats["residual_max"] < 1e-8
    res64, _ = _max_col_residual(c64, s, xmx)
    assert res64 < 1e-8
    for a, b in zip([xmx] if s.nspin == 1 else xmx, [x64] if s.nspin == 1 else x64):
        assert np.abs(a - b).max() < 1e-7
