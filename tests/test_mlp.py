"""Learned initial guess / preconditioner: oracle self-checks (CPU) and the GPU kernels against
the oracle (forward, gradients), GPU training, and what the trained network gains."""

import numpy as np
import pytest

from conftest import rel_err
from oracle import mlp as omlp


def _toy_batch(n=300, seed=0):
    rng = np.random.default_rng(seed)
    feat = np.stack([rng.uniform(0.4, 25.0, n), 0.1 * rng.standard_normal(n), rng.uniform(0.0, 0.2, n)], axis=1)
    target = np.stack([feat[:, 1] / (1.0 + 0.3 * rng.random(n)), 0.3 * rng.random(n)], axis=1)
    return feat.astype(np.float32), target.astype(np.float32)


def test_oracle_gradient_matches_finite_differences():
    feat, target = _toy_batch(40)
    w = omlp.init_weights(1).astype(np.float64)
    w += 0.05 * np.random.default_rng(2).standard_normal(w.size)
    _, g = omlp.loss_and_grad(w, feat, target)
    rng = np.random.default_rng(3)
    for k in rng.choice(w.size, 25, replace=False):
        e = np.zeros_like(w)
        e[k] = 1e-6
        fd = (omlp.loss_and_grad(w + e, feat, target)[0] - omlp.loss_and_grad(w - e, feat, target)[0]) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-8


def test_training_targets():
    rng = np.random.default_rng(4)
    d = rng.uniform(0.0, 0.4, 50)
    x = rng.standard_normal((50, 7))
    b = x * (1.0 + d)[:, None]
    t1, t2 = omlp.training_targets(b, x)
    assert np.allclose(t2, d) and np.array_equal(t1, x)


# ---------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def ctx_mlp():
    from cphf_gb300 import Context, synth
    s = synth.make_system(dict(nao=48, naux=150, nocc=(8,), natm=4, decay=10.0), seed=21)
    ctx = Context(cphf_tol=1e-10)
    ctx.set_cderi(s.cderi, s.scale_j, s.scale_k)
    ctx.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])
    return s, ctx


@pytest.mark.gpu
def test_gpu_forward_and_gradient_match_oracle(ctx_mlp):
    s, ctx = ctx_mlp
    w = omlp.init_weights(5)
    w += (0.05 * np.random.default_rng(6).standard_normal(w.size)).astype(np.float32)
    ctx.set_mlp_weights(w)
    feat, target = _toy_batch(1000, seed=7)
    o_ref, _ = omlp.forward(w.astype(np.float64), feat)
    assert rel_err(ctx.mlp_forward(feat), o_ref) < 1e-5
    assert rel_err(ctx.mlp_forward(feat, bf16=True), o_ref) < 5e-2    # BF16 inference
    loss, g = ctx.mlp_loss_grad(feat, target)
    loss_ref, g_ref = omlp.loss_and_grad(w.astype(np.float64), feat, target)
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    assert rel_err(g, g_ref) < 1e-4


@pytest.mark.gpu
def test_gpu_features_match_definition(ctx_mlp):
    s, ctx = ctx_mlp
    feat = ctx.mlp_features(s.rhs[0])
    no, nmo = s.nocc[0], s.nao
    e = s.mo_energy[0]
    nvir = nmo - no
    nrhs = 3 * s.natm
    assert feat.shape == (nvir * no * nrhs, 3)
    gap = (e[no:, None] - e[None, :no]).reshape(-1, order="F")
    assert np.allclose(feat[:nvir * no, 0], gap, rtol=1e-6)
    assert np.allclose(feat[:, 1], s.rhs[0][no:].reshape(-1, order="F"), rtol=1e-6, atol=1e-9)
    # (ia|ia) = sum_P (C_a^T B_P C_i)^2
    from oracle.rijk import unpack_tri_sym
    cd = unpack_tri_sym(s.cderi, s.nao)
    C = s.mo_coeff[0]
    bmo = np.einsum("ua,uvP,vi->aiP", C[:, no:], cd, C[:, :no], optimize=True)
    iaia = (bmo ** 2).sum(axis=2).reshape(-1, order="F")
    assert rel_err(feat[:nvir * no, 2], iaia) < 1e-5


def _training_set(systems, ctx_factory):
    feats, targs = [], []
    for s in systems:
        ctx = ctx_factory(s)
        x = ctx.solve_dimless_cphf(s.rhs[0])
        f = ctx.mlp_features(s.rhs[0])
        no = s.nocc[0]
        nvir = s.nao - no
        nrhs = 3 * s.natm
        b = s.rhs[0][no:].reshape(nvir * no, nrhs, order="F")
        xv = x[no:].reshape(nvir * no, nrhs, order="F")
        t1, t2 = omlp.training_targets(b, xv)
        targs.append(np.stack([t1.reshape(-1, order="F"), np.repeat(t2[:, None], nrhs, 1).reshape(-1, order="F")],
                              axis=1))
        feats.append(f)
    return np.concatenate(feats).astype(np.float32), np.concatenate(targs).astype(np.float32)


@pytest.mark.gpu
def test_gpu_training_and_learned_solve_gain():
    """Train on solver-generated data; the learned guess/preconditioner must cut the Krylov
    cycles on held-out systems while the solution stays the FP64 one."""
    from cphf_gb300 import Context, synth

    def factory(s, **cfg):
        ctx = Context(**cfg)
        ctx.set_cderi(s.cderi, s.scale_j, s.scale_k)
        ctx.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])
        return ctx

    train = [synth.make_system(dict(nao=nao, naux=3 * nao, nocc=(nao // 8,), natm=4, decay=12.0), seed=100 + k)
             for k, nao in enumerate([56, 64, 72, 80, 88, 96])]
    feat, target = _training_set(train, lambda s: factory(s, cphf_tol=1e-10))
    trainer = factory(train[0])
    trainer.set_mlp_weights(omlp.init_weights(0))
    hist = trainer.mlp_train(feat, target, epochs=30, batch=2048, lr=3e-3, seed=1)
    assert hist[-1] < 0.5 * hist[0]
    w = trainer.mlp_weights()

    test = synth.make_system(dict(nao=104, naux=320, nocc=(13,), natm=4, decay=12.0), seed=999)
    base = factory(test, cphf_tol=1e-8)
    x_base = base.solve_dimless_cphf(test.rhs[0])
    cyc_base = base.last_stats["cycles"]
    learned = factory(test, cphf_tol=1e-8, use_learned_guess=1)
    learned.set_mlp_weights(w)
    x_learn = learned.solve_dimless_cphf(test.rhs[0])
    cyc_learn = learned.last_stats["cycles"]
    ref = factory(test, cphf_tol=1e-11).solve_dimless_cphf(test.rhs[0])
    assert np.abs(x_learn - ref).max() < 1e-7 and np.abs(x_base - ref).max() < 1e-7
    assert cyc_learn < cyc_base, (cyc_learn, cyc_base)
