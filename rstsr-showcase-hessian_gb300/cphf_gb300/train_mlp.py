"""Train the learned initial guess / preconditioner on solver-generated data (GPU).

For a set of seeded synthetic RHF systems (the generators of ``synth``), the library
solves the CPHF equations (mixed precision, FP64-verified residual < 1e-8); every
(vir a, occ i, right-hand side r) sample gives features (gap, b, (ia|ia)) and targets
(x*, d*) where d* is the pair's effective diagonal (x* ~ b / (1 + d*) in least squares over
the right-hand sides).  The network is trained with the library's own forward/backward
kernels and Adam (``Context.mlp_train``) and the weights are written to ``mlp_weights.npy``
next to this file.

Usage: ``python -m cphf_gb300.train_mlp [--systems 40] [--epochs 30] [--out PATH]``
"""

import argparse
import time
from pathlib import Path

import numpy as np

from . import synth
from .api import Context

WEIGHTS = Path(__file__).resolve().parent / "mlp_weights.npy"


def init_weights(seed=0):
    """He-style initial weights in the packed layout W1[64,3] b1 W2[64,64] b2 W3[2,64] b3."""
    rng = np.random.default_rng(seed)
    parts = [rng.standard_normal((64, 3)) / np.sqrt(3), np.zeros(64), rng.standard_normal((64, 64)) / 8.0,
             np.zeros(64), rng.standard_normal((2, 64)) * 0.01, np.zeros(2)]
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)


def system_dims(k, rng):
    nao = int(rng.integers(15, 46)) * 8          # 120 .. 360
    natm = max(4, nao // 10)
    return dict(nao=nao, naux=int(3.3 * nao), nocc=(nao // 10,), natm=natm, decay=20.0)


def training_data(nsys, seed=1000, device=0, verbose=True):
    rng = np.random.default_rng(seed)
    feats, targs = [], []
    for k in range(nsys):
        dims = system_dims(k, rng)
        s = synth.make_system(dims, seed=seed + k)
        ctx = Context(precision="mixed", device=device)
        ctx.set_cderi(s.cderi, s.scale_j, s.scale_k)
        ctx.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])
        x = ctx.solve_dimless_cphf(s.rhs[0])
        f = ctx.mlp_features(s.rhs[0])
        no, nvir, nrhs = s.nocc[0], s.nao - s.nocc[0], 3 * s.natm
        b = s.rhs[0][no:].reshape(nvir * no, nrhs, order="F")
        xv = x[no:].reshape(nvir * no, nrhs, order="F")
        num = (xv * (b - xv)).sum(axis=1)
        den = (xv * xv).sum(axis=1)
        d = np.where(den > 0, num / np.maximum(den, 1e-300), 0.0)
        t = np.stack([xv.reshape(-1, order="F"), np.repeat(d[:, None], nrhs, 1).reshape(-1, order="F")], axis=1)
        feats.append(f)
        targs.append(t.astype(np.float32))
        ctx.close()
        if verbose:
            print(f"system {k}: nao={s.nao} samples={len(f)} residual={ctx.last_stats['residual_max']:.1e}",
                  flush=True)
    return np.concatenate(feats), np.concatenate(targs)


def train(feat, target, epochs=30, batch=65536, lr=3e-3, seed=0, device=0):
    ctx = Context(device=device)
    ctx.set_nao(8)
    ctx.set_mlp_weights(init_weights(seed))
    hist = ctx.mlp_train(feat, target, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return ctx.mlp_weights(), hist


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--systems", type=int, default=40)
    p.add_argument("--epochs", type=int, default=30)
    p.add_argument("--max-samples", type=int, default=4_000_000)
    p.add_argument("--out", default=str(WEIGHTS))
    a = p.parse_args()
    t0 = time.time()
    feat, target = training_data(a.systems)
    if len(feat) > a.max_samples:
        idx = np.random.default_rng(0).choice(len(feat), a.max_samples, replace=False)
        feat, target = feat[idx], target[idx]
    w, hist = train(feat, target, epochs=a.epochs)
    np.save(a.out, w)
    print(f"trained on {len(feat)} samples in {time.time() - t0:.1f} s; loss {hist[0]:.3e} -> {hist[-1]:.3e}")


if __name__ == "__main__":
    main()
