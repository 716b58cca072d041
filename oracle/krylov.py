"""Block Krylov solver for ``(I + A) x = b`` -- oracle restatement (test infrastructure only).

Follows ``src/util/krylov_block.rs`` of the reference line by line:

* ``krylov_block``     -- ``krylov_block.rs:39-197``
* ``_projected_solve`` -- ``krylov_block.rs:204-215``
* ``_orth_block``      -- ``krylov_block.rs:225-253``

Layout is col-major as in the reference: ``b`` and ``x`` are ``[n, nset]``,
each right-hand side a column, and ``aop`` maps ``[n, nblock] -> [n, nblock]``.
Where the reference panics (non-convergence, ``krylov_block.rs:188-194``)
this raises :class:`KrylovNotConverged`.
"""

import numpy as np


class KrylovNotConverged(RuntimeError):
    """Raised where the reference panics with "krylov_block failed to converge"."""


def _orth_block(vec, lindep):
    """Serial modified Gram-Schmidt over the columns of ``vec`` (krylov_block.rs:225-253).

    Keeps non-normalized orthogonal columns and their squared norms; drops a
    column whose remaining squared norm is ``<= lindep``.
    """
    n, nblock = vec.shape
    result = []
    norms_sq = []
    for i in range(nblock):
        vi = vec[:, i].copy()
        for j in range(len(result)):
            coeff = float(vi @ result[j]) / norms_sq[j]
            vi -= coeff * result[j]
        nsq = float(vi @ vi)
        if nsq > lindep:
            result.append(vi)
            norms_sq.append(nsq)
    if not result:
        return np.zeros((n, 0)), []
    return np.stack(result, axis=1), norms_sq


def _projected_solve(xs, ax, inner, b):
    """Galerkin solve on the subspace (krylov_block.rs:204-215).

    ``h = xs^T ax + diag(inner)``, ``g = xs^T b``, ``c = solve(h, g)``; returns ``xs c``.
    """
    h = xs.T @ ax
    h[np.diag_indices_from(h)] += np.asarray(inner)
    g = xs.T @ b
    c = np.linalg.solve(h, g)
    return xs @ c


def krylov_block(aop, b, x0=None, tol=1e-8, max_cycle=42, max_space=14, lindep=1e-14,
                 stats=None, verbose=False):
    """Solve ``(I + aop) x = b`` (krylov_block.rs:39-197).

    ``stats`` (optional dict) receives ``aop_calls``, ``aop_columns`` (sum of
    block widths), ``cycles``, ``restarts`` and ``max_innerprod``.
    """
    b = np.asarray(b, dtype=np.float64)
    n, nset = b.shape
    b_orig = b.copy()
    x_accum = np.zeros((n, nset)) if x0 is None else np.array(x0, dtype=np.float64)

    max_basis = nset * (max_space + 1)
    xs = np.zeros((n, max_basis))
    ax = np.zeros((n, max_basis))
    all_innerprod = []

    conv_thresh = max(lindep, tol * tol)
    total_cycles = 0
    restart_idx = 0
    last_nd = 0
    last_b = b_orig.copy()
    last_max_innerprod = 0.0
    calls = [0, 0]

    def _aop(v):
        calls[0] += 1
        calls[1] += v.shape[1]
        return np.asarray(aop(v))

    while total_cycles < max_cycle:
        # krylov_block.rs:86-87 -- residual of the accumulated solution
        if restart_idx == 0 and x0 is None:
            b_residual = b_orig.copy()
        else:
            b_residual = b_orig - (x_accum + _aop(x_accum))

        x1, innerprod = _orth_block(b_residual, lindep)
        if x1.shape[1] == 0:
            last_nd = 0
            last_b = b_residual
            break

        all_innerprod = []
        nd = 0
        inner_converged = False
        for inner in range(max_space):
            if total_cycles >= max_cycle:
                break
            total_cycles += 1
            nblock = x1.shape[1]
            axt = _aop(x1)
            xs[:, nd:nd + nblock] = x1
            ax[:, nd:nd + nblock] = axt
            all_innerprod.extend(innerprod)
            nd += nblock

            # krylov_block.rs:119-122 -- project axt off the whole subspace at once
            xs_slc = xs[:, :nd]
            ip_vec = np.asarray(all_innerprod)
            coeffs = (xs_slc.T @ axt) / ip_vec[:, None]
            x1_new = axt - xs_slc @ coeffs

            next_x1, next_ip = _orth_block(x1_new, lindep)
            max_innerprod = max(next_ip) if next_ip else 0.0

            keep = [ip > conv_thresh for ip in next_ip]
            if not all(keep):
                idx = [k for k, m in enumerate(keep) if m]
                next_x1 = next_x1[:, idx]
                next_ip = [next_ip[k] for k in idx]
            if verbose:
                print(f"restart {restart_idx} inner {inner + 1} (total cycle {total_cycles}): "
                      f"max(||v||^2) = {max_innerprod:.3e}")
            x1 = next_x1
            innerprod = next_ip
            last_max_innerprod = max_innerprod
            if max_innerprod < conv_thresh:
                inner_converged = True
                break

        last_nd = nd
        last_b = b_residual
        if inner_converged or total_cycles >= max_cycle:
            break

        # krylov_block.rs:172-174 -- hard restart
        x_accum = x_accum + _projected_solve(xs[:, :nd], ax[:, :nd], all_innerprod, last_b)
        restart_idx += 1

    if last_nd == 0:
        x_out = x_accum
    else:
        x_out = x_accum + _projected_solve(xs[:, :last_nd], ax[:, :last_nd], all_innerprod, last_b)

    if stats is not None:
        stats.update(aop_calls=calls[0], aop_columns=calls[1], cycles=total_cycles,
                     restarts=restart_idx, max_innerprod=last_max_innerprod)

    if last_max_innerprod >= conv_thresh:
        raise KrylovNotConverged(
            f"krylov_block failed to converge: max(||v||^2) = {last_max_innerprod:.3e} >= "
            f"tol^2 = {conv_thresh:.3e} after {total_cycles} cycles ({restart_idx} restarts, "
            f"max_cycle = {max_cycle}, max_space = {max_space})")
    return x_out
