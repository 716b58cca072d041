"""Two-centre metric decomposition and cderi build -- oracle restatement (test infrastructure only).

Restates ``src/ri_jk/pure_decompose.rs`` of the reference with numpy / scipy LAPACK:

* :func:`decomp_j2c_cd` -- ``decomp_j2c_cd`` (``pure_decompose.rs:29-57``) with ``uplo = Upper``:
  ``j2c = U^T U``; when the factorisation fails or ``min diag(U) <= threshold`` the eigenvalues
  are clamped at the threshold, ``j2c' = V max(e, thr) V^T``, and ``j2c'`` is factored without a
  further check; ``threshold = None`` raises on failure (the reference panics).
* :func:`solve_by_j2c_right` -- ``solve_by_j2c(j3c, Cd Upper, Right, flip_uplo = false)``
  (``pure_decompose.rs:205-252``): ``solve_triangular(U^T, j3c^T, Lower)`` transposed back,
  i.e. ``cderi = j3c U^-1``.
* :func:`generate_cderi` -- ``generate_cderi_with_decomp`` (``src/ri_jk/hess_r.rs:1725-1735``)
  with ``RHessRIJK::new_without_cderi``'s options (``hess_r.rs:1752``: Cd, 1e-14, Upper) on
  caller-supplied integrals.

Parity is pinned by the property the reference's own test checks
(``pure_decompose.rs:333-356``, ``test_check_recoverable``: ``U^T U`` reproduces ``j2c``) and by
LAPACK's Cholesky / triangular solve, which the reference reaches through rstsr's linalg.
"""

import numpy as np
import scipy.linalg


def decomp_j2c_cd(j2c, threshold=1e-14):
    """Returns ``(U, fallback)`` with ``j2c = U^T U`` (U upper triangular)."""
    j2c = np.asarray(j2c, dtype=np.float64)
    try:
        L = np.linalg.cholesky(j2c)
        ok = True
    except np.linalg.LinAlgError:
        ok = False
    if threshold is None:
        if not ok:
            raise np.linalg.LinAlgError("Cholesky decomposition failed and no threshold is given")
        return np.ascontiguousarray(L.T), False
    if ok and np.diag(L).min() > threshold:
        return np.ascontiguousarray(L.T), False
    e, v = np.linalg.eigh(j2c)
    e = np.maximum(e, threshold)
    j2c2 = (v * e[None, :]) @ v.T
    L = np.linalg.cholesky(j2c2)
    return np.ascontiguousarray(L.T), True


def solve_by_j2c_right(j3c, U):
    """``cderi = j3c U^-1`` for j3c ``[n, naux]``."""
    x = scipy.linalg.solve_triangular(U.T, np.asarray(j3c).T, lower=True)
    return np.asfortranarray(x.T)


def generate_cderi(j3c, j2c, threshold=1e-14):
    U, fallback = decomp_j2c_cd(j2c, threshold)
    return solve_by_j2c_right(j3c, U), U, fallback


def synthetic_metric(naux, seed=0, cond=1e4):
    """A seeded SPD metric with eigenvalues log-spaced over ``cond``, for tests and benchmarks
    (the reference builds j2c from libcint's int2c2e)."""
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((naux, naux)))
    e = np.logspace(0.0, -np.log10(cond), naux)
    return np.asfortranarray((q * e[None, :]) @ q.T)
