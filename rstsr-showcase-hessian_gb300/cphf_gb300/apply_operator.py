"""Time applications of the response operator on a synthetic workload.

    python -m cphf_gb300.apply_operator rks_nao600 --nb 180 --reps 3 [--precision fp64]

Builds the seeded system, prepares a context and applies the dimensionless operator
(``response_dimless_cphf_lowp`` for the mixed context's split-precision operator,
``response_dimless_cphf`` for FP64) ``reps`` times to nb random columns, printing the
host-side time of each application (host<->device copies of the columns included).  A small,
self-contained invocation of the operator's kernels for launch lists and profiler captures.
"""

import argparse
import time

import numpy as np

from . import synth
from .api import Context


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("workload", help="synthetic workload name (synth.CONFIGS)")
    ap.add_argument("--nb", type=int, default=None, help="columns per application (default: all RHS)")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--precision", default="mixed", choices=("mixed", "fp64"))
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    s = synth.make_system(a.workload, seed=a.seed)
    nb = a.nb or 3 * s.natm
    ctx = Context(precision=a.precision)
    ctx.set_cderi(s.cderi, s.scale_j, s.scale_k)
    if s.grid is not None:
        ctx.set_grid(s.grid.ao, s.grid.weights, s.grid.fxc, s.nspin, s.grid.atom_offsets)
    rng = np.random.default_rng(a.seed + 1)
    if s.nspin == 1:
        ctx.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])
        mo1 = rng.standard_normal((s.nao, s.nocc[0], nb))
    else:
        ctx.make_response_preparation(s.mo_coeff, s.mo_occ, s.mo_energy)
        mo1 = [rng.standard_normal((s.nao, s.nocc[t], nb)) for t in range(2)]
    op = ctx.response_dimless_cphf_lowp if a.precision == "mixed" else ctx.response_dimless_cphf
    for r in range(a.reps):
        t0 = time.perf_counter()
        op(mo1)
        print(f"application {r}: {time.perf_counter() - t0:.4f} s ({a.workload}, nb={nb}, {a.precision})", flush=True)


if __name__ == "__main__":
    main()
