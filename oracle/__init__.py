"""CPU oracle for the CPHF response path -- TEST INFRASTRUCTURE ONLY.

This package is a plain numpy (FP64) restatement of the reference crate
``rstsr-showcase-hessian``'s CPHF response path.  It exists to check the GPU
library, never to produce results for it:

* only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
  leg (and its ``--impl reference`` arm) may import it;
* the product path (``cphf_gb300`` + ``libcphf.so``) never imports, calls or
  falls back to anything here.

Modules and the reference code each one restates (paths inside the reference
project):

* ``krylov``  -- ``src/util/krylov_block.rs:39-253`` (block Krylov with hard
  restarts, MGS, projected solve, panic on non-convergence).
* ``rijk``    -- ``src/ri_jk/hess_r.rs:82-186`` (separated RI-J/RI-K response
  core), RHF assembly ``hess_r.rs:1916-1953``, UHF assembly
  ``src/ri_jk/hess_u.rs:270-313``, packing ``src/util/density_matrices.rs:48-77``
  and the einsum cross-check ``src/ri_jk/hess_r_naive.rs:861-903``.
* ``xc``      -- RKS/UKS XC response: ``src/numint_matmul/hess_rks.rs:570-605``,
  ``pure_eval_rho.rs:216-334`` (RHO branch), ``pure_xcpot.rs:285-465``,
  ``hess_uks.rs:390-441`` and ``pure_xcpot.rs:921-1028``.
* ``cphf``    -- the CPHF driver: ``src/hessian/rscf.rs:210-399`` and
  ``src/hessian/uscf.rs:203-446``.

Parity pin: ``tests/golden/make_golden.py`` runs the reference's own Python
twin (``pyhessref/krylov_block.py``, ``pyhessref/hess_scf_restricted.py``,
``pyhessref/hess_scf_unrestricted.py``) and the reference's Krylov fixture
generator (``prototype/02-7-krylov_testing_setup.py``) and stores their
outputs under ``tests/golden/``; ``tests/test_oracle_golden.py`` checks this
oracle against them.  The XC restatement has no runnable reference twin (its
Python counterpart needs PySCF); it is cross-checked against the independent
density-matrix form of the same kernel (``xc.rks_response_bra_dm_form``).
"""
