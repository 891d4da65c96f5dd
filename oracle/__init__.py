"""CPU oracle for the stochastic-Galerkin hot path of ExtendableASGFEM.jl.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
directory; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` use it, and only as the checker or as the timed CPU
reference.  It is a plain restatement of the reference algorithms (Julia
package ExtendableASGFEM.jl v1.0.1), each function citing the reference file
and line it follows.

Parity pins
-----------
* The one-dimensional orthonormal bases and the tensorised triple products
  (hence the coupling tensor ``G`` for Hermite) are pinned to the closed forms
  of the reference's own tests (``test/runtests.jl:51-127``), see
  ``tests/golden/``.
* The Legendre coupling tensor is pinned to the closed form
  ``beta_n = n / sqrt(4 n^2 - 1)``.
* The operator apply, the solvers, the estimator and the sampling error are
  NOT pinned by any reference test (the reference has none for them and Julia
  is not available to run it); they are restated literally from the cited
  source lines and cross-checked by mathematical identities (Kronecker direct
  solve, symmetry, P=1 reduction).  The spatial finite-element layer
  (ExtendableFEM / ExtendableGrids / ExtendableFEMBase: meshes, quadrature
  rules, FaceInterpolator) is not part of the reference tree; ``fem.py``
  restates it on a structured mesh and that part is "parity unpinned".
"""
