"""The timed CPU reference (oracle/refsolve.py: solve_primal! with the C mul!,
the C per-mode LU solves and full left-preconditioned GMRES) against the
pure-Python oracle it must equal: ldiv! of the SuperLU factors, GMRES of
oracle/sg.py and the Kronecker direct solve (solvers_poisson_primal.jl:
23-78, 130-169, 172-230).  CPU only."""
import numpy as np
import pytest

from oracle import refsolve
from oracle import sg as osg
from tests.problems import build, config1_like


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("order,N,threads", [(1, 16, 1), (2, 8, 3)])
def test_ldiv_matches_superlu_per_mode(pkg, order, N, threads):
    p = build(N, order, 4, pkg.total_degree_multiindices(4, 2))  # P = 15: two groups of right-hand sides
    rs = refsolve.ReferenceSolver(p.Kall, p.G, p.bdofs, p.P, nthreads=threads)
    b = np.random.default_rng(0).standard_normal(p.n * p.P)
    ref = osg.MeanPreconditioner(p.K0, p.bdofs, p.P).ldiv(b)
    assert rel(rs.ldiv(b), ref) <= 1e-13


def test_solve_reaches_true_residual_and_matches_direct(pkg):
    p = config1_like(N=16)
    rs = refsolve.ReferenceSolver(p.Kall, p.G, p.bdofs, p.P, nthreads=2)
    for rtol in (1e-8, 1e-11):
        x, st = rs.solve(p.b0, rtol=rtol)
        b = osg.reference_rhs(np.zeros(p.n * p.P), p.b0, p.bdofs, p.P)
        r = b - osg.mul_literal(x, p.K0, p.Ks, p.G, p.bdofs, p.P)
        assert np.linalg.norm(r) / np.linalg.norm(b) <= rtol
        assert abs(st["relres"] - np.linalg.norm(r) / np.linalg.norm(b)) <= 1e-3 * rtol
    ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
    assert rel(x, ref) <= 1e-9


def test_solve_iterates_like_oracle_gmres(pkg):
    """Same Krylov space and rotations as oracle/sg.py:gmres_left: stopped at the
    same iteration, the iterates agree."""
    p = config1_like(N=8, M=3)
    rs = refsolve.ReferenceSolver(p.Kall, p.G, p.bdofs, p.P, nthreads=1)
    x, st = rs.solve(p.b0, rtol=1e-9)
    prec = osg.MeanPreconditioner(p.K0, p.bdofs, p.P)
    b = osg.reference_rhs(np.zeros(p.n * p.P), p.b0, p.bdofs, p.P)
    xo, so = osg.gmres_left(lambda v: osg.mul_literal(v, p.K0, p.Ks, p.G, p.bdofs, p.P), prec.ldiv, b,
                            np.zeros(p.n * p.P), atol=0.0, rtol=1e-9, itmax=st["iterations"])
    assert so["niter"] <= st["iterations"]
    if so["niter"] == st["iterations"]:
        assert rel(x, xo) <= 1e-10


def test_warm_start_rhs(pkg):
    """b = x0 + e_1 (x) b0 with boundary rows zeroed (solvers_poisson_primal.jl:149-155)."""
    p = config1_like(N=8, M=3)
    rs = refsolve.ReferenceSolver(p.Kall, p.G, p.bdofs, p.P, nthreads=1)
    x0 = np.random.default_rng(1).standard_normal(p.n * p.P) * 1e-2 * osg.interior_mask(p.n, p.P, p.bdofs)
    assert np.array_equal(rs.rhs(p.b0, x0), osg.reference_rhs(x0, p.b0, p.bdofs, p.P))
