"""The exact mean-based preconditioner on meshes that are not power-of-two
lattices (SGFEM_PREC_CHOLESKY: sparse Cholesky of K_0 in nested-dissection
order, triangular solves on the GPU) against the reference's ldiv! with
LU(K_0) (solvers_poisson_primal.jl:23-78, the oracle's MeanPreconditioner).

Bars: the preconditioner 1e-10 relative in FP64 and 1e-4 in FP32; FP64 PCG
takes the oracle PCG's iteration count with the LU preconditioner to within
one, and its solution matches the oracle's GMRES solution (the reference
solve) to 1e-8; mixed precision and the lognormal GMRES meet their FP64
residual tolerances on the same meshes."""
import numpy as np
import pytest

from oracle import sg as osg
from tests.problems import build

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def perturbed(order, N, M, deg, seed=1, basis="legendre", mean=1.0):
    import __graft_entry__ as ge
    from types import SimpleNamespace
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=mean, maxm=150)
    V = pkg.H1Pk(pkg.perturbed_unit_square_mesh(N, 0.2, seed=seed), order)
    mis = pkg.total_degree_multiindices(M, deg)
    B = pkg.LegendrePolynomials if basis == "legendre" else pkg.HermitePolynomials
    TB = pkg.TensorizedBasis(B, M, deg, deg + 4, multi_indices=mis)
    sol = pkg.SGFEVector(V, TB)
    problem = pkg.PoissonProblemPrimal if basis == "legendre" else pkg.LogTransformedPoissonProblemPrimal
    Ks, b0 = pkg.assemble(problem, sol, C, rhs=lambda x, y: np.ones_like(x))
    return SimpleNamespace(pkg=pkg, C=C, V=V, TB=TB, sol=sol, Kall=Ks, K0=Ks[0], Ks=Ks[1:], b0=b0,
                           G=TB.G.toarray(), bdofs=V.bdofs, n=V.ndofs, P=TB.nmodes, M=M)


@pytest.fixture(scope="module", params=["p1_perturbed", "p2_perturbed"])
def case(request, built_pkg):
    p = {"p1_perturbed": lambda: perturbed(1, 24, 4, 2), "p2_perturbed": lambda: perturbed(2, 10, 3, 2)}[request.param]()
    op = p.pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    assert not op.has_lattice and op.mean_preconditioner == p.pkg.PREC_CHOLESKY
    yield p, op
    op.close()


def test_cholesky_preconditioner_matches_lu(case):
    p, op = case
    pkg = p.pkg
    assert "not factored" in op.ctx.cholesky_log
    b = np.random.default_rng(4).standard_normal(p.n * p.P)
    mask = osg.interior_mask(p.n, p.P, p.bdofs)
    b[~mask] = 0.0
    ref = osg.MeanPreconditioner(p.K0, p.bdofs, p.P).ldiv(b)
    y = op.ldiv(b, pkg.PREC_CHOLESKY, pkg.FP64)
    assert "nnz(L)" in op.ctx.cholesky_log, op.ctx.cholesky_log
    assert rel(y[mask], ref[mask]) <= 1e-10
    assert np.all(y[~mask] == 0.0)
    assert rel(op.ldiv(b, pkg.PREC_CHOLESKY, pkg.FP32)[mask], ref[mask]) <= 1e-4
    # the host check of the same factor and schedule agrees to rounding
    zh, _ = pkg.cholesky_host_solve(p.K0, p.bdofs, b)
    assert rel(y, zh) <= 1e-13
    # bitwise reproducible
    assert np.array_equal(y, op.ldiv(b, pkg.PREC_CHOLESKY, pkg.FP64))


def test_pcg_iterations_and_solution_match_oracle(case):
    p, op = case
    pkg = p.pkg
    n, P = p.n, p.P
    prec = osg.MeanPreconditioner(p.K0, p.bdofs, P)
    b = osg.reference_rhs(np.zeros(n * P), p.b0, p.bdofs, P)
    apply = lambda v: osg.apply_fast(v, p.K0, p.Ks, p.G, p.bdofs, P)
    _, st_o = osg.pcg(apply, prec.ldiv, b, np.zeros(n * P), osg.interior_mask(n, P, p.bdofs), tol=1e-10)
    x = np.zeros(n * P)
    st = op.solve_primal(p.b0, x, rtol=1e-10, precision=pkg.FP64, check_every=1)
    assert abs(st["iterations"] - st_o["niter"]) <= 1, (st["iterations"], st_o["niter"])
    xg, _ = osg.gmres_left(apply, prec.ldiv, b, np.zeros(n * P))
    assert rel(x, xg) <= 1e-8
    # a Jacobi-preconditioned solve needs many more iterations on the same system
    xj = np.zeros(n * P)
    stj = op.solve_primal(p.b0, xj, rtol=1e-10, precision=pkg.FP64, preconditioner=pkg.PREC_JACOBI)
    assert stj["iterations"] > 2 * st["iterations"]


def test_mixed_solve_with_cholesky(case):
    p, op = case
    pkg = p.pkg
    n, P = p.n, p.P
    x = np.zeros(n * P)
    st = op.solve_primal(p.b0, x, rtol=1e-10, precision=pkg.MIXED)
    b = osg.reference_rhs(np.zeros(n * P), p.b0, p.bdofs, P)
    r = b - osg.apply_fast(x, p.K0, p.Ks, p.G, p.bdofs, P)
    assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(b), st


def test_package_solve_on_perturbed_mesh(built_pkg):
    """solve!(PoissonProblemPrimal, sol, C) picks the Cholesky form by itself."""
    p = perturbed(1, 16, 3, 2, seed=5)
    pkg = p.pkg
    pkg.solve(pkg.PoissonProblemPrimal, p.sol, p.C, rhs=lambda x, y: np.ones_like(x), rtol=1e-11,
              precision=pkg.FP64)
    ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
    assert rel(p.sol.entries, ref) <= 1e-9
    assert p.sol.solve_stats["iterations"] < 40


def test_lognormal_gmres_on_perturbed_mesh(built_pkg):
    p = perturbed(1, 12, 3, 2, seed=2, basis="hermite", mean=0.0)
    pkg = p.pkg
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    for prec, tol in ((pkg.FP64, 1e-12), (pkg.MIXED, 1e-10)):
        x = np.zeros(p.n * p.P)
        st = op.solve_logpoisson(p.b0, x, rtol=tol, precision=prec)
        assert st["relres"] <= tol
        ref = osg.kron_direct_full(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
        assert rel(x, ref) <= 1e-7
    op.close()


def test_cholesky_equals_lattice_form_on_a_lattice(built_pkg):
    """On a P1 lattice both exact forms are K_0^-1: same preconditioned vector."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    p = build(16, 1, 3, pkg.total_degree_multiindices(3, 2))
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    assert op.has_lattice
    b = np.random.default_rng(8).standard_normal(p.n * p.P)
    mask = osg.interior_mask(p.n, p.P, p.bdofs)
    b[~mask] = 0.0
    assert rel(op.ldiv(b, pkg.PREC_CHOLESKY), op.ldiv(b, pkg.PREC_LATTICE)) <= 1e-11
    xa, xb = np.zeros(p.n * p.P), np.zeros(p.n * p.P)
    sa = op.solve_primal(p.b0, xa, rtol=1e-10, precision=pkg.FP64, preconditioner=pkg.PREC_CHOLESKY)
    sb = op.solve_primal(p.b0, xb, rtol=1e-10, precision=pkg.FP64, preconditioner=pkg.PREC_LATTICE)
    assert abs(sa["iterations"] - sb["iterations"]) <= 1
    assert rel(xa, xb) <= 1e-9
    op.close()


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_sample_solves_on_perturbed_mesh(built_pkg, precision):
    """Deterministic sample solves (poisson_primal.jl:14-35) on a non-lattice P2
    mesh use the Cholesky mean preconditioner and match direct solves."""
    from oracle import sampling as osm
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    V = pkg.H1Pk(pkg.perturbed_unit_square_mesh(8, 0.2, seed=4), 2)
    Ms = 6
    Ks = pkg.assemble_stiffness(V, C, list(range(Ms + 1)), 4)
    b0 = pkg.assemble_rhs(V, lambda x, y: np.ones_like(x), 2)
    y = np.random.default_rng(6).uniform(-1, 1, size=(Ms, 40))
    sp_ = pkg.SampleProblems(V, Ks, y)
    assert not sp_.ctx.has_lattice
    U = sp_.solve(b0, rtol=1e-10, precision=getattr(pkg, precision))
    assert sp_.stats["relres"] <= 1e-10
    assert sp_.stats["iterations"] < 60
    for s in range(y.shape[1]):
        ref = osm.deterministic_solve(Ks, b0, V.bdofs, y[:, s])
        assert np.linalg.norm(U[:, s] - ref) <= 1e-8 * np.linalg.norm(ref)
    sp_.close()


def test_precision_switch_on_one_context(built_pkg):
    """FP64 then FP32 and mixed solves with the Cholesky form on one context of a
    structured P1 mesh (exact zeros in K_0): the shared work vectors hold the
    previous precision's data, which no application may read before writing."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    p = build(12, 1, 6, pkg.top_weight_multiindices(6, 20, C.decay_factors))
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    assert op.mean_preconditioner == pkg.PREC_CHOLESKY
    b = np.random.default_rng(4).standard_normal(p.n * p.P)
    mask = osg.interior_mask(p.n, p.P, p.bdofs)
    b[~mask] = 0.0
    ref = osg.MeanPreconditioner(p.K0, p.bdofs, p.P).ldiv(b)
    for prec, tol, pt in ((pkg.FP64, 1e-10, 1e-10), (pkg.FP32, 1e-6, 1e-4), (pkg.MIXED, 1e-10, 1e-4),
                          (pkg.FP64, 1e-10, 1e-10)):
        x = np.zeros(p.n * p.P)
        st = op.solve_primal(p.b0, x, rtol=tol, precision=prec)
        assert st["relres"] <= tol, (prec, st)
        y = op.ldiv(b, pkg.PREC_CHOLESKY, pkg.FP32 if prec != pkg.FP64 else pkg.FP64)
        assert rel(y[mask], ref[mask]) <= pt, prec
    op.close()
