"""GPU path of LogTransformedPoissonProblemPrimal (src/modelproblems/
logpoisson_primal.jl, solvers_logpoisson_primal.jl): the SG operator with the
non-symmetric convection blocks N_m, and the device GMRES against the oracle's
assembled Kronecker solve (solve_logpoisson_primal_full!).

Bars: FP64 apply 1e-12 relative (2-norm) to the oracle's literal mul!; FP32
apply 1e-5; FP64 GMRES to rtol 1e-12, solution within 1e-9 of the direct
solve; mixed precision to rtol 1e-10, within 1e-7 of the FP64 solution."""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import sg as osg

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def build_log(N=16, order=1, M=4, deg=2):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.0, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), order)
    mis = pkg.total_degree_multiindices(M, deg)
    TB = pkg.TensorizedBasis(pkg.HermitePolynomials, M, deg, deg + 4, multi_indices=mis)
    sol = pkg.SGFEVector(V, TB)
    Ks, b = pkg.assemble(pkg.LogTransformedPoissonProblemPrimal, sol, C, rhs=lambda x, y: np.ones_like(x))
    return SimpleNamespace(pkg=pkg, C=C, V=V, TB=TB, sol=sol, Ks=Ks, A=Ks[0], Ns=Ks[1:], b=b, G=TB.G.toarray(),
                           bdofs=V.bdofs, n=V.ndofs, P=TB.nmodes, M=M)


@pytest.fixture(scope="module", params=["p1_lattice", "p2_lattice", "p1_jacobi"])
def case(request, built_pkg):
    p = {"p1_lattice": lambda: build_log(16, 1, 4, 2), "p2_lattice": lambda: build_log(8, 2, 3, 2),
         "p1_jacobi": lambda: build_log(12, 1, 3, 2)}[request.param]()
    op = p.pkg.SGOperator(p.V, p.TB, p.Ks, device=0)
    yield p, op
    op.close()


def test_log_apply_matches_oracle(case):
    p, op = case
    x = np.random.default_rng(0).standard_normal(p.n * p.P)
    y = op.mul(x, p.pkg.FP64)
    yref = osg.mul_literal(x, p.A, p.Ns, p.G, p.bdofs, p.P)
    assert rel(y, yref) <= 1e-12
    assert rel(op.mul(x, p.pkg.FP32), yref) <= 1e-5


def test_log_gmres_fp64_matches_direct(case):
    p, op = case
    x = np.zeros(p.n * p.P)
    st = op.solve_logpoisson(p.b, x, rtol=1e-12, precision=p.pkg.FP64)
    assert st["relres"] <= 1e-12
    ref = osg.kron_direct_full(p.A, p.Ns, p.G, p.b, p.bdofs, p.P)
    assert rel(x, ref) <= 1e-9


def test_log_gmres_mixed(case):
    p, op = case
    x64 = np.zeros(p.n * p.P)
    op.solve_logpoisson(p.b, x64, rtol=1e-12, precision=p.pkg.FP64)
    x = np.zeros(p.n * p.P)
    st = op.solve_logpoisson(p.b, x, rtol=1e-10, precision=p.pkg.MIXED)
    assert st["relres"] <= 1e-10
    assert st["outer_iterations"] >= 1
    assert rel(x, x64) <= 1e-7


def test_log_gmres_warm_start_rhs(case):
    """b = x0 + b0 with boundary rows zeroed (solvers_logpoisson_primal.jl:149-155);
    the boundary entries of the iterate keep their start values (zero, as in an
    SGFEVector after a solve; nonzero ones would enter the interior equations)."""
    p, op = case
    rng = np.random.default_rng(3)
    mask = osg.interior_mask(p.n, p.P, p.bdofs)
    x0 = rng.standard_normal(p.n * p.P) * 1e-2 * mask
    x = x0.copy()
    op.solve_logpoisson(p.b, x, rtol=1e-12, precision=p.pkg.FP64, restart=10)
    ref = osg.kron_direct_full(p.A, p.Ns, p.G, p.b + x0, p.bdofs, p.P)
    assert rel(x[mask], ref[mask]) <= 1e-9
    assert np.array_equal(x[~mask], x0[~mask])


def test_gmres_on_symmetric_problem_equals_pcg(built_pkg):
    from tests.problems import config1_like
    p = config1_like(N=16)
    op = p.pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    xa = np.zeros(p.n * p.P)
    op.solve_primal(p.b0, xa, rtol=1e-12, precision=p.pkg.FP64)
    b_full = np.zeros(p.n * p.P)
    b_full[:p.n] = p.b0
    xb = np.zeros(p.n * p.P)
    st = op.solve_logpoisson(b_full, xb, rtol=1e-12, precision=p.pkg.FP64)
    assert st["relres"] <= 1e-12
    assert rel(xb, xa) <= 1e-10
    op.close()


def test_solve_dispatch_logpoisson(built_pkg):
    """solve!(LogTransformedPoissonProblemPrimal, sol, C; rhs) through the host mirror."""
    p = build_log(8, 1, 2, 2)
    pkg = p.pkg
    pkg.solve(pkg.LogTransformedPoissonProblemPrimal, p.sol, p.C, rhs=lambda x, y: np.ones_like(x), rtol=1e-12,
              precision=pkg.FP64)
    ref = osg.kron_direct_full(p.A, p.Ns, p.G, p.b, p.bdofs, p.P)
    assert rel(p.sol.entries, ref) <= 1e-9
