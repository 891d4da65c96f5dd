"""Appending modes to a finalized operator (sgfem_update_coupling, the
adaptive loop of scripts/poisson.jl:341-420): the updated operator applies
the oracle's mul! for the new basis (solvers_poisson_primal.jl:86-124, 1e-12
relative), its solve meets the FP64 residual recomputed on the host with the
oracle's operator, and it applies, preconditions and solves exactly
like an operator finalized from scratch with the new basis, while the K_m
stay on the GPU."""
import numpy as np
import pytest

from oracle import sg as osg
from tests.problems import build

pytestmark = pytest.mark.gpu


def _ops(pkg, p, TB2, Ks2):
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    fresh = pkg.SGOperator(p.V, TB2, Ks2, device=0)
    return op, fresh


@pytest.mark.parametrize("order,N", [(2, 16), (1, 12)])
def test_update_matches_fresh_operator(built_pkg, order, N):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    p = build(N, order, 6, pkg.top_weight_multiindices(6, 20, C.decay_factors))
    mis2 = pkg.top_weight_multiindices(6, 40, C.decay_factors)
    d2 = max(max(m) for m in mis2)
    TB2 = pkg.TensorizedBasis(pkg.LegendrePolynomials, 6, d2, d2 + 4, multi_indices=mis2)
    op, fresh = _ops(pkg, p, TB2, p.Kall)
    x0 = np.zeros(p.n * p.TB.nmodes)
    op.solve_primal(p.b0, x0, rtol=1e-10, precision=pkg.MIXED)  # the old basis, kernels compiled
    op.update_basis(TB2)
    x = np.random.default_rng(3).standard_normal(p.n * TB2.nmodes)
    G2 = TB2.G.toarray()
    yref = osg.mul_literal(x, p.K0, p.Ks, G2, p.bdofs, TB2.nmodes)
    y = op.mul(x, pkg.FP64)
    assert np.linalg.norm(y - yref) <= 1e-12 * np.linalg.norm(yref)
    assert np.linalg.norm(op.mul(x, pkg.FP32) - yref) <= 1e-5 * np.linalg.norm(yref)
    for prec in (pkg.FP64, pkg.FP32):
        assert np.array_equal(op.mul(x, prec), fresh.mul(x, prec))
    if op.has_lattice:
        assert np.array_equal(op.ldiv(x), fresh.ldiv(x))
    for prec in (pkg.FP64, pkg.MIXED):
        xa = np.zeros(p.n * TB2.nmodes)
        xb = np.zeros(p.n * TB2.nmodes)
        sa = op.solve_primal(p.b0, xa, rtol=1e-10, precision=prec)
        sb = fresh.solve_primal(p.b0, xb, rtol=1e-10, precision=prec)
        assert sa["iterations"] == sb["iterations"] and np.array_equal(xa, xb)
        b = osg.reference_rhs(np.zeros(p.n * TB2.nmodes), p.b0, p.bdofs, TB2.nmodes)
        r = b - osg.apply_fast(xa, p.K0, p.Ks, G2, p.bdofs, TB2.nmodes)
        assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(b)
    op.close()
    fresh.close()


def test_update_to_shorter_multi_indices_and_errors(built_pkg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    p = build(16, 2, 6, pkg.top_weight_multiindices(6, 20, C.decay_factors))
    mis4 = pkg.total_degree_multiindices(4, 2)
    TB4 = pkg.TensorizedBasis(pkg.LegendrePolynomials, 4, 2, 6, multi_indices=mis4)
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    op.update_basis(TB4)
    fresh = pkg.SGOperator(p.V, TB4, p.Kall[:5], device=0)
    x = np.random.default_rng(4).standard_normal(p.n * TB4.nmodes)
    assert np.array_equal(op.mul(x, pkg.FP64), fresh.mul(x, pkg.FP64))
    yref = osg.mul_literal(x, p.K0, p.Ks[:4], TB4.G.toarray(), p.bdofs, TB4.nmodes)
    assert np.linalg.norm(op.mul(x, pkg.FP64) - yref) <= 1e-12 * np.linalg.norm(yref)
    xa = np.zeros(p.n * TB4.nmodes)
    xb = np.zeros(p.n * TB4.nmodes)
    op.solve_primal(p.b0, xa, rtol=1e-10, precision=pkg.MIXED)
    fresh.solve_primal(p.b0, xb, rtol=1e-10, precision=pkg.MIXED)
    assert np.linalg.norm(xa - xb) <= 1e-9 * np.linalg.norm(xb)
    mis8 = pkg.total_degree_multiindices(8, 1)
    TB8 = pkg.TensorizedBasis(pkg.LegendrePolynomials, 8, 1, 5, multi_indices=mis8)
    with pytest.raises(ValueError):
        op.update_basis(TB8)
    op.close()
    fresh.close()
