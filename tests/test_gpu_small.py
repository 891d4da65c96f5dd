"""The one-cluster inner PCG of the mixed solve (csrc/small.cu) for small P1
lattice problems: the whole FP32 PCG of a refinement step (the iterations of
solve_primal!, solvers_poisson_primal.jl:130-169, with the mean-based
preconditioner :47-78) in one thread-block-cluster launch.

Bars: the mixed solve meets rtol on the FP64 residual, matches the oracle's
GMRES solution (the reference solve) to 100 * rtol, and agrees with the
multi-launch inner PCG (SGFEM_SMALL=0) to 1e-8 with the same iteration count
to within two."""
import re

import numpy as np
import pytest

from oracle import sg as osg
from tests.problems import build, config1_like

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def launches(op):
    """One-cluster PCG launches on the context so far (parsed from its log)."""
    m = re.search(r"launches: (\d+)", op.ctx.small_solve_log)
    return int(m.group(1)) if m else -1


def oracle_solution(p):
    n, P = p.n, p.P
    prec = osg.MeanPreconditioner(p.K0, p.bdofs, P)
    b = osg.reference_rhs(np.zeros(n * P), p.b0, p.bdofs, P)
    xg, _ = osg.gmres_left(lambda v: osg.apply_fast(v, p.K0, p.Ks, p.G, p.bdofs, P), prec.ldiv, b, np.zeros(n * P))
    return xg


@pytest.mark.parametrize("rtol", [1e-8, 1e-10])
def test_small_mixed_solve_config1(built_pkg, monkeypatch, rtol):
    p = config1_like()
    pkg = p.pkg
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    assert "one-cluster" in op.ctx.small_solve_log, op.ctx.small_solve_log
    monkeypatch.setenv("SGFEM_SMALL", "0")
    op_ml = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    monkeypatch.delenv("SGFEM_SMALL")
    assert "disabled" in op_ml.ctx.small_solve_log
    ref = oracle_solution(p)
    xs, xm = np.zeros(p.n * p.P), np.zeros(p.n * p.P)
    ss = op.solve_primal(p.b0, xs, rtol=rtol, precision=pkg.MIXED)
    assert launches(op) == ss["outer_iterations"] > 0, (op.ctx.small_solve_log, ss)
    sm = op_ml.solve_primal(p.b0, xm, rtol=rtol, precision=pkg.MIXED)
    assert ss["relres"] <= rtol and sm["relres"] <= rtol
    assert rel(xs, ref) <= 100 * rtol
    assert rel(xs, xm) <= 100 * rtol
    assert abs(ss["iterations"] - sm["iterations"]) <= 2, (ss, sm)
    b = osg.reference_rhs(np.zeros(p.n * p.P), p.b0, p.bdofs, p.P)
    r = b - osg.apply_fast(xs, p.K0, p.Ks, p.G, p.bdofs, p.P)
    assert np.linalg.norm(r) <= 1.01 * rtol * np.linalg.norm(b)
    # repeated solves on the context give the same answer
    x2 = np.zeros(p.n * p.P)
    op.solve_primal(p.b0, x2, rtol=rtol, precision=pkg.MIXED)
    assert np.array_equal(xs, x2)
    op.close()
    op_ml.close()


@pytest.mark.parametrize("N,M,deg,cl", [(16, 3, 2, None), (32, 4, 2, "8"), (8, 6, 1, None), (32, 5, 2, "8"),
                                         (16, 10, 1, None)])
def test_small_other_shapes_and_update(built_pkg, monkeypatch, N, M, deg, cl):
    """Other lattice sizes (cluster shares of 0 to 5 lines), term counts (4 to 7
    with the specialised applies, 11 with the run-time one), both cluster sizes
    (16 CTAs, and the portable 8), and a coupling update (new tables for the
    grown multi-index set)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    if cl:
        monkeypatch.setenv("SGFEM_SMALL_CLUSTER", cl)
    p = build(N, 1, M, pkg.total_degree_multiindices(M, deg))
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    assert "one-cluster" in op.ctx.small_solve_log, op.ctx.small_solve_log
    if cl:
        assert f"{cl} CTAs" in op.ctx.small_solve_log
    x = np.zeros(p.n * p.P)
    st = op.solve_primal(p.b0, x, rtol=1e-10, precision=pkg.MIXED)
    assert launches(op) == st["outer_iterations"] > 0, (op.ctx.small_solve_log, st)
    ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P) if p.n * p.P < 30000 else oracle_solution(p)
    assert st["relres"] <= 1e-10 and rel(x, ref) <= 1e-8
    mis2 = pkg.total_degree_multiindices(M, deg + 1)
    TB2 = pkg.TensorizedBasis(pkg.LegendrePolynomials, M, deg + 1, deg + 5, multi_indices=mis2)
    if TB2.nmodes <= 32:
        op.update_basis(TB2)
        x2 = np.zeros(p.n * TB2.nmodes)
        n0 = launches(op)
        st2 = op.solve_primal(p.b0, x2, rtol=1e-10, precision=pkg.MIXED)
        assert launches(op) - n0 == st2["outer_iterations"] > 0, (op.ctx.small_solve_log, st2)
        b = osg.reference_rhs(np.zeros(p.n * TB2.nmodes), p.b0, p.bdofs, TB2.nmodes)
        r = b - osg.apply_fast(x2, p.K0, p.Ks, TB2.G.toarray(), p.bdofs, TB2.nmodes)
        assert st2["relres"] <= 1e-10 and np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(b)
    op.close()


def test_small_not_used_where_it_does_not_apply(built_pkg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    p2 = build(16, 2, 3, pkg.total_degree_multiindices(3, 2))  # P2: rows couple lines two apart
    op = pkg.SGOperator(p2.V, p2.TB, p2.Kall, device=0)
    assert "beyond the neighbouring lattice lines" in op.ctx.small_solve_log, op.ctx.small_solve_log
    op.close()
    odd = build(12, 1, 3, pkg.total_degree_multiindices(3, 2))  # 12 intervals: no power-of-two lattice
    op = pkg.SGOperator(odd.V, odd.TB, odd.Kall, device=0)
    assert "power-of-two P1 dof lattice" in op.ctx.small_solve_log, op.ctx.small_solve_log
    op.close()
    big = build(16, 1, 6, pkg.total_degree_multiindices(6, 2))  # 28 modes: fits; 7 terms
    op = pkg.SGOperator(big.V, big.TB, big.Kall, device=0)
    assert "one-cluster" in op.ctx.small_solve_log
    op.close()
    many = build(16, 1, 8, pkg.total_degree_multiindices(8, 2))  # 45 modes: more than 32
    op = pkg.SGOperator(many.V, many.TB, many.Kall, device=0)
    assert "32 modes" in op.ctx.small_solve_log
    op.close()
    large = build(128, 1, 3, pkg.total_degree_multiindices(3, 1))  # 129 lines: no cluster share fits
    op = pkg.SGOperator(large.V, large.TB, large.Kall, device=0)
    assert "no cluster shape fits" in op.ctx.small_solve_log
    op.close()


def test_small_reports_breakdown_like_the_multi_launch_path(built_pkg, monkeypatch):
    """An indefinite SG operator (mean 0.05 against KLE amplitudes summing to ~1.3;
    the oracle's PCG meets p'Ap < 0 at its second iteration): the one-cluster inner
    PCG returns SGFEM_ERR_BREAKDOWN (with a zero correction) like the multi-launch
    FP32 PCG, through the same error of sgfem_solve."""
    import sys
    import __graft_entry__ as ge
    pkg = ge.load_package()
    lib = sys.modules[pkg.__name__ + "._lib"]
    ERR_BREAKDOWN, SGError = lib.ERR_BREAKDOWN, lib.SGError
    p = build(32, 1, 5, pkg.total_degree_multiindices(5, 2), mean=0.05)
    codes = {}
    for small in ("1", "0"):
        monkeypatch.setenv("SGFEM_SMALL", small)
        op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
        assert ("one-cluster" in op.ctx.small_solve_log) == (small == "1"), op.ctx.small_solve_log
        x = np.zeros(p.n * p.P)
        with pytest.raises(SGError) as e:
            op.solve_primal(p.b0, x, rtol=1e-8, precision=pkg.MIXED)
        codes[small] = e.value.code
        if small == "1":
            assert launches(op) == 1
        assert np.all(np.isfinite(x))
        op.close()
    assert codes["1"] == codes["0"] == ERR_BREAKDOWN, codes
