"""GPU residual estimator (K4) against the oracle's restatement of
estimate(::Type{PoissonProblemPrimal}), src/estimate.jl:260-418.
Bar: per element (every cell and extended mode) 1e-10 relative to the largest
value of that mode (cells where a mode's estimator is exactly zero stay
zero), eta4modes 1e-10 relative, identical extended multi-index sets."""
import numpy as np
import pytest

from oracle import basis as ob
from oracle import coefficient as oc
from oracle import estimate as oe
from oracle import fem as of
from tests.problems import build, config1_like

pytestmark = pytest.mark.gpu


def run_both(p, bonus=2, tail=(10, 2), solve=True):
    pkg = p.pkg
    if solve:
        op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
        op.solve_primal(p.b0, p.sol.entries, rtol=1e-11, precision=pkg.FP64)
    else:
        op = None
        p.sol.entries[:] = np.random.default_rng(5).standard_normal(len(p.sol.entries))
    f = lambda x, y: np.ones_like(x)
    em, ec, ext = pkg.estimate(pkg.PoissonProblemPrimal, p.sol, p.C, rhs=f, bonus_quadorder=bonus,
                               tail_extension=tail, op=op)
    Vo = of.LagrangeSpace(of.StructuredMesh(p.V.mesh.ncells and int(round(np.sqrt(p.V.mesh.ncells / 2)))), p.V.order)
    Co = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=p.C.mean_value, maxm=p.C.maxm())
    obt = ob.LEGENDRE if p.TB.basis.name == "legendre" else ob.HERMITE
    om, oc_, oext = oe.estimate_primal(Vo, p.sol.entries, p.mis, obt, Co, lambda x, y: 1.0 + 0 * x,
                                       bonus_quadorder=bonus, tail_extension=tail)
    if op is not None:
        op.close()
    return (em, ec, ext), (om, oc_, oext)


def check(g, o):
    em, ec, ext = g
    om, oc_, oext = o
    assert ext == oext
    assert ec.shape == oc_.shape
    assert np.max(np.abs(em - om) / np.maximum(np.abs(om), 1e-300)) <= 1e-10
    scale = np.maximum(np.abs(oc_).max(axis=0), 1e-300)
    assert np.max(np.abs(ec - oc_) / scale) <= 1e-10
    assert np.array_equal(ec == 0.0, oc_ == 0.0)


def test_estimator_config1(built_pkg):
    p = config1_like(N=16)
    check(*run_both(p))


def test_estimator_p2(built_pkg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    p = build(8, 2, 4, pkg.top_weight_multiindices(4, 10, C.decay_factors))
    check(*run_both(p, bonus=2))


def test_estimator_random_solution_and_tail(built_pkg):
    """Any SG vector (not only solutions), other tail extension and quadrature."""
    p = build(8, 2, 3, [[0, 0, 0], [1, 0, 0], [0, 1, 0], [2, 0, 0], [0, 0, 1]])
    check(*run_both(p, bonus=1, tail=(5, 1), solve=False))


def test_estimator_marking_decision(built_pkg):
    """Marking on the GPU estimator gives the oracle's (bit-exact) decisions."""
    from oracle import mopcontrol as om_
    p = config1_like(N=16, M=3, deg=2)
    g, o = run_both(p)
    a = p.pkg.stochastic_marking(list(g[0]), g[2], p.P, p.mis)
    b = om_.stochastic_marking(list(o[0]), o[2], p.P, p.mis)
    assert a[0] == b[0] and a[1] == b[1] and a[2]["sorted_id"] == b[2]["sorted_id"]
