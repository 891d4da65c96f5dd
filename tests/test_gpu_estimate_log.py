"""GPU estimator of LogTransformedPoissonProblemPrimal against the oracle's
element loops (estimate.jl:70-257).  Bar: per element 1e-10 relative to the
largest value of the mode, eta4modes 1e-10 relative, zeta 1e-10 relative,
identical extended multi-index sets."""
import numpy as np
import pytest

from oracle import basis as ob
from oracle import coefficient as oc
from oracle import estimate as oe
from oracle import fem as of

pytestmark = pytest.mark.gpu


def setup_log(N, order, M, deg, solve=True):
    from tests.test_gpu_lognormal import build_log
    p = build_log(N, order, M, deg)
    if solve:
        op = p.pkg.SGOperator(p.V, p.TB, p.Ks, device=0)
        op.solve_logpoisson(p.b, p.sol.entries, rtol=1e-12, precision=p.pkg.FP64)
        op.close()
    return p


def compare(p, bonus):
    pkg = p.pkg
    f = lambda x, y: np.ones_like(x)
    em, ec, ext, z = pkg.estimate(pkg.LogTransformedPoissonProblemPrimal, p.sol, p.C, rhs=f,
                                  bonus_quadorder=bonus, tail_extension=(10, 2))
    N = int(round(np.sqrt(p.V.mesh.ncells / 2)))
    Vo = of.LagrangeSpace(of.StructuredMesh(N), p.V.order)
    Co = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.0, maxm=p.C.maxm())
    mis = [list(m) for m in p.TB.multi_indices]
    om, oc_, oext, oz = oe.estimate_logpoisson(Vo, p.sol.entries, mis, ob.HERMITE, Co, lambda x, y: 1.0,
                                               bonus_quadorder=bonus, tail_extension=(10, 2))
    assert ext == oext
    assert ec.shape == oc_.shape
    assert np.max(np.abs(em - om) / np.abs(om)) <= 1e-10
    scale = np.maximum(np.abs(oc_).max(axis=0), 1e-300)
    assert np.max(np.abs(ec - oc_) / scale) <= 1e-10
    assert abs(z - oz) <= 1e-10 * abs(oz)


def test_log_estimator_p1(built_pkg):
    compare(setup_log(4, 1, 2, 2), bonus=1)


def test_log_estimator_p1_bonus2(built_pkg):
    compare(setup_log(4, 1, 2, 1), bonus=2)


def test_log_estimator_p2(built_pkg):
    compare(setup_log(4, 2, 2, 1), bonus=0)  # quadorder 2: interpolation degree 2


def test_log_estimator_tail_extension_int_raises(built_pkg):
    p = setup_log(4, 1, 1, 1, solve=False)
    with pytest.raises(TypeError):
        p.pkg.estimate(p.pkg.LogTransformedPoissonProblemPrimal, p.sol, p.C, rhs=lambda x, y: np.ones_like(x),
                       tail_extension=5)
