"""Adjoint gradient of J = int_[0.25,0.75]^2 E[u] dx with respect to the KLE
block factors theta_m and the nodal mean field alpha (forward and adjoint
device PCG + sgfem_adjoint_gradient) against the oracle's assembled Kronecker
solves, and against central finite differences (h = 1e-6) of the device
forward solve on 20 random directions (config-1 sizes)."""
import numpy as np
import pytest

from oracle import adjoint as oa
from oracle import basis as ob
from oracle import coefficient as oc
from oracle import fem as of

pytestmark = pytest.mark.gpu


def setup(N, M, deg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), 1)
    mis = pkg.total_degree_multiindices(M, deg)
    TB = pkg.TensorizedBasis(pkg.LegendrePolynomials, M, deg, deg + 4, multi_indices=mis)
    Q = pkg.MeanQoI(V, TB, C, rhs=lambda x, y: np.ones_like(x))
    return pkg, C, V, TB, mis, Q


def test_adjoint_gradient_matches_oracle(built_pkg):
    pkg, C, V, TB, mis, Q = setup(8, 3, 2)
    rng = np.random.default_rng(1)
    theta = 1.0 + 0.2 * rng.standard_normal(3)
    alpha = 1.0 + 0.2 * rng.random(V.mesh.nnodes)
    J, gt, ga, st = Q.value_and_gradient(theta, alpha, rtol=1e-13)
    TBo = ob.TensorizedBasis(ob.LEGENDRE, 3, 2, 6, multi_indices=mis)
    Vo = of.LagrangeSpace(of.StructuredMesh(8), 1)
    Co = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    Qo = oa.QoIOracle(Vo, Co, TBo.G, len(mis), 3, lambda x, y: 1.0)
    Jo, gto, gao = Qo.gradient(theta, alpha)
    assert abs(J - Jo) <= 1e-10 * abs(Jo)
    assert np.max(np.abs(gt - gto)) <= 1e-8 * np.max(np.abs(gto))
    assert np.max(np.abs(ga - gao)) <= 1e-8 * np.max(np.abs(gao))


def test_adjoint_gradient_finite_differences_config1(built_pkg):
    pkg, C, V, TB, mis, Q = setup(32, 5, 2)
    theta = np.ones(5)
    alpha = np.ones(V.mesh.nnodes)
    J, gt, ga, st = Q.value_and_gradient(theta, alpha, rtol=2e-13)
    rng = np.random.default_rng(2)
    h = 1e-6
    errs = []
    for _ in range(20):
        dt = rng.standard_normal(5)
        da = rng.standard_normal(V.mesh.nnodes)
        fd = (Q.value(theta + h * dt, alpha + h * da, rtol=2e-13) -
              Q.value(theta - h * dt, alpha - h * da, rtol=2e-13)) / (2 * h)
        an = gt @ dt + ga @ da
        errs.append(abs(fd - an) / abs(an))
    assert max(errs) <= 1e-5, errs


def test_torch_function_and_rrule(built_pkg):
    torch = pytest.importorskip("torch")
    pkg, C, V, TB, mis, Q = setup(8, 2, 1)
    from importlib import import_module
    adj = import_module(pkg.__name__ + ".adjoint")
    theta = torch.ones(2, dtype=torch.float64, requires_grad=True)
    alpha = torch.ones(V.mesh.nnodes, dtype=torch.float64, requires_grad=True)
    J = adj.MeanQoIFunction.apply(theta, alpha, Q)
    (2.0 * J).backward()
    J2, pb = Q.rrule(theta.detach().numpy(), alpha.detach().numpy())
    gt, ga = pb(2.0)
    assert abs(J.item() - J2) <= 1e-14 * abs(J2)
    assert np.allclose(theta.grad.numpy(), gt, rtol=1e-13, atol=0)
    assert np.allclose(alpha.grad.numpy(), ga, rtol=1e-13, atol=0)
