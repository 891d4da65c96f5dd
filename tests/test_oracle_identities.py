"""Identities that pin the oracle's operator and solvers where the reference
has no tests (CPU only): the literal per-G-nonzero apply equals the explicit
Kronecker matrix of solve_full_primal!, the C restatement equals the Python
one, the operator is symmetric on interior dofs, GMRES (the reference's
solver) and PCG agree with the direct Kronecker solve, and P = 1 reduces to
the deterministic problem."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle import cbuild
from oracle import sg as osg
from tests.problems import config1_like


@pytest.fixture(scope="module")
def prob():
    return config1_like(N=8, M=3, deg=2)


def test_literal_apply_equals_grouped(prob):
    x = np.random.default_rng(0).standard_normal(prob.n * prob.P)
    a = osg.mul_literal(x, prob.K0, prob.Ks, prob.G, prob.bdofs, prob.P)
    b = osg.apply_fast(x, prob.K0, prob.Ks, prob.G, prob.bdofs, prob.P)
    assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a)


def test_c_restatement_equals_python(prob):
    op = cbuild.COperator([prob.K0] + prob.Ks, prob.G, prob.bdofs, prob.P)
    x = np.random.default_rng(1).standard_normal(prob.n * prob.P)
    a = osg.mul_literal(x, prob.K0, prob.Ks, prob.G, prob.bdofs, prob.P)
    for th in (1, 4):
        b = op.mul(x, nthreads=th)
        assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a)


def test_symmetric_on_interior(prob):
    rng = np.random.default_rng(2)
    mask = osg.interior_mask(prob.n, prob.P, prob.bdofs)
    u = rng.standard_normal(prob.n * prob.P) * mask
    v = rng.standard_normal(prob.n * prob.P) * mask
    au = osg.mul_literal(u, prob.K0, prob.Ks, prob.G, prob.bdofs, prob.P)
    av = osg.mul_literal(v, prob.K0, prob.Ks, prob.G, prob.bdofs, prob.P)
    assert abs(v @ au - u @ av) <= 1e-13 * abs(v @ au)
    assert u @ au > 0


def test_gmres_pcg_direct_agree(prob):
    n, P = prob.n, prob.P
    prec = osg.MeanPreconditioner(prob.K0, prob.bdofs, P)
    b = osg.reference_rhs(np.zeros(n * P), prob.b0, prob.bdofs, P)
    ap = lambda v: osg.mul_literal(v, prob.K0, prob.Ks, prob.G, prob.bdofs, P)
    xg, st = osg.gmres_left(ap, prec.ldiv, b, np.zeros(n * P))
    assert st["solved"]
    xk = osg.kron_direct(prob.K0, prob.Ks, prob.G, prob.b0, prob.bdofs, P)
    xp, _ = osg.pcg(ap, prec.ldiv, b, np.zeros(n * P), osg.interior_mask(n, P, prob.bdofs), tol=1e-13)
    assert np.linalg.norm(xg - xk) <= 1e-12 * np.linalg.norm(xk)
    assert np.linalg.norm(xp - xk) <= 1e-11 * np.linalg.norm(xk)


def test_single_mode_is_deterministic_solve():
    p = config1_like(N=8, M=2, deg=0)
    assert p.P == 1
    xk = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, 1)
    inner = np.setdiff1d(np.arange(p.n), p.bdofs)
    u = np.zeros(p.n)
    u[inner] = spla.spsolve(p.K0[inner][:, inner].tocsc(), p.b0[inner])
    assert np.linalg.norm(xk - u) <= 1e-12 * np.linalg.norm(u)


def test_pce_lambda_generating_function():
    """lambda_mu of exp(factor a) (coefficients.jl:219-260) are the normalised
    Hermite chaos coefficients: sum_mu lambda_mu H_mu(y) -> exp(factor a(x, y))
    (generating function exp(t y - t^2/2) = sum_k t^k He_k(y) / k!)."""
    from oracle import basis as ob
    from oracle import coefficient as oc
    C = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.3, maxm=2)
    x1, x2 = 0.31, 0.77
    y = np.array([0.7, -1.3])
    K = 28
    mis = [[i, j] for i in range(K + 1) for j in range(K + 1 - i)]
    TB = ob.TensorizedBasis(ob.HERMITE, 2, K, K, multi_indices=mis)
    TB.set_sample(list(y))
    for factor in (-1.0, 1.0):
        s = sum(oc.pce_lambda(C, mu, x1, x2, factor, N_truncate=2) * TB.evaluate(k) for k, mu in enumerate(mis))
        a = C.get_a(x1, x2, y)
        assert abs(s - np.exp(factor * float(a))) <= 1e-11 * np.exp(factor * float(a))


def test_adjoint_oracle_matches_finite_differences():
    """The oracle's adjoint gradient of J = int_box E[u] against central
    differences of its own assembled Kronecker solves."""
    from oracle import adjoint as oa
    from oracle import basis as ob
    from oracle import coefficient as oc
    from oracle import fem as of
    from oracle import mopcontrol as om
    M = 2
    mis = om.generate_multiindices(M, 2)
    TB = ob.TensorizedBasis(ob.LEGENDRE, M, 2, 4, multi_indices=mis)
    V = of.LagrangeSpace(of.StructuredMesh(4), 1)
    C = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=10)
    Q = oa.QoIOracle(V, C, TB.G, len(mis), M, lambda x, y: 1.0)
    rng = np.random.default_rng(0)
    theta = 1.0 + 0.1 * rng.standard_normal(M)
    alpha = 1.0 + 0.1 * rng.standard_normal(V.mesh.nnodes)
    J, gt, ga = Q.gradient(theta, alpha)
    h = 1e-6
    for _ in range(3):
        dt = rng.standard_normal(M)
        da = rng.standard_normal(V.mesh.nnodes)
        fd = (Q.value(theta + h * dt, alpha + h * da) - Q.value(theta - h * dt, alpha - h * da)) / (2 * h)
        an = gt @ dt + ga @ da
        assert abs(fd - an) <= 1e-6 * abs(an)


@pytest.mark.parametrize("order,N", [(1, 8), (2, 4), (2, 8)])
def test_sine_transform_blocks_of_lattice_stiffness(order, N):
    """The exact lattice preconditioner rests on this: the orthonormal 2-D sine
    transform S maps the interior stiffness K_0 of P1/P2 on the uniform
    triangulation to 4x4 blocks on the frequencies {i, Nl-i} x {j, Nl-j}, and the
    blocks equal the separable sums over the stencil of each parity class,
      B_ab = sum_c sum_d w_c(d) X_c,dx(a_x, b_x) X_c,dy(a_y, b_y)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from tests.problems import build
    p = build(N, order, 1, [[0]])
    K = p.K0.toarray()
    Nl = N * order
    xy = np.rint(p.V.dof_coords * Nl).astype(int)
    idx = {(x, y): i for i, (x, y) in enumerate(xy)}
    interior = [(x, y) for y in range(1, Nl) for x in range(1, Nl)]
    I = [idx[q] for q in interior]
    j = np.arange(1, Nl)
    S1 = np.sqrt(2.0 / Nl) * np.sin(np.pi * np.outer(j, j) / Nl)
    T = np.kron(S1, S1) @ K[np.ix_(I, I)] @ np.kron(S1, S1)
    pos = lambda kx, ky: (ky - 1) * (Nl - 1) + kx - 1
    R = 2
    w = np.zeros((2, 2, 2 * R + 1, 2 * R + 1))
    for cy in range(2):
        for cx in range(2):
            x0, y0 = Nl // 2 + cx, Nl // 2 + cy
            for dy in range(-R, R + 1):
                for dx in range(-R, R + 1):
                    w[cy, cx, dy + R, dx + R] = K[idx[(x0, y0)], idx[(x0 + dx, y0 + dy)]]
    s = lambda k, x: np.sqrt(2.0 / Nl) * np.sin(np.pi * k * x / Nl)

    def X(i, c, d, a, b):
        f = (i, Nl - i)
        return sum(s(f[a], x) * s(f[b], x + d) for x in range(c, Nl, 2) if 1 <= x and 1 <= x + d <= Nl - 1)

    H = Nl // 2
    for kx in range(1, Nl):
        for ky in range(1, Nl):
            row = T[pos(kx, ky)]
            alias = {pos(a, b) for a in (kx, Nl - kx) for b in (ky, Nl - ky)}
            assert np.all(np.abs(np.delete(row, sorted(alias))) <= 1e-12)
    for i in range(1, H + 1):
        for jy in range(1, H + 1):
            fx, fy = (i, Nl - i), (jy, Nl - jy)
            for a in range(4):
                for b in range(4):
                    if (i == H and (a % 2 or b % 2)) or (jy == H and (a // 2 or b // 2)):
                        continue
                    B = sum(w[cy, cx, dy + R, dx + R] * X(i, cx, dx, a % 2, b % 2) * X(jy, cy, dy, a // 2, b // 2)
                            for cy in range(2) for cx in range(2) for dy in range(-R, R + 1) for dx in range(-R, R + 1)
                            if w[cy, cx, dy + R, dx + R] != 0.0)
                    assert abs(B - T[pos(fx[a % 2], fy[a // 2]), pos(fx[b % 2], fy[b // 2])]) <= 1e-12


@pytest.mark.parametrize("k", [1, 2])
def test_equilibration_rt_space_is_conforming(k):
    """The oracle's RT_k basis (per physical cell, dual to normal-flux point
    values on each edge and interior moments): the normal flux of a face dof
    agrees from both sides of the face, every other basis function of the two
    cells has zero normal flux there, and div maps onto P_k (piecewise)."""
    from oracle import equilibration as oq
    from oracle import fem as of
    m = of.StructuredMesh(3)
    rt = oq.RTSpace(m, k)
    worst = 0.0
    for f in range(m.nfaces):
        c0, c1 = m.face_cells[f]
        if c1 < 0:
            continue
        A, B = sorted(m.face_nodes[f])
        pa, pb = m.coords[A], m.coords[B]
        nrm = np.array([pb[1] - pa[1], -(pb[0] - pa[0])])
        for t in (0.11, 0.5, 0.83):
            x = pa + t * (pb - pa)
            flux = {}
            for c in (c0, c1):
                v, _ = rt.eval(c, x)
                for i, dof in enumerate(rt.celldofs[c]):
                    on_face = (k + 1) * f <= dof < (k + 1) * (f + 1)
                    if on_face:
                        flux.setdefault(dof, []).append(v[i] @ nrm)
                    else:
                        worst = max(worst, abs(v[i] @ nrm))
            for vals in flux.values():
                assert len(vals) == 2
                worst = max(worst, abs(vals[0] - vals[1]))
    assert worst <= 1e-10


def test_equilibration_oracle_vanishes_for_zero_data():
    """u_h = 0 and f = 0: every local flux and the estimate vanish."""
    from oracle import basis as ob
    from oracle import coefficient as oc
    from oracle import equilibration as oq
    from oracle import fem as of
    V = of.LagrangeSpace(of.StructuredMesh(3), 1)
    C = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=40)
    mis = [[0, 0], [1, 0], [0, 1]]
    em, ec, ext = oq.estimate_equilibration(V, np.zeros(V.ndofs * 3), mis, ob.LEGENDRE, C, lambda x, y: 0.0 * x)
    assert np.all(em == 0.0) and np.all(ec == 0.0)


def test_equilibration_oracle_is_basis_independent(monkeypatch):
    """The estimate does not depend on the RT_k basis: the oracle with its edge
    functionals at other points along each edge (another basis of the same
    constrained spaces) agrees to the conditioning of the penalised patch
    systems (div penalty 1e5: 1e-7 per element, 1e-8 for eta4modes)."""
    import numpy as np
    from oracle import basis as ob
    from oracle import coefficient as oc
    from oracle import equilibration as oq
    from oracle import fem as of
    V = of.LagrangeSpace(of.StructuredMesh(4), 2)
    C = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=40)
    mis = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [2, 0, 0], [0, 0, 1]]
    U = np.random.default_rng(11).standard_normal(V.ndofs * len(mis))
    f = lambda x, y: 1.0 + x * y
    a = oq.estimate_equilibration(V, U, mis, ob.LEGENDRE, C, f)
    orig = oq.RTSpace.__init__

    def other_points(self, mesh, k):
        gauss = np.polynomial.legendre.leggauss
        np.polynomial.legendre.leggauss = lambda n: (np.linspace(-0.8, 0.8, n), np.ones(n))
        try:
            orig(self, mesh, k)
        finally:
            np.polynomial.legendre.leggauss = gauss

    monkeypatch.setattr(oq.RTSpace, "__init__", other_points)
    b = oq.estimate_equilibration(V, U, mis, ob.LEGENDRE, C, f)
    assert a[2] == b[2]
    assert np.max(np.abs(a[0] - b[0]) / a[0]) <= 1e-8
    assert np.max(np.abs(a[1] - b[1]) / np.abs(a[1]).max(axis=0)) <= 1e-7
