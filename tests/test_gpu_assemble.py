"""GPU assembly of the stiffness matrices K_m of the cosine coefficient
(sgfem_assemble_stiffness) against the host assembly (the caller-side
restatement of ExtendableFEM's BilinearOperator assembly, poisson_primal.jl:
56-68): same pattern, values within 1e-13 of the largest entry, bitwise
reproducible, and a solve on GPU-assembled blocks matches one on host blocks.
Right-hand sides (sgfem_assemble_rhs, sgfem_assemble_pce_rhs) against the host
LinearOperator restatement (poisson_primal.jl:65-68, logpoisson_primal.jl:
109-131 with lambda_mu of coefficients.jl:219-260)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order,N,M", [(1, 16, 6), (2, 8, 6), (2, 16, 20)])
def test_gpu_stiffness_matches_host(built_pkg, order, N, M):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.3, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), order)
    qo = 2 * (order - 1) + 2
    host = pkg.assemble_stiffness(V, C, list(range(M + 1)), qo)
    gpu = pkg.assemble_stiffness_gpu(V, C, list(range(M + 1)), qo)
    for m, (A, B) in enumerate(zip(host, gpu)):
        assert np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)
        scale = np.abs(A.data).max()
        assert np.abs(A.data - B.data).max() <= 1e-13 * scale, m
    again = pkg.assemble_stiffness_gpu(V, C, list(range(M + 1)), qo)
    assert all(np.array_equal(a.data, b.data) for a, b in zip(gpu, again))
    part = pkg.assemble_stiffness_gpu(V, C, [3, 4, 5], qo)
    assert all(np.array_equal(a.data, b.data) for a, b in zip(part, gpu[3:6]))


@pytest.mark.parametrize("order,N", [(1, 16), (2, 8)])
def test_gpu_stiffness_and_rhs_match_oracle(built_pkg, order, N):
    """The GPU-assembled K_m and b directly against the oracle's element loops
    (oracle/fem.py: the same structured mesh, dof numbering and triangle rules)."""
    import __graft_entry__ as ge
    from oracle import coefficient as oc
    from oracle import fem as of
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.3, maxm=150)
    Co = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.3, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), order)
    Vo = of.LagrangeSpace(of.StructuredMesh(N), order)
    ms = list(range(7))
    qo = 2 * (order - 1) + 2
    gpu = pkg.assemble_stiffness_gpu(V, C, ms, qo)
    ref = of.assemble_stiffness(Vo, Co, ms, qo)
    for m, A, R in zip(ms, gpu, ref):
        d = (A - R).toarray()
        assert np.abs(d).max() <= 1e-13 * np.abs(R.toarray()).max(), m
    bg = pkg.assemble_rhs_gpu(V, lambda x, y: np.ones_like(x), order)
    bo = of.assemble_rhs(Vo, lambda x, y: 1.0, order)
    assert np.abs(bg - bo).max() <= 1e-14 * np.abs(bo).max()


def test_solve_on_gpu_assembled_blocks(built_pkg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(16), 2)
    mis = pkg.top_weight_multiindices(6, 30, C.decay_factors)
    TB = pkg.TensorizedBasis(pkg.LegendrePolynomials, 6, max(max(m) for m in mis), max(max(m) for m in mis) + 4,
                             multi_indices=mis)
    sol = pkg.SGFEVector(V, TB)
    f = lambda x, y: np.ones_like(x)
    Kh, b0 = pkg.assemble(pkg.PoissonProblemPrimal, sol, C, rhs=f)
    Kg, b0g = pkg.assemble(pkg.PoissonProblemPrimal, sol, C, rhs=f, device=0)
    assert np.abs(b0 - b0g).max() <= 1e-14 * np.abs(b0).max()
    xs = []
    for Ks in (Kh, Kg):
        op = pkg.SGOperator(V, TB, Ks, device=0)
        x = np.zeros(V.ndofs * TB.nmodes)
        st = op.solve_primal(b0, x, rtol=1e-10, precision=pkg.FP64)
        assert st["relres"] <= 1e-10
        xs.append(x)
        op.close()
    assert np.linalg.norm(xs[0] - xs[1]) <= 1e-11 * np.linalg.norm(xs[0])


def test_assembly_argument_errors(built_pkg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=10)
    V = pkg.H1Pk(pkg.unit_square_mesh(4), 1)
    with pytest.raises(ValueError):
        pkg.assemble_stiffness_gpu(V, C, [0, 2], 2)  # not a contiguous range of terms
    with pytest.raises(pkg.SGError):
        pkg.assemble_stiffness_gpu(V, C, list(range(0, 12)), 2)  # beyond maxm = 10


@pytest.mark.parametrize("order,N,qo", [(1, 16, 1), (2, 12, 2), (2, 8, 4)])
def test_gpu_rhs_matches_host(built_pkg, order, N, qo):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    V = pkg.H1Pk(pkg.unit_square_mesh(N), order)
    f = lambda x, y: np.sin(3 * x) * (1 + y * y) - 0.5
    host = pkg.assemble_rhs(V, f, qo)
    gpu = pkg.assemble_rhs_gpu(V, f, qo)
    assert np.abs(host - gpu).max() <= 1e-14 * np.abs(host).max()
    assert np.array_equal(gpu, pkg.assemble_rhs_gpu(V, f, qo))


@pytest.mark.parametrize("order,N,M,deg,factor,ntrunc", [(1, 16, 4, 2, -1.0, None), (2, 8, 6, 3, -1.0, 8),
                                                         (1, 8, 3, 3, 0.5, 3)])
def test_gpu_pce_rhs_matches_host(built_pkg, order, N, M, deg, factor, ntrunc):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.3, maxm=20)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), order)
    mis = pkg.total_degree_multiindices(M, deg)
    f = lambda x, y: 1.0 + x * y
    qo = order + 1
    host = pkg.assemble_pce_rhs(V, C, mis, f, qo, factor=factor, N_truncate=ntrunc)
    gpu = pkg.assemble_pce_rhs_gpu(V, C, mis, f, qo, factor=factor, N_truncate=ntrunc)
    n = V.ndofs
    for k in range(len(mis)):
        h, g = host[k * n:(k + 1) * n], gpu[k * n:(k + 1) * n]
        assert np.abs(h - g).max() <= 1e-13 * max(np.abs(h).max(), 1e-300), (k, mis[k])


def test_lognormal_solve_on_gpu_rhs(built_pkg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.0, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(16), 1)
    mis = pkg.total_degree_multiindices(4, 2)
    TB = pkg.TensorizedBasis(pkg.HermitePolynomials, 4, 2, 6, multi_indices=mis)
    sol = pkg.SGFEVector(V, TB)
    f = lambda x, y: np.ones_like(x)
    Kh, bh = pkg.assemble(pkg.LogTransformedPoissonProblemPrimal, sol, C, rhs=f)
    Kg, bg = pkg.assemble(pkg.LogTransformedPoissonProblemPrimal, sol, C, rhs=f, device=0)
    assert np.abs(bh - bg).max() <= 1e-13 * np.abs(bh).max()
    for m, (A, B) in enumerate(zip(Kh, Kg)):
        assert abs(A - B).max() <= 1e-13 * abs(A).max(), m
    xs = []
    for Ks, b in ((Kh, bh), (Kg, bg)):
        op = pkg.SGOperator(V, TB, Ks, device=0)
        x = np.zeros(V.ndofs * TB.nmodes)
        st = op.solve_logpoisson(b, x, rtol=1e-10, precision=pkg.FP64)
        assert st["relres"] <= 1e-10
        xs.append(x)
        op.close()
    assert np.linalg.norm(xs[0] - xs[1]) <= 1e-10 * np.linalg.norm(xs[0])


@pytest.mark.parametrize("order,N,M", [(1, 16, 5), (2, 8, 4)])
def test_gpu_convection_matches_host(built_pkg, order, N, M):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.0, maxm=20)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), order)
    qa = 2 * order - 1 + 2
    host = pkg.assemble_convection(V, C, list(range(1, M + 1)), qa)
    gpu = pkg.assemble_convection_gpu(V, C, list(range(1, M + 1)), qa)
    for m, (A, B) in enumerate(zip(host, gpu)):
        assert abs(A - B).max() <= 1e-13 * abs(A).max(), m
        assert abs(B - B.T).max() > 1e-3 * abs(B).max()   # non-symmetric: the orientation is checked
    lap = pkg.assemble_laplacian_gpu(V)
    assert abs(lap - pkg.assemble_laplacian(V)).max() <= 1e-13 * abs(lap).max()


def test_rhs_argument_errors(built_pkg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.0, maxm=3)
    V = pkg.H1Pk(pkg.unit_square_mesh(4), 1)
    f = lambda x, y: np.ones_like(x)
    with pytest.raises(pkg.SGError):
        pkg.assemble_pce_rhs_gpu(V, C, pkg.total_degree_multiindices(4, 1), f, 2)  # M = 4 > maxm = 3
    with pytest.raises(pkg.SGError):
        pkg.assemble_pce_rhs_gpu(V, C, [[0, 1, 0]], f, 2, factor=0.0)


@pytest.mark.parametrize("qo", [12, 14])
def test_gpu_assembly_with_rules_beyond_16_points(built_pkg, qo):
    """Cell rules of 49 and 64 points (the gather runs the rule in chunks of 16):
    K_m, the convection blocks N_m and b against the oracle's element loops."""
    import __graft_entry__ as ge
    from oracle import coefficient as oc
    from oracle import fem as of
    pkg = ge.load_package()
    assert len(pkg.triangle_rule(qo)[1]) > 16
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.3, maxm=150)
    Co = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.3, maxm=150)
    for order, N in ((1, 8), (2, 6)):
        V = pkg.H1Pk(pkg.unit_square_mesh(N), order)
        Vo = of.LagrangeSpace(of.StructuredMesh(N), order)
        ms = list(range(5))
        gpu = pkg.assemble_stiffness_gpu(V, C, ms, qo)
        ref = of.assemble_stiffness(Vo, Co, ms, qo)
        for m, A, R in zip(ms, gpu, ref):
            assert np.abs((A - R).toarray()).max() <= 1e-13 * np.abs(R.toarray()).max(), (order, m)
        host = pkg.assemble_convection(V, C, [1, 2, 3], qo)
        dev = pkg.assemble_convection_gpu(V, C, [1, 2, 3], qo)
        for A, B in zip(host, dev):
            assert np.abs((A - B).toarray()).max() <= 1e-13 * np.abs(A.toarray()).max()
        bg = pkg.assemble_rhs_gpu(V, lambda x, y: np.ones_like(x) + x * y, qo)
        bo = of.assemble_rhs(Vo, lambda x, y: 1.0 + x * y, qo)
        assert np.abs(bg - bo).max() <= 1e-14 * np.abs(bo).max()
