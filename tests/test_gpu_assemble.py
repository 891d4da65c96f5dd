"""GPU assembly of the stiffness matrices K_m of the cosine coefficient
(sgfem_assemble_stiffness) against the host assembly (the caller-side
restatement of ExtendableFEM's BilinearOperator assembly, poisson_primal.jl:
56-68): same pattern, values within 1e-13 of the largest entry, bitwise
reproducible, and a solve on GPU-assembled blocks matches one on host blocks."""
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
    assert np.array_equal(b0, b0g)
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
