"""GPU parity of the device-resident PCG (FP64 and mixed precision) against
the oracle's restatement of the reference solve (left-preconditioned GMRES
with the LU mean preconditioner, atol = rtol = 1e-14).

Bar: the solution matches the oracle to within the CG tolerance: relative
2-norm error <= 100 * rtol (the preconditioned operator has condition number
<= ~40 here), and the reported FP64 true residual is <= rtol."""
import numpy as np
import pytest

from oracle import sg as osg
from tests.problems import build, config1_like

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def oracle_solution(p, x0=None):
    n, P = p.n, p.P
    x0 = np.zeros(n * P) if x0 is None else x0
    prec = osg.MeanPreconditioner(p.K0, p.bdofs, P)
    b = osg.reference_rhs(x0, p.b0, p.bdofs, P)
    xg, st = osg.gmres_left(lambda v: osg.apply_fast(v, p.K0, p.Ks, p.G, p.bdofs, P), prec.ldiv, b, x0.copy())
    return xg


@pytest.fixture(scope="module")
def c1(built_pkg):
    p = config1_like()
    op = p.pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    ref = oracle_solution(p)
    yield p, op, ref
    op.close()


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
@pytest.mark.parametrize("rtol", [1e-8, 1e-10])
def test_solve_matches_oracle(c1, precision, rtol):
    p, op, ref = c1
    x = np.zeros(p.n * p.P)
    st = op.solve_primal(p.b0, x, rtol=rtol, precision=getattr(p.pkg, precision))
    assert st["relres"] <= rtol
    assert rel(x, ref) <= 100 * rtol
    mask = osg.interior_mask(p.n, p.P, p.bdofs)
    assert np.all(x[~mask] == 0.0)


def test_mixed_uses_few_fp64_applies(c1):
    p, op, ref = c1
    x = np.zeros(p.n * p.P)
    st = op.solve_primal(p.b0, x, rtol=1e-10, precision=p.pkg.MIXED)
    assert st["outer_iterations"] <= 4 and st["fp64_applies"] <= 5


def test_iteration_count_matches_exact_preconditioner(c1):
    """For P1 the lattice preconditioner is the reference's LU(K_0): FP64 PCG
    needs the same number of iterations as the oracle's PCG with LU."""
    p, op, ref = c1
    n, P = p.n, p.P
    prec = osg.MeanPreconditioner(p.K0, p.bdofs, P)
    b = osg.reference_rhs(np.zeros(n * P), p.b0, p.bdofs, P)
    _, st_o = osg.pcg(lambda v: osg.apply_fast(v, p.K0, p.Ks, p.G, p.bdofs, P), prec.ldiv, b, np.zeros(n * P),
                      osg.interior_mask(n, P, p.bdofs), tol=1e-10)
    x = np.zeros(n * P)
    st = op.solve_primal(p.b0, x, rtol=1e-10, precision=p.pkg.FP64, check_every=1)
    assert abs(st["iterations"] - st_o["niter"]) <= 1


def test_warm_start_reference_rhs(c1):
    """solve_primal! builds b = x0 + e_1 (x) b0 (solvers_poisson_primal.jl:149-150)."""
    p, op, _ = c1
    rng = np.random.default_rng(11)
    x0 = 0.1 * rng.standard_normal(p.n * p.P)
    for mu in range(p.P):
        x0[mu * p.n + p.bdofs] = 0.0
    ref = oracle_solution(p, x0)
    x = x0.copy()
    st = op.solve_primal(p.b0, x, rtol=1e-11, precision=p.pkg.FP64, reference_rhs=True)
    assert rel(x, ref) <= 1e-9
    x = x0.copy()
    op.solve_primal(p.b0, x, rtol=1e-11, precision=p.pkg.FP64, reference_rhs=False)
    assert rel(x, oracle_solution(p)) <= 1e-9


def test_jacobi_and_none_paths(c1):
    p, op, ref = c1
    for kind in (p.pkg.PREC_JACOBI, p.pkg.PREC_NONE):
        x = np.zeros(p.n * p.P)
        st = op.solve_primal(p.b0, x, rtol=1e-9, precision=p.pkg.MIXED, preconditioner=kind)
        assert rel(x, ref) <= 1e-7


def test_maxit_reports_status(c1):
    p, op, _ = c1
    x = np.zeros(p.n * p.P)
    with pytest.raises(p.pkg.SGError) as e:
        op.solve_primal(p.b0, x, rtol=1e-12, precision=p.pkg.FP64, maxit=2)
    assert e.value.code == 6
    st = op.solve_primal(p.b0, x, rtol=1e-12, precision=p.pkg.FP64, maxit=2, allow_maxit=True)
    assert st["iterations"] <= 2 + 8


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_pinned_solution_copy_overlaps_the_last_check(c1, monkeypatch, capfd, precision):
    """sgfem_solve into pinned host memory copies the solution of the step expected
    to end the solve during the final convergence check: the caller gets the same
    bits as through pageable memory (copy after the solve), also with a warm start
    and after a step that did not end the solve (rtol 1e-12 forces a later step)."""
    torch = pytest.importorskip("torch")
    p, op, ref = c1
    prec = getattr(p.pkg, precision)
    monkeypatch.setenv("SGFEM_TRACE", "1")
    rng = np.random.default_rng(5)
    x0 = 0.1 * rng.standard_normal(p.n * p.P)
    for rtol in (1e-10, 1e-12):
        for start in (np.zeros(p.n * p.P), x0):
            xa = start.copy()
            sa = op.solve_primal(p.b0, xa, rtol=rtol, precision=prec)
            capfd.readouterr()
            xp = torch.zeros(p.n * p.P, dtype=torch.float64, pin_memory=True).numpy()
            xp[:] = start
            sp = op.solve_primal(p.b0, xp, rtol=rtol, precision=prec)
            err = capfd.readouterr().err
            assert "solution copy overlapped" in err, err
            assert np.array_equal(xa, xp)
            assert sa["iterations"] == sp["iterations"] and sa["relres"] == sp["relres"] <= rtol
    monkeypatch.setenv("SGFEM_OVERLAP_COPY", "0")
    xq = torch.zeros(p.n * p.P, dtype=torch.float64, pin_memory=True).numpy()
    op.solve_primal(p.b0, xq, rtol=1e-10, precision=prec)
    assert "solution copy overlapped" not in capfd.readouterr().err
    assert rel(xq, ref) <= 1e-8


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_device_loop_body_length(c1, monkeypatch, precision):
    """The PCG runs as a device-side WHILE loop of check_every iterations per
    body: every body length gives the same iterates bit for bit (iterations of a
    body after convergence return at once) and the same iteration count; the cap
    maxit stops the loop at exactly maxit iterations."""
    p, op, ref = c1
    monkeypatch.setenv("SGFEM_SMALL", "0")  # the mixed solve's inner PCG through the device loop
    op_ml = p.pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    prec = getattr(p.pkg, precision)
    xs, sts = [], []
    for ce in (1, 3, 4, 64):
        x = np.zeros(p.n * p.P)
        sts.append(op_ml.solve_primal(p.b0, x, rtol=1e-10, precision=prec, check_every=ce))
        xs.append(x)
    for x, st in zip(xs[1:], sts[1:]):
        assert np.array_equal(x, xs[0])
        assert st["iterations"] == sts[0]["iterations"] and st["relres"] == sts[0]["relres"]
    assert sts[0]["relres"] <= 1e-10 and rel(xs[0], ref) <= 1e-8
    assert sts[-1]["kernel_launches"] > sts[0]["kernel_launches"]  # the early-return iterations count
    # the host-checked replay loop (SGFEM_PCG_LOOP=host) runs the same iterations
    monkeypatch.setenv("SGFEM_PCG_LOOP", "host")
    for ce in (1, 4):
        x = np.zeros(p.n * p.P)
        st = op_ml.solve_primal(p.b0, x, rtol=1e-10, precision=prec, check_every=ce)
        assert np.array_equal(x, xs[0]) and st["iterations"] == sts[0]["iterations"]
    x = np.zeros(p.n * p.P)
    st = op_ml.solve_primal(p.b0, x, rtol=1e-14, precision=p.pkg.FP64, maxit=5, check_every=4, allow_maxit=True)
    assert st["iterations"] == 5
    monkeypatch.delenv("SGFEM_PCG_LOOP")
    for ce in (1, 4, 64):
        x = np.zeros(p.n * p.P)
        st = op_ml.solve_primal(p.b0, x, rtol=1e-14, precision=p.pkg.FP64, maxit=5, check_every=ce,
                                allow_maxit=True)
        assert st["iterations"] == 5, (ce, st)
    op_ml.close()


@pytest.mark.parametrize("order,N,M,P", [(2, 8, 4, 12), (2, 16, 6, 30)])
def test_solve_p2_mixed(built_pkg, order, N, M, P):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    p = build(N, order, M, pkg.top_weight_multiindices(M, P, C.decay_factors))
    ref = oracle_solution(p)
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    assert op.has_lattice
    for prec in (pkg.FP64, pkg.MIXED):
        x = np.zeros(p.n * p.P)
        st = op.solve_primal(p.b0, x, rtol=1e-10, precision=prec)
        assert st["relres"] <= 1e-10
        assert rel(x, ref) <= 1e-8
    op.close()


def test_solve_rhs_lands_on_mode_zero_for_permuted_columns(built_pkg):
    """M=20, P=150 top-weight set (the bench's coupling structure) on a small mesh:
    the device column order differs from the caller's mode order there, and
    e_1 (x) b0 must still land on caller mode 0."""
    import __graft_entry__ as ge
    from oracle import sg as osg
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    p = build(4, 1, 20, pkg.top_weight_multiindices(20, 150, C.decay_factors))
    ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    x = np.zeros(p.n * p.P)
    op.solve_primal(p.b0, x, rtol=1e-12, precision=pkg.FP64, preconditioner=pkg.PREC_JACOBI)
    assert rel(x, ref) <= 1e-9
    op.close()


def test_package_solve_entry_point(built_pkg):
    """solve(PoissonProblemPrimal, sol, C; rhs) writes sol.entries like solve! does."""
    p = config1_like(N=16, M=3, deg=2)
    pkg = p.pkg
    bd = pkg.solve(pkg.PoissonProblemPrimal, p.sol, p.C, rhs=lambda x, y: np.ones_like(x), rtol=1e-11)
    assert np.array_equal(np.sort(bd), p.bdofs)
    assert rel(p.sol.entries, oracle_solution(p)) <= 1e-9
    with pytest.raises(ValueError):
        pkg.solve(pkg.PoissonProblemPrimal, p.sol, p.C, rhs=None)


@pytest.mark.parametrize("order,N", [(1, 32), (2, 16)])
def test_mixed_residual_certificate(built_pkg, monkeypatch, order, N):
    """The mixed solver's refinement residuals are evaluated in double-FP32
    arithmetic (difference form, error-free products and sums); the relres it
    reports equals the FP64 residual of the returned solution, and it agrees
    with the FP64-residual mode (SGFEM_RESIDUAL=fp64)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    p = build(N, order, 6, pkg.top_weight_multiindices(6, 30, C.decay_factors))
    b = osg.reference_rhs(np.zeros(p.n * p.P), p.b0, p.bdofs, p.P)
    out = {}
    for mode in ("default", "fp64"):
        if mode == "fp64":
            monkeypatch.setenv("SGFEM_RESIDUAL", "fp64")
        op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
        for rtol in (1e-8, 1e-11):
            x = np.zeros(p.n * p.P)
            st = op.solve_primal(p.b0, x, rtol=rtol, precision=pkg.MIXED)
            r = b - osg.apply_fast(x, p.K0, p.Ks, p.G, p.bdofs, p.P)
            host = np.linalg.norm(r) / np.linalg.norm(b)
            assert st["relres"] <= rtol and host <= 1.01 * rtol, (mode, rtol, st["relres"], host)
            assert abs(st["relres"] - host) <= 0.02 * host + 1e-14, (mode, rtol, st["relres"], host)
            out[(mode, rtol)] = x
            assert (st["fp64_applies"] == 0) == (mode == "default")
        op.close()
    for rtol in (1e-8, 1e-11):
        assert rel(out[("default", rtol)], out[("fp64", rtol)]) <= 1e3 * rtol

