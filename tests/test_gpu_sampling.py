"""GPU sampling pieces against the oracle (src/sampling_error.jl,
src/sgfevector.jl:43-69): batched deterministic sample solves (each sample to
the requested tolerance), evaluation of the SG solution at samples, and the
sampling error integrals."""
import numpy as np
import pytest

from oracle import sampling as osm

pytestmark = pytest.mark.gpu


def det_setup(N=16, order=2, M=20, S=40, seed=3):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), order)
    Ks = pkg.assemble_stiffness(V, C, list(range(M + 1)), 2 * (order - 1) + 2)
    b0 = pkg.assemble_rhs(V, lambda x, y: np.ones_like(x), order)
    y = np.random.default_rng(seed).uniform(-1, 1, size=(M, S))
    return pkg, C, V, Ks, b0, y


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_sample_solves_match_direct(built_pkg, precision):
    pkg, C, V, Ks, b0, y = det_setup()
    sp_ = pkg.SampleProblems(V, Ks, y)
    assert sp_.ctx.has_lattice
    U = sp_.solve(b0, rtol=1e-10, precision=getattr(pkg, precision))
    assert sp_.stats["relres"] <= 1e-10
    for s in range(y.shape[1]):
        ref = osm.deterministic_solve(Ks, b0, V.bdofs, y[:, s])
        assert np.linalg.norm(U[:, s] - ref) <= 1e-8 * np.linalg.norm(ref)
    sp_.close()


def test_sample_operator_forms_agree(built_pkg, monkeypatch):
    """The sample operators K(y_s) combined in double-FP32 and applied four samples per
    lane (default) against the exactly rounded FP64 combination applied one sample per
    lane (SGFEM_SAMPLES_COMBINE=fp64, SGFEM_SAMPLES_VEC=0): the same solutions to 1e-9
    in both precisions, all within 1e-8 of the oracle's direct solves (an operator off
    at FP32 level, 1e-7, would miss both bars)."""
    pkg, C, V, Ks, b0, y = det_setup(N=16, order=2, M=20, S=40)
    res = {}
    for comb, vec in (("df", "1"), ("fp64", "0")):
        monkeypatch.setenv("SGFEM_SAMPLES_COMBINE", comb)
        monkeypatch.setenv("SGFEM_SAMPLES_VEC", vec)
        for prec in ("FP64", "MIXED"):
            sp_ = pkg.SampleProblems(V, Ks, y)
            res[comb, prec] = sp_.solve(b0, rtol=1e-12, precision=getattr(pkg, prec))
            sp_.close()
    for prec in ("FP64", "MIXED"):
        a, b = res["df", prec], res["fp64", prec]
        assert np.linalg.norm(a - b) <= 1e-9 * np.linalg.norm(b), prec
    for s in (0, 39):
        ref = osm.deterministic_solve(Ks, b0, V.bdofs, y[:, s])
        for key, U in res.items():
            assert np.linalg.norm(U[:, s] - ref) <= 1e-8 * np.linalg.norm(ref), key


def test_sample_solves_p1_odd_count(built_pkg):
    pkg, C, V, Ks, b0, y = det_setup(N=32, order=1, M=5, S=37)
    sp_ = pkg.SampleProblems(V, Ks, y)
    U = sp_.solve(b0, rtol=1e-9)
    for s in (0, 17, 36):
        ref = osm.deterministic_solve(Ks, b0, V.bdofs, y[:, s])
        assert np.linalg.norm(U[:, s] - ref) <= 1e-7 * np.linalg.norm(ref)
    sp_.close()


# ---- evaluation at samples and the sampling error -------------------------

from oracle import basis as ob  # noqa: E402
from oracle import coefficient as oc  # noqa: E402
from oracle import fem as of  # noqa: E402
from tests.problems import build  # noqa: E402

def sg_case(N=8, M=3, deg=2, basis="legendre", solve=True):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    p = build(N, 1, M, pkg.total_degree_multiindices(M, deg), basis=basis)
    if solve:
        op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
        op.solve_primal(p.b0, p.sol.entries, rtol=1e-12, precision=pkg.FP64)
        op.close()
    else:
        p.sol.entries[:] = np.random.default_rng(11).standard_normal(len(p.sol.entries))
    obt = ob.LEGENDRE if basis == "legendre" else ob.HERMITE
    maxdeg = max(max(mi) for mi in p.mis)
    TBo = ob.TensorizedBasis(obt, M, maxdeg, maxdeg + 4, multi_indices=p.mis)
    return pkg, p, TBo


@pytest.mark.parametrize("basis", ["legendre", "hermite"])
def test_evaluate_samples_matches_oracle(built_pkg, basis):
    pkg, p, TBo = sg_case(M=4, deg=3, basis=basis, solve=False)
    rng = np.random.default_rng(12)
    Ms, S = 6, 37
    y = rng.uniform(-1, 1, (Ms, S)) if basis == "legendre" else rng.standard_normal((Ms, S))
    for m in (0, 1, 3, 4, 6):
        out = pkg.evaluate_samples(p.sol, y, m=m)
        assert out.shape == (p.n, S)
        mm = min(m, p.M)  # dimensions beyond the multi-index length do not enter
        ref = np.stack([osm.sg_evaluate(p.sol.entries, p.n, TBo, y[:mm, s]) for s in range(S)], axis=1)
        assert np.max(np.abs(out - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("basis", ["legendre", "hermite"])
def test_set_sample_on_the_gpu_matches_oracle(built_pkg, basis):
    """SGFEVector.set_sample (set_sample!, sgfevector.jl:43-69) evaluates on the
    GPU: FEV against the oracle for samples shorter than, equal to and longer than
    the multi-index length (and empty), and the stored sample."""
    pkg, p, TBo = sg_case(M=4, deg=3, basis=basis, solve=False)
    rng = np.random.default_rng(21)
    for L in (0, 2, 4, 7):
        S = rng.uniform(-1, 1, L) if basis == "legendre" else rng.standard_normal(L)
        fev = p.sol.set_sample(S).copy()
        ref = osm.sg_evaluate(p.sol.entries, p.n, TBo, S[:p.M])
        assert np.max(np.abs(fev - ref)) <= 1e-13 * np.max(np.abs(ref)), L
        assert np.array_equal(p.sol.last_sample[:min(L, p.M)], S[:min(L, p.M)])
        assert not np.any(p.sol.last_sample[min(L, p.M):])


def det_oracle(p, Ms, order=2, bonus_a=10):
    N = int(round(np.sqrt(p.V.mesh.ncells / 2)))
    mesh = of.StructuredMesh(N)
    Vo_sg = of.LagrangeSpace(mesh, 1)
    Vo_det = of.LagrangeSpace(mesh, order)
    Co = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=p.C.mean_value, maxm=p.C.maxm())
    Kdo = of.assemble_stiffness(Vo_det, Co, list(range(Ms + 1)), 2 * (order - 1) + bonus_a)
    bdo = of.assemble_rhs(Vo_det, lambda x, y: 1.0 + 0 * x, order)
    return Vo_sg, Vo_det, Kdo, bdo


def test_sampling_error_integrals_match_oracle(built_pkg):
    """Error integrals for every truncation m, deterministic solutions given."""
    pkg, p, TBo = sg_case(M=3, deg=2)
    Ms, S = 5, 19
    y = np.random.default_rng(13).uniform(-1, 1, (Ms, S))
    Vo_sg, Vo_det, Kdo, bdo = det_oracle(p, Ms)
    D = np.stack([osm.deterministic_solve(Kdo, bdo, Vo_det.bdofs, y[:, s]) for s in range(S)], axis=1)
    Vd = pkg.H1Pk(p.V.mesh, 2)
    Kd = pkg.assemble_stiffness(Vd, p.C, list(range(Ms + 1)), 12)
    sp_ = pkg.SampleProblems(Vd, Kd, y)
    eh, el = sp_.sampling_error(p.sol, 4, det_solutions=D)
    sp_.close()
    assert eh.shape == (p.M + 1, S)
    for s in range(S):
        for m in range(p.M + 1):
            us = osm.sg_evaluate(p.sol.entries, p.n, TBo, y[:m, s])
            h1, l2 = osm.error_integrals(Vo_det, D[:, s], Vo_sg, us, 4)
            assert abs(eh[m, s] - h1) <= 1e-11 * h1
            assert abs(el[m, s] - l2) <= 1e-11 * l2


@pytest.mark.parametrize("sg_order,det_order", [(1, 2), (2, 2), (1, 1), (2, 1)])
def test_sampling_error_forms_match_oracle(built_pkg, monkeypatch, sg_order, det_order):
    """The error sums as quadratic forms in the error's local coefficients (the SG
    space embeds in the deterministic one: P1 in P2, equal orders) and point by point
    (no embedding, or SGFEM_SAMPLING_QF=0): both against the oracle's point-by-point
    sums (1e-11 per (m, s)) and against each other (1e-12), for the 3- and 9-point rules
    of orders 2 and 4."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    M, N, Ms, S = 3, 8, 5, 37
    p = build(N, sg_order, M, pkg.total_degree_multiindices(M, 2))
    rng = np.random.default_rng(21)
    p.sol.entries[:] = rng.standard_normal(len(p.sol.entries))
    maxdeg = max(max(mi) for mi in p.mis)
    TBo = ob.TensorizedBasis(ob.LEGENDRE, M, maxdeg, maxdeg + 4, multi_indices=p.mis)
    y = rng.uniform(-1, 1, (Ms, S))
    Vd = pkg.H1Pk(p.V.mesh, det_order)
    Kd = pkg.assemble_stiffness(Vd, p.C, list(range(Ms + 1)), 6)
    D = rng.standard_normal((Vd.ndofs, S))
    mesh = of.StructuredMesh(N)
    Vo_det, Vo_sg = of.LagrangeSpace(mesh, det_order), of.LagrangeSpace(mesh, sg_order)
    embeds = sg_order <= det_order
    sp_ = pkg.SampleProblems(Vd, Kd, y)
    for quadorder in (2, 4):
        res = {}
        for qf in ("1", "0"):
            monkeypatch.setenv("SGFEM_SAMPLING_QF", qf)
            res[qf] = sp_.sampling_error(p.sol, quadorder, det_solutions=D)
            want = "quadratic forms" if (qf == "1" and embeds) else "quadrature points"
            assert sp_.ctx.sampling_error_log == want, sp_.ctx.sampling_error_log
        for k in range(2):
            a, b = res["1"][k], res["0"][k]
            assert np.max(np.abs(a - b) / np.abs(b)) <= 1e-12
        eh, el = res["1"]
        for s in (0, 13, 36):
            for m in range(M + 1):
                us = osm.sg_evaluate(p.sol.entries, p.n, TBo, y[:m, s])
                h1, l2 = osm.error_integrals(Vo_det, D[:, s], Vo_sg, us, quadorder)
                assert abs(eh[m, s] - h1) <= 1e-11 * h1
                assert abs(el[m, s] - l2) <= 1e-11 * l2
    sp_.close()


def test_calculate_sampling_error_matches_oracle(built_pkg):
    """The whole driver: batched device solves (3 batches, last one padded) and
    the weighted / uniform means against the oracle's direct solves."""
    pkg, p, TBo = sg_case(M=3, deg=2)
    Ms, S = 5, 21
    y = np.random.default_rng(14).uniform(-1, 1, (Ms, S))
    w = np.prod(np.where(np.abs(y) <= 1, 0.5, 0.0), axis=0) * np.linspace(0.5, 1.5, S)
    f = lambda x, y_: np.ones_like(x)
    got, (eh, el) = pkg.calculate_sampling_error(p.sol, p.C, order=2, rhs=f, Msamples=Ms, samples=y, weights=w,
                                                 batch=8, rtol=1e-12, return_per_sample=True)
    Vo_sg, Vo_det, Kdo, bdo = det_oracle(p, Ms)
    ref = osm.calculate_sampling_error(p.sol.entries, TBo, Vo_sg, Vo_det, Kdo, bdo, y, w, order=2)
    for g, r in zip(got, ref):
        assert np.max(np.abs(g - r) / r) <= 1e-8
    assert np.all(np.diff(got[2]) < 0)  # error decreases with the truncation length here
    got2 = pkg.calculate_sampling_error(p.sol, p.C, order=2, rhs=f, Msamples=Ms, samples=y, weights=w, batch=32,
                                        rtol=1e-12, dimensionwise_error=False)
    assert np.all(got2[0][:-1] == 0.0) and abs(got2[0][-1] - got[0][-1]) <= 1e-9 * got[0][-1]


def test_sampling_error_needs_solutions(built_pkg):
    pkg, p, TBo = sg_case(M=2, deg=1, solve=False)
    Vd = pkg.H1Pk(p.V.mesh, 2)
    Kd = pkg.assemble_stiffness(Vd, p.C, [0, 1, 2], 4)
    sp_ = pkg.SampleProblems(Vd, Kd, np.zeros((2, 4)))
    with pytest.raises(pkg.SGError):
        sp_.sampling_error(p.sol, 4)
    with pytest.raises(pkg.SGError):
        sp_.ctx.set_samples(np.zeros((2, 5)))
    sp_.close()
