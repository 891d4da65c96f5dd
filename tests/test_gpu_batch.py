"""Batched SG solves (sgfem_batch_*): every problem of a batch with uneven
mesh sizes, coefficient lengths and multi-index sets against the oracle's
assembled Kronecker solve (solve_full_primal!, solvers_poisson_primal.jl:
172-230).  Bar: rtol 1e-10 on the FP64 true residual, solutions within 1e-8."""
import numpy as np
import pytest

from oracle import sg as osg
from tests.problems import build

pytestmark = pytest.mark.gpu


def test_batch_matches_kronecker_solves(built_pkg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    shapes = [(5, 2, 2), (7, 3, 1), (6, 4, 3), (4, 2, 1), (9, 3, 2), (8, 1, 3), (5, 5, 2), (6, 3, 3)]
    probs = [build(N, 1, M, pkg.total_degree_multiindices(M, d)) for N, M, d in shapes]
    probs.append(build(4, 2, 3, pkg.total_degree_multiindices(3, 2)))  # one P2 problem
    B = pkg.SGBatch(0)
    for p in probs:
        B.add(p.V, p.TB, p.Kall, p.b0)
    B.finalize()
    assert "chosen" in B.tuning
    xs, st = B.solve(rtol=1e-10, check_every=8)
    assert st["converged"] == len(probs)
    assert st["relres_max"] <= 1e-10
    for i, (p, x) in enumerate(zip(probs, xs)):
        ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
        assert np.linalg.norm(x - ref) <= 1e-8 * np.linalg.norm(ref), i
        it, rr = B.problem_stats(i)
        assert it > 0 and rr <= 1e-10
    B.close()


def test_batch_equals_single_problem_solver(built_pkg):
    """A problem solved inside a batch gives the single-problem solver's answer."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    p = build(16, 1, 4, pkg.total_degree_multiindices(4, 2))
    q = build(12, 1, 3, pkg.total_degree_multiindices(3, 3))
    B = pkg.SGBatch(0)
    B.add(p.V, p.TB, p.Kall, p.b0)
    B.add(q.V, q.TB, q.Kall, q.b0)
    B.finalize()
    xs, st = B.solve(rtol=1e-11)
    for prob, x in ((p, xs[0]), (q, xs[1])):
        op = pkg.SGOperator(prob.V, prob.TB, prob.Kall, device=0)
        y = np.zeros(prob.n * prob.P)
        op.solve_primal(prob.b0, y, rtol=1e-11, precision=pkg.FP64, reference_rhs=False)
        op.close()
        assert np.linalg.norm(x - y) <= 1e-8 * np.linalg.norm(y)
    B.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_precisions_agree(built_pkg, monkeypatch, precision):
    """The default mixed solve (FP32 inner PCG, FP64 residuals and solution) and
    the plain FP64 PCG (SGFEM_BATCH_PRECISION=fp64) both meet rtol on the FP64
    residual and agree with the single-problem FP64 solve."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    if precision == "fp64":
        monkeypatch.setenv("SGFEM_BATCH_PRECISION", "fp64")
    probs = [build(16, 1, 4, pkg.total_degree_multiindices(4, 2)), build(8, 2, 3, pkg.total_degree_multiindices(3, 2)),
             build(11, 1, 5, pkg.total_degree_multiindices(5, 1))]
    B = pkg.SGBatch(0)
    for p in probs:
        B.add(p.V, p.TB, p.Kall, p.b0)
    B.finalize()
    xs, st = B.solve(rtol=1e-9)
    assert st["converged"] == len(probs) and st["relres_max"] <= 1e-9
    for p, x in zip(probs, xs):
        ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
        assert np.linalg.norm(x - ref) <= 1e-7 * np.linalg.norm(ref)
    B.close()


def test_batch_many_kle_terms(built_pkg):
    """A problem with 41 KLE terms (every K_m coupled through the mean mode) next
    to a small one: all M + 1 values of a nonzero reach the batch apply."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    units = [[0] * 40] + [[int(k == m) for k in range(40)] for m in range(40)]
    probs = [build(6, 1, 40, units), build(5, 1, 2, pkg.total_degree_multiindices(2, 2))]
    B = pkg.SGBatch(0)
    for p in probs:
        B.add(p.V, p.TB, p.Kall, p.b0)
    B.finalize()
    xs, st = B.solve(rtol=1e-10)
    assert st["converged"] == len(probs) and st["relres_max"] <= 1e-10
    for p, x in zip(probs, xs):
        ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
        assert np.linalg.norm(x - ref) <= 1e-8 * np.linalg.norm(ref)
    B.close()


def test_batch_tuning_cache(built_pkg, monkeypatch, tmp_path):
    """The launch shapes tuned at finalize go to the on-disk cache; a batch of
    the same shapes finalized again takes them from there (no timing sweep) and
    solves to the same answer."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    cache = tmp_path / "tuning.txt"
    monkeypatch.setenv("SGFEM_TUNE_CACHE", str(cache))
    probs = [build(12, 1, 3, pkg.total_degree_multiindices(3, 2)), build(6, 1, 2, pkg.total_degree_multiindices(2, 3))]
    out = []
    for attempt in range(2):
        B = pkg.SGBatch(0)
        for p in probs:
            B.add(p.V, p.TB, p.Kall, p.b0)
        B.finalize()
        assert ("from the tuning cache" in B.tuning) == (attempt == 1), B.tuning
        xs, st = B.solve(rtol=1e-10)
        assert st["converged"] == len(probs) and st["relres_max"] <= 1e-10
        out.append(xs)
        B.close()
    assert cache.exists() and len(cache.read_text().splitlines()) == 1
    for a, b in zip(*out):
        assert np.linalg.norm(a - b) <= 1e-9 * np.linalg.norm(b)


def test_batch_work_queue_apply_is_bitwise_the_block_map(built_pkg, monkeypatch, tmp_path):
    """The FP32 apply over the persistent work queue (SGFEM_BATCH_QUEUE=1: resident
    blocks take the block map's items in descending-cost order) computes every item
    as the one-block-per-item launch does and leaves each partial in the same
    slot, so the mixed solves are bitwise equal and meet rtol.  The two batches share
    one tuning cache: the second takes the first's timed shapes (forms, warps, block
    map), so only the queue bit differs between them."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    shapes = [(9, 3, 2), (5, 2, 2), (12, 4, 2), (6, 5, 1), (7, 2, 3), (16, 3, 2)]
    probs = [build(N, 1, M, pkg.total_degree_multiindices(M, d)) for N, M, d in shapes]
    monkeypatch.setenv("SGFEM_TUNE_CACHE", str(tmp_path / "tuning.txt"))
    out = {}
    for q in ("0", "1"):
        monkeypatch.setenv("SGFEM_BATCH_QUEUE", q)
        B = pkg.SGBatch(0)
        for p in probs:
            B.add(p.V, p.TB, p.Kall, p.b0)
        B.finalize()
        assert ("work queue" in B.tuning.split(";")[0]) == (q == "1"), B.tuning
        xs, st = B.solve(rtol=1e-10, check_every=8)
        assert st["converged"] == len(probs) and st["relres_max"] <= 1e-10
        out[q] = xs
        B.close()
    for a, b in zip(out["0"], out["1"]):
        assert np.array_equal(a, b)
    for p, x in zip(probs, out["1"]):
        ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
        assert np.linalg.norm(x - ref) <= 1e-8 * np.linalg.norm(ref)


def _solve_batch(pkg, probs, rtol, check_every=8):
    B = pkg.SGBatch(0)
    for p in probs:
        B.add(p.V, p.TB, p.Kall, p.b0)
    B.finalize()
    xs, st = B.solve(rtol=rtol, check_every=check_every)
    tuning = B.tuning
    B.close()
    return xs, st, tuning


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_column_slot_apply_matches_kronecker_solves(built_pkg, monkeypatch, precision):
    """The column-slot form of the batch apply (SGFEM_BATCH_APPLY=cols: lanes own
    columns, each slot takes its KLE value from the lane holding it) in both
    precisions: total-degree sets (M = 16 and degree 2: groups of 16 and 1 slots for
    the low-degree columns, 4 for the others; M = 7: 8 slots; degree 3), an
    irregular top-weight set, a P2 problem and M + 1 = 31 (the largest the form
    takes) against the Kronecker solves."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    monkeypatch.setenv("SGFEM_BATCH_APPLY", "cols")
    monkeypatch.setenv("SGFEM_TUNE_CACHE", "off")
    if precision == "fp64":
        monkeypatch.setenv("SGFEM_BATCH_PRECISION", "fp64")
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    probs = [build(5, 1, 16, pkg.total_degree_multiindices(16, 2)),
             build(6, 1, 7, pkg.total_degree_multiindices(7, 2)),
             build(9, 1, 5, pkg.total_degree_multiindices(5, 3)),
             build(7, 1, 8, pkg.top_weight_multiindices(8, 40, C.decay_factors)),
             build(4, 2, 3, pkg.total_degree_multiindices(3, 2)),
             build(4, 1, 30, pkg.total_degree_multiindices(30, 1)),
             build(6, 1, 2, pkg.total_degree_multiindices(2, 1))]
    xs, st, tuning = _solve_batch(pkg, probs, 1e-10)
    head = tuning.split(";")[0]
    assert "chosen column slots" in head and "FP32: column slots" in head, tuning
    assert st["converged"] == len(probs) and st["relres_max"] <= 1e-10
    for p, x in zip(probs, xs):
        ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
        assert np.linalg.norm(x - ref) <= 1e-8 * np.linalg.norm(ref)


def test_batch_column_slot_queue_is_bitwise_the_block_map(built_pkg, monkeypatch, tmp_path):
    """The column-slot FP32 apply over the persistent work queue computes every
    item as the one-block-per-item launch does: bitwise equal mixed solves (one
    shared tuning cache, so only the queue bit differs between the two batches)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    monkeypatch.setenv("SGFEM_BATCH_APPLY", "cols")
    monkeypatch.setenv("SGFEM_TUNE_CACHE", str(tmp_path / "tuning.txt"))
    shapes = [(9, 3, 2), (5, 2, 2), (12, 4, 3), (6, 5, 1), (7, 12, 2)]
    probs = [build(N, 1, M, pkg.total_degree_multiindices(M, d)) for N, M, d in shapes]
    out = {}
    for q in ("0", "1"):
        monkeypatch.setenv("SGFEM_BATCH_QUEUE", q)
        xs, st, tuning = _solve_batch(pkg, probs, 1e-10)
        head = tuning.split(";")[0]
        assert "column slots" in head and ("work queue" in head) == (q == "1"), tuning
        assert st["converged"] == len(probs) and st["relres_max"] <= 1e-10
        out[q] = xs
    for a, b in zip(out["0"], out["1"]):
        assert np.array_equal(a, b)


def test_batch_column_slots_need_at_most_31_terms(built_pkg, monkeypatch):
    """A problem with M + 1 > 31 keeps the whole batch on the pair form even when
    the column-slot form is asked for (lane 31 must hold the zero value)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    monkeypatch.setenv("SGFEM_BATCH_APPLY", "cols")
    monkeypatch.setenv("SGFEM_TUNE_CACHE", "off")
    units = [[0] * 31] + [[int(k == m) for k in range(31)] for m in range(31)]
    probs = [build(5, 1, 31, units), build(5, 1, 2, pkg.total_degree_multiindices(2, 2))]
    xs, st, tuning = _solve_batch(pkg, probs, 1e-10)
    assert "column slots" not in tuning.split(";")[0], tuning
    assert st["converged"] == len(probs)
    for p, x in zip(probs, xs):
        ref = osg.kron_direct(p.K0, p.Ks, p.G, p.b0, p.bdofs, p.P)
        assert np.linalg.norm(x - ref) <= 1e-8 * np.linalg.norm(ref)
