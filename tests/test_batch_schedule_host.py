"""The column-slot schedule of the batch apply, checked on the host.

sgfem_batch_host_apply schedules one problem as sgfem_batch_finalize does
(virtual groups of 1-16 slots per column block, passes of one kind, the
combination entries grouped by pass) and evaluates the sums of k_bapply_cols
on the host in FP64, so the schedule itself is compared with the oracle's
literal mul! (solvers_poisson_primal.jl:86-124) without a GPU.  Bar: 1e-12
relative in the 2-norm, for the FP32 and the FP64 pass structures."""
import numpy as np
import pytest

from oracle import sg as osg
from tests.problems import build


def _sets(pkg):
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    return [
        (5, 1, 16, pkg.total_degree_multiindices(16, 3)),   # 969 modes: 16 + 1 slots, 1-4 slots
        (6, 1, 7, pkg.total_degree_multiindices(7, 2)),     # 8 slots
        (7, 1, 8, pkg.top_weight_multiindices(8, 40, C.decay_factors)),  # irregular set
        (4, 2, 3, pkg.total_degree_multiindices(3, 2)),     # P2
        (4, 1, 30, pkg.total_degree_multiindices(30, 1)),   # M + 1 = 31, the largest the form takes
        (5, 1, 2, pkg.total_degree_multiindices(2, 1)),     # 3 modes: one partly empty group
    ]


@pytest.mark.parametrize("precision", [1, 0])
def test_column_slot_schedule_matches_oracle(built_pkg, precision):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from extendableasgfem_gb300.batch import host_apply_column_slots
    rng = np.random.default_rng(5)
    for args in _sets(pkg):
        p = build(*args)
        x = rng.standard_normal(p.n * p.P)
        y, summary = host_apply_column_slots(p.Kall, p.TB, p.bdofs, x, precision)
        ref = osg.mul_literal(x, p.K0, p.Ks, p.G, p.bdofs, p.P)
        assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref), (args[:3], summary)
        assert "passes" in summary


def test_column_slot_schedule_padding(built_pkg):
    """On a total-degree set the slots stay close to the pairs (M = 16, degree 3:
    6048 slots for 5593 pairs)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from extendableasgfem_gb300.batch import host_apply_column_slots
    p = build(3, 1, 16, pkg.total_degree_multiindices(16, 3))
    _, summary = host_apply_column_slots(p.Kall, p.TB, p.bdofs, np.zeros(p.n * p.P), 1)
    ratio = float(summary.split(",")[2].split()[0])
    assert ratio <= 1.1, summary


def test_column_slot_schedule_needs_at_most_31_terms(built_pkg):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from extendableasgfem_gb300.batch import host_apply_column_slots
    units = [[0] * 31] + [[int(k == m) for k in range(31)] for m in range(31)]
    p = build(4, 1, 31, units)
    with pytest.raises(pkg.SGError) as e:
        host_apply_column_slots(p.Kall, p.TB, p.bdofs, np.zeros(p.n * p.P), 1)
    assert e.value.code == 7 and "M + 1 <= 31" in str(e.value)


@pytest.mark.parametrize("nl", [2, 3, 4, 16, 17, 64, 100, 127, 128])
def test_split_sine_transform_matches_dense(built_pkg, nl):
    """The batch preconditioner's sine transform, split by output parity (odd outputs
    from x_k + x_{nl-k} and the middle point, even outputs from x_k - x_{nl-k}), equals
    the dense S_ik = sin(pi i k / nl) within its FP32 tables (1e-6 relative), and
    S S = (nl / 2) I."""
    from extendableasgfem_gb300.batch import host_sine_transform
    N = nl - 1
    k = np.arange(1, N + 1)
    S = np.sin(np.pi * np.outer(k, k) / nl)
    x = np.random.default_rng(nl).standard_normal((N, 5))
    y = host_sine_transform(nl, x)
    assert np.linalg.norm(y - S @ x) <= 1e-6 * np.linalg.norm(S @ x)
    z = host_sine_transform(nl, y)
    assert np.linalg.norm(z - 0.5 * nl * x) <= 1e-6 * np.linalg.norm(0.5 * nl * x)


def test_batch_host_helpers(built_pkg):
    """The batch's host helpers: the lattice test (P1 on the unit-square mesh in
    x-fastest order, n = (nl + 1)^2, 2 <= nl <= 128; not P2, not a perturbed mesh)
    and the values of every K_m on K_0's pattern (refused when a K_m has an entry
    outside it)."""
    import scipy.sparse as sp
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from extendableasgfem_gb300.batch import _lattice_size, _shared_pattern_values
    assert _lattice_size(pkg.H1Pk(pkg.unit_square_mesh(16), 1)) == 16
    assert _lattice_size(pkg.H1Pk(pkg.unit_square_mesh(16), 2)) == 0
    assert _lattice_size(pkg.H1Pk(pkg.perturbed_unit_square_mesh(8, 0.2), 1)) == 0
    p = build(6, 1, 3, pkg.total_degree_multiindices(3, 1))
    K0, vals = _shared_pattern_values(p.Kall)
    assert vals.shape == (len(p.Kall), K0.nnz)
    for m, K in enumerate(p.Kall):
        Km = sp.csc_matrix((vals[m], K0.indices, K0.indptr), shape=K0.shape)
        assert abs(Km - K).max() == 0.0
    extra = p.Kall[1].tolil()
    extra[0, p.n - 1] = 1.0
    with pytest.raises(ValueError):
        _shared_pattern_values([p.Kall[0], extra.tocsc()])
