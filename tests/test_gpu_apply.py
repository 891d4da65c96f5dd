"""GPU parity of the SG operator apply (K1) and the mean-based preconditioner
(K2) against the oracle, through the C ABI.

Tolerances: FP64 apply 1e-12 relative in the 2-norm (the bar for the plain
FP64 operator); FP32 apply 1e-5 relative to the FP64 result; lattice
preconditioner 1e-10 against the oracle's LU solve (P1, where the two
operators are identical) or against a direct solve with the lattice
Laplacian (P2)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import sg as osg
from tests.problems import build, config1_like

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def problems():
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    return {
        "config1": lambda: config1_like(),
        "p2_top_weight": lambda: build(16, 2, 6, pkg.top_weight_multiindices(6, 30, C.decay_factors)),
        "hermite_full": lambda: build(8, 1, 3, pkg.generate_multiindices(3, 2), basis="hermite", mean=2.0),
        "p1_odd_mesh": lambda: build(12, 1, 4, pkg.total_degree_multiindices(4, 2)),
        "single_mode": lambda: build(8, 1, 2, [[0, 0]]),
        # 41 KLE terms: every K_m reaches the apply (the mean mode couples to each e_m)
        "many_terms": lambda: build(6, 1, 40, [[0] * 40] + [[int(k == m) for k in range(40)] for m in range(40)]),
    }


@pytest.fixture(scope="module", params=list(problems().keys()))
def case(request, built_pkg):
    p = problems()[request.param]()
    op = p.pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    yield p, op
    op.close()


def test_apply_fp64_matches_oracle(case):
    p, op = case
    x = np.random.default_rng(0).standard_normal(p.n * p.P)
    y = op.mul(x, p.pkg.FP64)
    yref = osg.mul_literal(x, p.K0, p.Ks, p.G, p.bdofs, p.P)
    assert rel(y, yref) <= 1e-12
    n = p.n
    for mu in range(p.P):
        assert np.all(y[mu * n + p.bdofs] == 0.0)


def test_apply_fp32_error(case):
    p, op = case
    x = np.random.default_rng(1).standard_normal(p.n * p.P)
    y64 = op.mul(x, p.pkg.FP64)
    y32 = op.mul(x, p.pkg.FP32)
    assert rel(y32, y64) <= 1e-5


def test_apply_deterministic(case):
    p, op = case
    x = np.random.default_rng(2).standard_normal(p.n * p.P)
    assert np.array_equal(op.mul(x, p.pkg.FP64), op.mul(x, p.pkg.FP64))


def test_apply_linearity(case):
    p, op = case
    rng = np.random.default_rng(3)
    x, z = rng.standard_normal((2, p.n * p.P))
    lhs = op.mul(2.0 * x - 0.5 * z)
    rhs = 2.0 * op.mul(x) - 0.5 * op.mul(z)
    assert rel(lhs, rhs) <= 1e-13


def test_preconditioner(case):
    p, op = case
    pkg = p.pkg
    rng = np.random.default_rng(4)
    b = rng.standard_normal(p.n * p.P)
    for mu in range(p.P):
        b[mu * p.n + p.bdofs] = 0.0
    inner = np.setdiff1d(np.arange(p.n), p.bdofs)
    # the reference's preconditioner: LU(K_0) on interior rows, every mode
    ref = osg.MeanPreconditioner(p.K0, p.bdofs, p.P).ldiv(b)
    if op.has_lattice:
        assert "exact" in op.ctx.lattice_log, op.ctx.lattice_log
        y = op.ldiv(b, pkg.PREC_LATTICE, pkg.FP64)
        mask = osg.interior_mask(p.n, p.P, p.bdofs)
        assert rel(y[mask], ref[mask]) <= 1e-10
        assert np.all(y[~mask] == 0.0)
        y32 = op.ldiv(b, pkg.PREC_LATTICE, pkg.FP32)
        assert rel(y32[mask], ref[mask]) <= 1e-4
    yj = op.ldiv(b, pkg.PREC_JACOBI, pkg.FP64)
    dj = np.zeros(p.n)
    dj[inner] = 1.0 / p.K0.diagonal()[inner]
    assert rel(yj, b * np.tile(dj, p.P)) <= 1e-14


def lattice_laplacian_solve(p, b):
    """(a0 L)^-1 on interior rows, L the 5-point Laplacian of the dof lattice, a0 the
    mean interior diagonal of K_0 over 4."""
    Nl = int(round(np.sqrt(p.n))) - 1
    ij = np.rint(p.V.dof_coords * Nl).astype(int)
    pos = {(a, c): k for k, (a, c) in enumerate(ij)}
    rows, cols, vals = [], [], []
    for k, (a, c) in enumerate(ij):
        rows.append(k); cols.append(k); vals.append(4.0)
        for da, dc in ((1, 0), (-1, 0), (0, 1), (0, -1)):
            j = pos.get((a + da, c + dc))
            if j is not None:
                rows.append(k); cols.append(j); vals.append(-1.0)
    L = sp.csr_matrix((vals, (rows, cols)), shape=(p.n, p.n))
    inner = np.setdiff1d(np.arange(p.n), p.bdofs)
    a0 = p.K0.diagonal()[inner].sum() / (4 * len(inner))
    lu = spla.splu((a0 * L[inner][:, inner]).tocsc())
    ref = np.zeros_like(b)
    for mu in range(p.P):
        ref[mu * p.n + inner] = lu.solve(b[mu * p.n + inner])
    return ref


@pytest.mark.parametrize("order", [1, 2])
def test_laplacian_lattice_preconditioner(built_pkg, monkeypatch, order):
    """With the block form switched off (or K_0 not translation invariant) the
    lattice preconditioner is (a0 L)^-1 with the 5-point Laplacian."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    p = build(16, order, 3, pkg.total_degree_multiindices(3, 2))
    monkeypatch.setenv("SGFEM_LAT_BLOCK", "0")
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    assert op.has_lattice and "Laplacian" in op.ctx.lattice_log
    b = np.random.default_rng(5).standard_normal(p.n * p.P)
    for mu in range(p.P):
        b[mu * p.n + p.bdofs] = 0.0
    ref = lattice_laplacian_solve(p, b)
    mask = osg.interior_mask(p.n, p.P, p.bdofs)
    for prec, tol in ((pkg.FP64, 1e-10), (pkg.FP32, 1e-4)):
        y = op.ldiv(b, pkg.PREC_LATTICE, prec)
        assert rel(y[mask], ref[mask]) <= tol
    op.close()


def test_block_preconditioner_needs_translation_invariance(built_pkg):
    """A mean coefficient that varies in space makes K_0 non-invariant: the
    Laplacian form is used and the log says why."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    p = build(16, 1, 2, pkg.total_degree_multiindices(2, 1))
    K0 = p.Kall[0].tolil()
    n1 = int(round(np.sqrt(p.n)))
    r = (n1 // 2) * n1 + n1 // 2  # one interior row scaled: no longer a repeating stencil
    K0[r, :] = K0[r, :] * 1.5
    Kall = [K0.tocsc()] + list(p.Kall[1:])
    op = pkg.SGOperator(p.V, p.TB, Kall, device=0)
    assert op.has_lattice and "not translation invariant" in op.ctx.lattice_log, op.ctx.lattice_log
    op.close()


def test_lattice_detection(case):
    p, op = case
    Nl = int(round(np.sqrt(p.n))) - 1
    expect = (Nl & (Nl - 1)) == 0
    assert op.has_lattice == expect


def test_apply_non_lattice_numbering(built_pkg):
    """A shuffled dof numbering without coordinates takes the generic path."""
    p = config1_like(N=8, M=3, deg=2)
    rng = np.random.default_rng(7)
    perm = rng.permutation(p.n)
    inv = np.argsort(perm)
    Kp = [K[perm][:, perm] for K in p.Kall]
    ctx = p.pkg._lib.Context(0)
    for m, K in enumerate(Kp):
        ctx.set_spatial_matrix(m, K)
    ctx.set_coupling(p.TB.G, p.P, p.M)
    ctx.set_boundary_dofs(inv[p.bdofs])
    ctx.finalize()
    assert not ctx.has_lattice
    x = rng.standard_normal(p.n * p.P)
    X = x.reshape(p.P, p.n)
    y = ctx.apply(X[:, perm].ravel())
    yref = osg.mul_literal(x, p.K0, p.Ks, p.G, p.bdofs, p.P).reshape(p.P, p.n)[:, perm].ravel()
    assert rel(y, yref) <= 1e-12
    ctx.close()


def test_specialised_fp32_apply_active_and_matches_generic(built_pkg, monkeypatch):
    """The FP32 apply compiled for the coupling structure (NVRTC) is the one in
    use, and it agrees with the generic kernel and with FP64."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    for p in (config1_like(), build(16, 2, 8, pkg.top_weight_multiindices(8, 60, C.decay_factors))):
        op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
        variant, log = op.ctx.apply_variant
        assert variant == 1, log
        monkeypatch.setenv("SGFEM_APPLY", "generic")
        opg = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
        monkeypatch.delenv("SGFEM_APPLY")
        assert opg.ctx.apply_variant[0] == 0
        x = np.random.default_rng(9).standard_normal(p.n * p.P)
        y64 = op.mul(x, pkg.FP64)
        ys = op.mul(x, pkg.FP32)
        yg = opg.mul(x, pkg.FP32)
        assert rel(ys, y64) <= 1e-5 and rel(yg, y64) <= 1e-5
        assert rel(ys, yg) <= 1e-5
        op.close()
        opg.close()



KNOBS = [
    {},
    {"SGFEM_JIT_DIFF": "0"},
    {"SGFEM_JIT_SPLIT": "1"},
    {"SGFEM_JIT_SPLIT": "1", "SGFEM_JIT_DIFF": "0"},
    {"SGFEM_JIT_SPLIT": "1", "SGFEM_JIT_WWPB": "8", "SGFEM_JIT_WRW": "2"},
    {"SGFEM_JIT_SPLIT": "1", "SGFEM_JIT_WWPB": "16", "SGFEM_JIT_WRW": "1"},
    {"SGFEM_JIT_WWPB": "4", "SGFEM_JIT_WRW": "3"},
    {"SGFEM_JIT_WRW": "1"},
    {"SGFEM_JIT_UNROLL": "2"},
    {"SGFEM_JIT_UNROLL": "4"},
    {"SGFEM_JIT_WINDOW": "0"},
    {"SGFEM_JIT_WINDOW": "0", "SGFEM_JIT_DIFF": "0"},
    {"SGFEM_JIT_WINDOW": "0", "SGFEM_JIT_PFD": "2"},
    {"SGFEM_JIT_WINDOW": "0", "SGFEM_JIT_NBUF": "2"},
    {"SGFEM_JIT_WINDOW": "0", "SGFEM_JIT_STAGE": "0"},
    {"SGFEM_JIT_PASSES": "2"},
    {"SGFEM_JIT_ASYNC": "1"},
    {"SGFEM_JIT_ASYNC": "2"},
    {"SGFEM_JIT_WINDOW": "0", "SGFEM_JIT_RCHUNK": "1", "SGFEM_JIT_PREFETCH": "1"},
]


@pytest.mark.parametrize("knobs", KNOBS, ids=lambda k: ",".join(f"{a[10:]}={b}" for a, b in k.items()) or "default")
def test_specialised_apply_launch_variants(built_pkg, monkeypatch, knobs):
    """Every generated form of the specialised FP32 apply (lattice window in its
    split-slot and pair-slot forms with their block shapes, register window with
    its prefetch depth and staging
    buffers, passes over column groups, cp.async ring, bulk copies with
    mbarriers) agrees with FP64 to FP32 accuracy."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    p = build(16, 2, 8, pkg.top_weight_multiindices(8, 60, C.decay_factors))
    for k, v in knobs.items():
        monkeypatch.setenv(k, v)
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    x = np.random.default_rng(11).standard_normal(p.n * p.P)
    y32 = op.mul(x, pkg.FP32)
    variant, log = op.ctx.apply_variant
    assert variant == 1, log
    if knobs in ({}, {"SGFEM_JIT_DIFF": "0"}):
        assert ("difference form" in log) == (knobs == {}), log
    windowed = not any(k in knobs for k in ("SGFEM_JIT_WINDOW", "SGFEM_JIT_PASSES", "SGFEM_JIT_ASYNC"))
    assert ("lattice window" in log) == windowed, log
    assert ("split slots" in log) == (windowed and knobs.get("SGFEM_JIT_SPLIT") == "1"), log
    y64 = op.mul(x, pkg.FP64)
    assert rel(y32, y64) <= 1e-5
    op.close()


def test_difference_form_accuracy_on_smooth_input(built_pkg, monkeypatch):
    """With vanishing row sums the FP32 apply evaluates sum_j K_ij (x_j - x_i):
    on a smooth x (where K x is small against |K| |x|: the direct sum cancels
    to O(h^2) |K| |x|, the differences only to O(h)) its error relative to
    FP64 is far below that of the direct sum."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    p = config1_like(N=64, order=2)
    xy = p.V.dof_coords
    base = np.sin(np.pi * xy[:, 0]) * np.sin(np.pi * xy[:, 1])
    # FP32-representable input: both forms apply the operator to the same vector
    x = np.concatenate([base * (0.5 ** k) for k in range(p.P)]).astype(np.float32).astype(np.float64)
    errs = {}
    for diff in ("1", "0"):
        monkeypatch.setenv("SGFEM_JIT_DIFF", diff)
        op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
        y32 = op.mul(x, pkg.FP32)
        assert ("difference form" in op.ctx.apply_variant[1]) == (diff == "1")
        errs[diff] = rel(y32, op.mul(x, pkg.FP64))
        op.close()
    assert errs["1"] < 0.2 * errs["0"], errs
