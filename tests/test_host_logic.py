"""Host-side logic of the package against the oracle (CPU only): multi-index
control (bit-exact integer work), coupling tensor, coefficient, spatial
assembly, the top-weight index set with its tie-break, and marking."""
import itertools
import math

import numpy as np
import pytest

from oracle import basis as ob
from oracle import coefficient as oc
from oracle import fem as of
from oracle import mopcontrol as om


SETS = [
    [[0], [1, 0], [0, 1], [2, 0], [0, 0, 1]],                 # scripts/poisson_simple.jl:24
    [[0]],                                                    # scripts/poisson.jl:74
    [[0, 0], [1, 0], [0, 1], [1, 1], [2, 0], [0, 2], [3, 0]],
    [[0, 0, 0], [1, 0, 0], [0, 0, 1], [2, 0, 0], [1, 0, 1], [0, 1, 0]],
]


def _copy(s):
    return [list(m) for m in s]


@pytest.mark.parametrize("mis", SETS)
@pytest.mark.parametrize("tail", [(10, 2), (3, 1), (5, 3)])
def test_add_boundary_modes_bitexact(pkg, mis, tail):
    a = om.add_boundary_modes(_copy(mis), tail_extension=tail)
    b = pkg.add_boundary_modes(_copy(mis), tail_extension=tail)
    assert a == b


@pytest.mark.parametrize("mis", SETS)
def test_classify_and_neighbours_bitexact(pkg, mis):
    ext = om.add_boundary_modes(_copy(mis))
    for nact in (1, len(mis), len(ext)):
        assert om.classify_modes(ext, ext[:nact]) == pkg.classify_modes(ext, ext[:nact])
    assert om.get_neighbours(ext) == pkg.get_neighbours(ext)


def test_classify_random_sets(pkg):
    rng = np.random.default_rng(3)
    for trial in range(20):
        M = int(rng.integers(2, 5))
        full = pkg.generate_multiindices(M, 2)
        keep = [full[0]] + [full[i] for i in range(1, len(full)) if rng.random() < 0.3]
        ext = om.add_boundary_modes(_copy(keep))
        assert pkg.add_boundary_modes(_copy(keep)) == ext
        assert om.classify_modes(ext, ext[:len(keep)]) == pkg.classify_modes(ext, ext[:len(keep)])


def test_generate_multiindices(pkg):
    for M, d in [(1, 3), (2, 2), (3, 3), (4, 1)]:
        assert pkg.generate_multiindices(M, d) == om.generate_multiindices(M, d)


def test_marking_bitexact(pkg):
    rng = np.random.default_rng(5)
    mis = _copy(SETS[0])
    ext = om.add_boundary_modes(_copy(mis))
    for trial in range(10):
        eta = rng.random(len(ext)) ** 3
        eta[rng.integers(0, len(ext), 3)] = eta[0]  # ties exercise the stable sort
        a = om.stochastic_marking(list(eta), ext, len(mis), mis, theta_stochastic=0.5)
        b = pkg.stochastic_marking(list(eta), ext, len(mis), mis, theta_stochastic=0.5)
        assert a[0] == b[0] and a[1] == b[1]
        assert a[2]["sorted_id"] == b[2]["sorted_id"] and a[2]["added"] == b[2]["added"]


@pytest.mark.parametrize("name,obt", [("legendre", ob.LEGENDRE), ("hermite", ob.HERMITE)])
def test_coupling_matrix_matches_oracle(pkg, name, obt):
    basis = pkg.LegendrePolynomials if name == "legendre" else pkg.HermitePolynomials
    for mis in (pkg.total_degree_multiindices(4, 3), pkg.generate_multiindices(3, 2)):
        Go = ob.get_tensor_multiplication_with_ym(obt, mis)
        Gp = pkg.coupling_matrix(basis, mis).toarray()
        assert np.array_equal(Go, Gp)


def test_onbasis_matches_oracle(pkg):
    for obt, basis in ((ob.HERMITE, pkg.HermitePolynomials), (ob.LEGENDRE, pkg.LegendrePolynomials)):
        a = ob.ONBasis(obt, 6, 12)
        b = pkg.ONBasis(basis, 6, 12)
        assert np.allclose(a.norms, b.norms, rtol=0, atol=1e-13)
        assert np.allclose(a.evaluate(0.3), b.evaluate(0.3), rtol=1e-13, atol=1e-14)


def test_coefficient_matches_oracle(pkg):
    a = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    b = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    assert np.array_equal(a.b1, b.b1) and np.array_equal(a.b2, b.b2)
    assert np.allclose(a.decay_factors, b.decay_factors, rtol=1e-15, atol=0)
    assert abs(b.decay_factors[0] - 0.9 * 6 / math.pi ** 2) < 1e-15  # 0.547 m^-2
    x = np.linspace(0, 1, 7)
    for m in (0, 1, 5, 40):
        assert np.allclose(a.get_am(x, x[::-1], m), b.get_am(x, x[::-1], m), rtol=1e-15, atol=1e-16)
        ga, gb = a.get_gradam(x, x[::-1], m), b.get_gradam(x, x[::-1], m)
        assert np.allclose(ga[0], gb[0], atol=1e-15) and np.allclose(ga[1], gb[1], atol=1e-15)


@pytest.mark.parametrize("order,N", [(1, 6), (2, 4)])
def test_assembly_matches_oracle(pkg, order, N):
    C = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=10)
    Cp = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=10)
    Vo = of.LagrangeSpace(of.StructuredMesh(N), order)
    Vp = pkg.H1Pk(pkg.unit_square_mesh(N), order)
    assert Vo.ndofs == Vp.ndofs
    assert np.array_equal(Vo.celldofs, Vp.celldofs)
    assert np.array_equal(Vo.bdofs, Vp.bdofs)
    assert np.allclose(Vo.dof_coords, Vp.dof_coords)
    q = 2 * (order - 1) + 2
    Ko = of.assemble_stiffness(Vo, C, [0, 1, 3], q)
    Kp = pkg.assemble_stiffness(Vp, Cp, [0, 1, 3], q)
    for a, b in zip(Ko, Kp):
        d = (a - b).toarray()
        assert np.abs(d).max() < 1e-14 * max(1.0, np.abs(a).max())
    bo = of.assemble_rhs(Vo, lambda x, y: 1.0, order)
    bp = pkg.assemble_rhs(Vp, lambda x, y: np.ones_like(x), order)
    assert np.allclose(bo, bp, rtol=0, atol=1e-15)
    mo, mp = Vo.mesh, Vp.mesh
    assert np.array_equal(mo.cellfaces, mp.cellfaces)
    assert np.array_equal(mo.face_cells, mp.face_cells)
    assert np.array_equal(mo.bfaces, mp.bfaces)


def test_p2_sizes_config2_mesh(pkg):
    """263 169 dofs on the 256 x 256 P2 mesh; 3 018 753 stiffness nonzeros."""
    V = pkg.H1Pk(pkg.unit_square_mesh(256), 2)
    assert V.ndofs == 263169
    indptr, col, _ = V.pattern()
    assert len(col) == 3018753


def _brute_top(M, P, d, maxdeg):
    best = []
    for mu in itertools.product(*[range(maxdeg + 1)] * M):
        w = sum(k * math.log(v) for k, v in zip(mu, d))
        best.append((-round(w, 11), sum(mu), tuple(-k for k in mu), list(mu)))
    best.sort()
    return [b[3] for b in best[:P]]


def test_top_weight_set_bruteforce(pkg):
    d = [0.9 * 6 / math.pi ** 2 / (m + 1) ** 2 for m in range(4)]
    for P in (5, 12, 30):
        assert pkg.top_weight_multiindices(4, P, d) == _brute_top(4, P, d, 8)


def test_top_weight_set_config2_tie(pkg):
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    mis = pkg.top_weight_multiindices(20, 150, C.decay_factors)
    assert len(mis) == 150 and mis[0] == [0] * 20
    assert max(mi[0] for mi in mis) == 12
    # the 150th index wins the tie with two others by lexicographic order
    assert mis[149] == [0, 1] + [0] * 9 + [1] + [0] * 8
    # downward closed
    s = {tuple(m) for m in mis}
    for mi in mis:
        for m in range(20):
            if mi[m] > 0:
                t = list(mi)
                t[m] -= 1
                assert tuple(t) in s
    G = pkg.coupling_matrix(pkg.LegendrePolynomials, mis)
    assert G.nnz == 560


def test_lognormal_assembly_matches_oracle(pkg):
    """A, N_m = -(grad a_m . grad u, v) and b_mu = (lambda_mu f, v) of the host
    assembly against the oracle's element loops (logpoisson_primal.jl:97-131)."""
    from oracle import coefficient as oc
    from oracle import fem as of
    for order in (1, 2):
        V = pkg.H1Pk(pkg.unit_square_mesh(4), order)
        C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.0, maxm=6)
        Co = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.0, maxm=6)
        Vo = of.LagrangeSpace(of.StructuredMesh(4), order)
        q = 2 * order - 1 + 2
        Ns = pkg.assemble_convection(V, C, [1, 2, 3], q)
        No = of.assemble_convection(Vo, Co, [1, 2, 3], q)
        for N, Nr in zip(Ns, No):
            d = (N - Nr).toarray()
            assert np.abs(d).max() <= 1e-13 * np.abs(Nr.toarray()).max()
            assert np.abs((N - N.T).toarray()).max() > 1e-3 * np.abs(Nr.toarray()).max()  # not symmetric
        A = pkg.assemble_laplacian(V)
        Ar = of.assemble_stiffness(Vo, type("One", (), {"get_am": staticmethod(lambda x1, x2, m: np.ones_like(np.asarray(x1, dtype=float)))})(), [0], 2 * (order - 1))[0]
        assert np.abs((A - Ar).toarray()).max() <= 1e-13 * np.abs(Ar.toarray()).max()
        mis = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [2, 0, 0], [1, 1, 1]]
        f = lambda x, y: 1.0 + x * 0
        b = pkg.assemble_pce_rhs(V, C, mis, lambda x, y: np.ones_like(x), order + 1)
        br = of.assemble_pce_rhs(Vo, Co, mis, f, order + 1)
        assert np.abs(b - br).max() <= 1e-13 * np.abs(br).max()


def test_splitmix64_and_config4_stream(pkg):
    """SplitMix64 (seed 0 gives 0xe220a8397b1dcdaf, the published first output) and
    the config-4 shapes drawn from it: n in [16, 128], M in [4, 16], degree in {1, 2, 3}."""
    assert pkg.splitmix64(0) == 0xE220A8397B1DCDAF
    shapes = pkg.config4_problems(256)
    assert len(shapes) == 256
    assert all(16 <= n <= 128 and 4 <= M <= 16 and 1 <= d <= 3 for n, M, d in shapes)
    assert len(set(shapes)) > 200


def test_total_degree_set_equals_filtered_tensor_set(pkg):
    """The pruned enumeration gives exactly the filtered generate_multiindices list."""
    for M, d in ((3, 2), (5, 2), (4, 3), (6, 1), (2, 4)):
        ref = sorted([mi for mi in pkg.generate_multiindices(M, d) if sum(mi) <= d], key=sum)
        assert pkg.total_degree_multiindices(M, d) == ref
    assert len(pkg.total_degree_multiindices(16, 3)) == 969


@pytest.mark.parametrize("name,obt", [("legendre", ob.LEGENDRE), ("hermite", ob.HERMITE)])
@pytest.mark.parametrize("tail", [(10, 2), (3, 1)])
def test_extension_couplings_match_oracle(pkg, name, obt, tail):
    """The estimators' extended set and per extended mode j its couplings to the
    active modes (self term, then for m = 1..M the j + e_m and j - e_m neighbours;
    estimate.jl:343-353, :385-393), vectorised on the host, against the oracle's
    G of the extended set and its neighbour lists: same entries in the same order,
    coefficients equal."""
    from extendableasgfem_gb300.estimate import extension_couplings
    basis = pkg.LegendrePolynomials if name == "legendre" else pkg.HermitePolynomials
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    for mis in (pkg.total_degree_multiindices(5, 2), pkg.top_weight_multiindices(8, 40, C.decay_factors),
                [[0], [1], [2]]):
        maxdeg = max(max(m) for m in mis)
        TB = pkg.TensorizedBasis(basis, len(mis[0]), maxdeg, maxdeg + 4, multi_indices=mis)
        ext, (ptr, ms, nus, gs) = extension_couplings(TB.multi_indices, TB.basis, tail)
        ext_o = om.add_boundary_modes(_copy(mis), tail_extension=tail)
        assert [list(e) for e in ext] == [list(e) for e in ext_o]
        G = ob.get_tensor_multiplication_with_ym(obt, ext_o)
        plus, minus = om.get_neighbours(ext_o)
        P_ext, nmodes, M_ext = len(ext_o), len(mis), len(ext_o[0])
        want = []
        for j in range(P_ext):
            row = [(0, j, 1.0)] if j < nmodes else []
            for m in range(1, M_ext + 1):
                for nb in (plus[m - 1][j], minus[m - 1][j]):
                    if 0 < nb <= nmodes:
                        row.append((m, nb - 1, G[(m - 1) * P_ext + j, nb - 1]))
            want.append(row)
        got = [list(zip(ms[ptr[j]:ptr[j + 1]], nus[ptr[j]:ptr[j + 1]], gs[ptr[j]:ptr[j + 1]])) for j in range(P_ext)]
        assert [[(int(a), int(b)) for a, b, _ in r] for r in got] == [[(a, b) for a, b, _ in r] for r in want]
        g_got = np.array([g for r in got for _, _, g in r])
        g_want = np.array([g for r in want for _, _, g in r])
        assert np.allclose(g_got, g_want, rtol=1e-14, atol=0)
