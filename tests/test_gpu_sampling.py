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


def test_sample_solves_p1_odd_count(built_pkg):
    pkg, C, V, Ks, b0, y = det_setup(N=32, order=1, M=5, S=37)
    sp_ = pkg.SampleProblems(V, Ks, y)
    U = sp_.solve(b0, rtol=1e-9)
    for s in (0, 17, 36):
        ref = osm.deterministic_solve(Ks, b0, V.bdofs, y[:, s])
        assert np.linalg.norm(U[:, s] - ref) <= 1e-7 * np.linalg.norm(ref)
    sp_.close()
