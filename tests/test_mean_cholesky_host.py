"""The sparse-Cholesky mean preconditioner (SGFEM_PREC_CHOLESKY) on the host:
sgfem_cholesky_host_solve runs its nested-dissection ordering, factorisation and
the device kernels' solve schedule without a GPU.  It must equal the
reference's ldiv! (solvers_poisson_primal.jl:23-78: LU of K_0 with 1e60 on the
boundary diagonals, one solve per mode; the oracle's MeanPreconditioner) to
1e-12 relative, on perturbed (non-lattice) and lattice meshes, P1 and P2."""
import numpy as np
import pytest

from oracle import sg as osg


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("order,N,mesh", [(1, 12, "perturbed"), (2, 8, "perturbed"), (1, 16, "lattice"),
                                          (2, 16, "lattice"), (1, 40, "perturbed"), (2, 3, "perturbed"),
                                          (1, 12, "lattice")])
def test_host_cholesky_matches_lu(pkg, order, N, mesh):
    import __graft_entry__ as ge
    ge.build()
    m = pkg.perturbed_unit_square_mesh(N, 0.2, seed=N) if mesh == "perturbed" else pkg.unit_square_mesh(N)
    V = pkg.H1Pk(m, order)
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=10)
    K0 = pkg.assemble_stiffness(V, C, [0], 2 * (order - 1) + 2)[0]
    P = 5
    B = np.random.default_rng(N).standard_normal(V.ndofs * P)
    Z, summary = pkg.cholesky_host_solve(K0, V.bdofs, B)
    ref = osg.MeanPreconditioner(K0, V.bdofs, P).ldiv(B)
    mask = osg.interior_mask(V.ndofs, P, V.bdofs)
    assert rel(Z[mask], ref[mask]) <= 1e-12, summary
    assert np.all(Z[~mask] == 0.0)
    assert "nnz(L)" in summary
    # structured P1 meshes carry exact zeros (the diagonal edges); they stay out of
    # both the dissection graph and the factor, and the factorisation checks that
    # every gathered entry lies in a descendant node (else it raises)


def test_host_cholesky_varying_mean_and_errors(pkg):
    """A spatially varying mean field (nodal P1 mean) and a matrix that is not
    positive definite on the interior dofs (reported, not solved)."""
    import __graft_entry__ as ge
    ge.build()
    V = pkg.H1Pk(pkg.perturbed_unit_square_mesh(10, 0.2, seed=3), 1)
    alpha = 1.0 + 0.5 * np.sin(3 * V.mesh.coords[:, 0]) ** 2
    K0 = pkg.assemble_stiffness_nodal_mean(V, alpha, 2)
    B = np.random.default_rng(1).standard_normal(V.ndofs * 3)
    Z, _ = pkg.cholesky_host_solve(K0, V.bdofs, B)
    ref = osg.MeanPreconditioner(K0, V.bdofs, 3).ldiv(B)
    mask = osg.interior_mask(V.ndofs, 3, V.bdofs)
    assert rel(Z[mask], ref[mask]) <= 1e-12
    with pytest.raises(pkg.SGError) as e:
        pkg.cholesky_host_solve(-K0, V.bdofs, B)
    assert "positive definite" in str(e.value)


def test_perturbed_mesh_is_valid(pkg):
    m = pkg.perturbed_unit_square_mesh(16, 0.24, seed=7)
    p, t = m.coords, m.cells
    area = 0.5 * ((p[t[:, 1], 0] - p[t[:, 0], 0]) * (p[t[:, 2], 1] - p[t[:, 0], 1])
                  - (p[t[:, 2], 0] - p[t[:, 0], 0]) * (p[t[:, 1], 1] - p[t[:, 0], 1]))
    assert np.all(area > 0)
    assert abs(area.sum() - 1.0) < 1e-12
    V = pkg.H1Pk(m, 1)
    assert len(V.bdofs) == 64
