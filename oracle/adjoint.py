"""Oracle for the adjoint gradient of the mean quantity of interest.

Test infrastructure only (see ``oracle/__init__.py``).  The reference package
has no derivative; this restates the forward problem it solves
(src/modelproblems/poisson_primal.jl:38-81 with solve_full_primal!,
solvers_poisson_primal.jl:172-230) with K_0 built from a nodal P1 mean field
a_0 = sum_i alpha_i phi_i and the KLE blocks scaled by theta_m, and the
adjoint formulas
  dJ/dtheta_m = -Lambda^T (G_m (x) K_m) U,
  dJ/dalpha_i = -sum_mu Lambda_mu^T K_0^(i) U_mu,  K_0^(i) = (phi_i grad u, grad v),
by element loops and the assembled Kronecker solve.  Pinned by central finite
differences of the forward solve (tests/test_oracle_identities.py).
"""
import numpy as np

from .fem import assemble_rhs, assemble_stiffness, triangle_rule
from .sg import kron_direct


def assemble_mean_field(space, alpha, quadorder):
    """K_0(alpha) by element loops; a_0(x) = sum_a alpha[node a] lambda_a(x)."""
    import scipy.sparse as sp
    pts, wts = triangle_rule(quadorder)
    nd = space.ndofs4cell()
    rows, cols, vals = [], [], []
    for c in range(space.mesh.ncells):
        p, J, gl = space.cell_geometry(c)
        vol = space.mesh.cell_volumes[c]
        nodes = space.mesh.cells[c]
        loc = np.zeros((nd, nd))
        for q in range(len(wts)):
            xi, eta = pts[q]
            lam = np.array([1 - xi - eta, xi, eta])
            _, g, _ = space.local_basis(lam, gl)
            a0 = float(alpha[nodes] @ lam)
            loc += wts[q] * vol * a0 * (g @ g.T)
        dofs = space.celldofs[c]
        for a_ in range(nd):
            for b_ in range(nd):
                rows.append(dofs[a_])
                cols.append(dofs[b_])
                vals.append(loc[a_, b_])
    n = space.ndofs
    K = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    K.sum_duplicates()
    return K


class QoIOracle:
    def __init__(self, space, coef, G, P, M, f, box=(0.25, 0.75, 0.25, 0.75), quadorder_a=2):
        self.space, self.coef, self.G, self.P, self.M = space, coef, G, P, M
        self.qa = quadorder_a
        self.Km = assemble_stiffness(space, coef, list(range(1, M + 1)), quadorder_a)
        self.b0 = assemble_rhs(space, f, space.order)
        x0, x1, y0, y1 = box
        self.l = assemble_rhs(space, lambda x, y: float(x0 <= x <= x1 and y0 <= y <= y1), space.order + 1)

    def solve(self, theta, alpha, rhs):
        K0 = assemble_mean_field(self.space, alpha, self.qa)
        return kron_direct(K0, [t * K for t, K in zip(theta, self.Km)], self.G, rhs, self.space.bdofs, self.P)

    def value(self, theta, alpha):
        U = self.solve(theta, alpha, self.b0)
        return float(self.l @ U[:self.space.ndofs])

    def gradient(self, theta, alpha):
        n, P, M = self.space.ndofs, self.P, self.M
        U = self.solve(theta, alpha, self.b0)
        L = self.solve(theta, alpha, self.l)
        dtheta = np.zeros(M)
        for m in range(M):
            for mu in range(P):
                for nu in range(P):
                    g = self.G[m * P + mu, nu]
                    if g != 0.0:
                        dtheta[m] -= g * (L[mu * n:(mu + 1) * n] @ (self.Km[m] @ U[nu * n:(nu + 1) * n]))
        dalpha = np.zeros(self.space.mesh.nnodes)
        pts, wts = triangle_rule(self.qa)
        for c in range(self.space.mesh.ncells):
            p, J, gl = self.space.cell_geometry(c)
            vol = self.space.mesh.cell_volumes[c]
            nodes = self.space.mesh.cells[c]
            dofs = self.space.celldofs[c]
            for a in range(3):
                loc = np.zeros((len(dofs), len(dofs)))
                for q in range(len(wts)):
                    xi, eta = pts[q]
                    lam = np.array([1 - xi - eta, xi, eta])
                    _, g, _ = self.space.local_basis(lam, gl)
                    loc += wts[q] * vol * lam[a] * (g @ g.T)
                s = 0.0
                for mu in range(P):
                    s += L[mu * n + dofs] @ loc @ U[mu * n + dofs]
                dalpha[nodes[a]] -= s
        return float(self.l @ U[:n]), dtheta, dalpha
