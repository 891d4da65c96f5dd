"""Oracle spatial layer: structured triangle mesh, P1/P2 Lagrange elements,
quadrature rules and element-by-element assembly.

Test infrastructure only (see ``oracle/__init__.py``).

This layer lives outside the reference tree (ExtendableGrids.simplexgrid /
uniform_refine, ExtendableFEMBase QuadratureRule and H1Pk, ExtendableFEM
assemble!), so it is a restatement of standard finite-element practice and
its parity with the reference is UNPINNED.  What it must agree with is the
reference's use of it:
  * K_m = (a_m grad u, grad v) for m = 0..M, quadrature order
    2(p-1) + bonus_quadorder_a        (src/modelproblems/poisson_primal.jl:56-63)
  * b = (f, v), quadrature order p + bonus_quadorder_f (poisson_primal.jl:66-68)
  * boundary dofs = all dofs on boundary faces (solvers_poisson_primal.jl:136-142)
Mesh: unit square, N x N squares, each split along the (i,j)-(i+1,j+1) diagonal.
Quadrature: weights sum to one on the reference cell (ExtendableFEMBase
convention, also visible in src/estimate.jl:345-346).
"""
import math

import numpy as np
import scipy.sparse as sp
from scipy.special import roots_jacobi


def triangle_rule(order):
    """Reference-triangle rule exact to ``order``: points (xi, eta), weights sum 1."""
    if order <= 1:
        return np.array([[1.0 / 3.0, 1.0 / 3.0]]), np.array([1.0])
    if order == 2:
        return (np.array([[1.0 / 6.0, 1.0 / 6.0], [2.0 / 3.0, 1.0 / 6.0], [1.0 / 6.0, 2.0 / 3.0]]),
                np.full(3, 1.0 / 3.0))
    n = int(math.ceil((order + 1) / 2.0))
    # conical product: xi with weight (1 - xi) (Gauss-Jacobi alpha=1), t Gauss-Legendre
    xj, wj = roots_jacobi(n, 1.0, 0.0)
    xl, wl = np.polynomial.legendre.leggauss(n)
    xi = (xj + 1.0) / 2.0
    t = (xl + 1.0) / 2.0
    pts = []
    wts = []
    for a in range(n):
        for b in range(n):
            pts.append([xi[a], (1.0 - xi[a]) * t[b]])
            wts.append(wj[a] * wl[b])
    w = np.array(wts)
    return np.array(pts), w / w.sum()


def line_rule(npts):
    x, w = np.polynomial.legendre.leggauss(npts)
    return (x + 1.0) / 2.0, w / w.sum()


class StructuredMesh:
    def __init__(self, N):
        self.N = N
        idx = lambda i, j: j * (N + 1) + i
        xs = np.arange(N + 1) / N
        X, Y = np.meshgrid(xs, xs)
        self.coords = np.stack([X.ravel(), Y.ravel()], axis=1)
        cells = []
        for j in range(N):
            for i in range(N):
                cells.append([idx(i, j), idx(i + 1, j), idx(i + 1, j + 1)])
                cells.append([idx(i, j), idx(i + 1, j + 1), idx(i, j + 1)])
        self.cells = np.array(cells, dtype=np.int64)
        self.nnodes = (N + 1) ** 2
        self.ncells = len(cells)
        edge_id = {}
        cellfaces = np.zeros((self.ncells, 3), dtype=np.int64)
        face_nodes = []
        face_cells = []
        for c in range(self.ncells):
            for e, (a, b) in enumerate(((0, 1), (1, 2), (2, 0))):
                key = tuple(sorted((int(self.cells[c, a]), int(self.cells[c, b]))))
                if key not in edge_id:
                    edge_id[key] = len(face_nodes)
                    face_nodes.append(key)
                    face_cells.append([c, -1])
                else:
                    face_cells[edge_id[key]][1] = c
                cellfaces[c, e] = edge_id[key]
        self.cellfaces = cellfaces
        self.face_nodes = np.array(face_nodes, dtype=np.int64)
        self.face_cells = np.array(face_cells, dtype=np.int64)
        self.nfaces = len(face_nodes)
        self.bfaces = np.nonzero(self.face_cells[:, 1] < 0)[0]
        p = self.coords
        self.cell_volumes = np.array([0.5 * abs((p[t[1], 0] - p[t[0], 0]) * (p[t[2], 1] - p[t[0], 1])
                                                - (p[t[2], 0] - p[t[0], 0]) * (p[t[1], 1] - p[t[0], 1]))
                                      for t in self.cells])
        fn = self.face_nodes
        self.face_volumes = np.hypot(p[fn[:, 1], 0] - p[fn[:, 0], 0], p[fn[:, 1], 1] - p[fn[:, 0], 1])


class LagrangeSpace:
    """H1-conforming P1 or P2 on a StructuredMesh (dofs: nodes, then faces)."""

    def __init__(self, mesh, order):
        assert order in (1, 2)
        self.mesh = mesh
        self.order = order
        if order == 1:
            self.celldofs = mesh.cells.copy()
            self.ndofs = mesh.nnodes
            self.dof_coords = mesh.coords.copy()
        else:
            self.celldofs = np.concatenate([mesh.cells, mesh.nnodes + mesh.cellfaces], axis=1)
            self.ndofs = mesh.nnodes + mesh.nfaces
            fn = mesh.face_nodes
            mid = 0.5 * (mesh.coords[fn[:, 0]] + mesh.coords[fn[:, 1]])
            self.dof_coords = np.concatenate([mesh.coords, mid], axis=0)
        bd = set()
        for f in mesh.bfaces:
            bd.add(int(mesh.face_nodes[f, 0]))
            bd.add(int(mesh.face_nodes[f, 1]))
            if order == 2:
                bd.add(int(mesh.nnodes + f))
        self.bdofs = np.array(sorted(bd), dtype=np.int64)

    def ndofs4cell(self):
        return 3 if self.order == 1 else 6

    def cell_geometry(self, c):
        p = self.mesh.coords[self.mesh.cells[c]]
        J = np.array([[p[1, 0] - p[0, 0], p[2, 0] - p[0, 0]],
                      [p[1, 1] - p[0, 1], p[2, 1] - p[0, 1]]])
        Jinv = np.linalg.inv(J)
        gl = np.zeros((3, 2))
        gl[1] = Jinv[0]
        gl[2] = Jinv[1]
        gl[0] = -gl[1] - gl[2]
        return p, J, gl  # gl[i] = grad lambda_i

    def local_basis(self, lam, gl):
        """values (nd,), gradients (nd, 2), laplacians (nd,) at barycentric lam."""
        if self.order == 1:
            return lam.copy(), gl.copy(), np.zeros(3)
        v = np.zeros(6)
        g = np.zeros((6, 2))
        lap = np.zeros(6)
        for i in range(3):
            v[i] = lam[i] * (2 * lam[i] - 1)
            g[i] = (4 * lam[i] - 1) * gl[i]
            lap[i] = 4 * gl[i] @ gl[i]
        for e, (a, b) in enumerate(((0, 1), (1, 2), (2, 0))):
            v[3 + e] = 4 * lam[a] * lam[b]
            g[3 + e] = 4 * (lam[a] * gl[b] + lam[b] * gl[a])
            lap[3 + e] = 8 * gl[a] @ gl[b]
        return v, g, lap


def assemble_stiffness(space, coef, ms, quadorder):
    """Element loop: returns [K_m] (CSR, shared pattern with explicit zeros)."""
    pts, wts = triangle_rule(quadorder)
    nd = space.ndofs4cell()
    rows, cols = [], []
    vals = {m: [] for m in ms}
    for c in range(space.mesh.ncells):
        p, J, gl = space.cell_geometry(c)
        vol = space.mesh.cell_volumes[c]
        loc = {m: np.zeros((nd, nd)) for m in ms}
        for q in range(len(wts)):
            xi, eta = pts[q]
            lam = np.array([1 - xi - eta, xi, eta])
            x = p[0] + J @ np.array([xi, eta])
            _, g, _ = space.local_basis(lam, gl)
            GG = g @ g.T
            for m in ms:
                a = float(coef.get_am(x[0], x[1], m))
                loc[m] += wts[q] * vol * a * GG
        dofs = space.celldofs[c]
        for a_ in range(nd):
            for b_ in range(nd):
                rows.append(dofs[a_])
                cols.append(dofs[b_])
        for m in ms:
            vals[m].extend(loc[m].ravel().tolist())
    n = space.ndofs
    out = []
    for m in ms:
        K = sp.coo_matrix((np.array(vals[m]), (np.array(rows), np.array(cols))), shape=(n, n)).tocsr()
        K.sum_duplicates()
        K.sort_indices()
        out.append(K)
    return out


def assemble_rhs(space, f, quadorder):
    pts, wts = triangle_rule(quadorder)
    b = np.zeros(space.ndofs)
    for c in range(space.mesh.ncells):
        p, J, gl = space.cell_geometry(c)
        vol = space.mesh.cell_volumes[c]
        for q in range(len(wts)):
            xi, eta = pts[q]
            lam = np.array([1 - xi - eta, xi, eta])
            x = p[0] + J @ np.array([xi, eta])
            v, _, _ = space.local_basis(lam, gl)
            b[space.celldofs[c]] += wts[q] * vol * f(x[0], x[1]) * v
    return b


def assemble_convection(space, coef, ms, quadorder):
    """N_m = -(grad a_m . grad u, v), test function v = phi_i (row), ansatz
    u = phi_j (column): src/modelproblems/logpoisson_primal.jl:101-107
    (BilinearOperator(get_gradam_x_sigma, [id(1)], [grad(1)]; factor = -1))."""
    pts, wts = triangle_rule(quadorder)
    nd = space.ndofs4cell()
    rows, cols = [], []
    vals = {m: [] for m in ms}
    for c in range(space.mesh.ncells):
        p, J, gl = space.cell_geometry(c)
        vol = space.mesh.cell_volumes[c]
        loc = {m: np.zeros((nd, nd)) for m in ms}
        for q in range(len(wts)):
            xi, eta = pts[q]
            lam = np.array([1 - xi - eta, xi, eta])
            x = p[0] + J @ np.array([xi, eta])
            v, g, _ = space.local_basis(lam, gl)
            for m in ms:
                ga = np.array([float(t) for t in coef.get_gradam(x[0], x[1], m)])
                loc[m] -= wts[q] * vol * np.outer(v, g @ ga)
        dofs = space.celldofs[c]
        for a_ in range(nd):
            for b_ in range(nd):
                rows.append(dofs[a_])
                cols.append(dofs[b_])
        for m in ms:
            vals[m].extend(loc[m].ravel().tolist())
    n = space.ndofs
    out = []
    for m in ms:
        K = sp.coo_matrix((np.array(vals[m]), (np.array(rows), np.array(cols))), shape=(n, n)).tocsr()
        K.sum_duplicates()
        K.sort_indices()
        out.append(K)
    return out


def assemble_pce_rhs(space, coef, multi_indices, f, quadorder, factor=-1.0, N_truncate=None):
    """b_mu = (lambda_mu f, v) (logpoisson_primal.jl:109-131), mode-major n*P."""
    from .coefficient import pce_lambda
    pts, wts = triangle_rule(quadorder)
    P = len(multi_indices)
    b = np.zeros((P, space.ndofs))
    for c in range(space.mesh.ncells):
        p, J, gl = space.cell_geometry(c)
        vol = space.mesh.cell_volumes[c]
        for q in range(len(wts)):
            xi, eta = pts[q]
            lam = np.array([1 - xi - eta, xi, eta])
            x = p[0] + J @ np.array([xi, eta])
            v, _, _ = space.local_basis(lam, gl)
            fx = f(x[0], x[1])
            for k in range(P):
                b[k, space.celldofs[c]] += wts[q] * vol * pce_lambda(coef, multi_indices[k], x[0], x[1], factor,
                                                                     N_truncate) * fx * v
    return b.ravel()
