"""Oracle restatement of the equilibration error estimator for PoissonProblemPrimal.

Test infrastructure only (see ``oracle/__init__.py``).

Follows estimate_equilibration (src/estimate.jl:607-954) literally, per node
patch:
  * extended multi-index set, coupling G and neighbour tables as in
    estimate_primal (estimate.jl:632-646);
  * for every node z and extended mode j one global system over all RT_k
    dofs (k = order of the H1Pk space, HDIVRTk{2, k}, estimate.jl:617-619):
    on each cell T of the patch and quadrature point x_q (rule of order
    2 (k + 1), :652-654)
        A += w |T| (phi_i . phi_j) + pen sqrt|T| w |T| div phi_i div phi_j,
        b += w |T| (F_j . phi_i) phi_z + pen sqrt|T| w |T| r div phi_i,
        r = F_j . grad phi_z - f phi_z [j = 1],
    F_j = a_0 grad u_j [j active] + sum_m a_m (G u_{j+e_m} + G u_{j-e_m}) at
    x_q (:733-750, :760-786); every dof of a cell without a vertex in the
    patch gets A[i, i] = 1e60, b[i] = 0 (:709-723, :792-798); solved with a
    sparse LU (:801);
  * sigma_j = sum_z X_{z, j} (:857-860) and, per cell and mode (:861-946),
    eta_{T,j}^2 = sum_q w |T| (|F_j - sigma_j|^2 + (f [j = 1] + div sigma_j)^2 / pi^2),
    eta4modes_j = sqrt(sum_T eta_{T,j}^2).
Each node is its own group (the reference solves the patches of one
NodePatchGroups group together; ExtendableGrids' grouping is not restated).
The RT_k basis here is built per physical cell, dual to point values of the
normal flux sigma . R(B - A) at the k + 1 Gauss points of each edge (A the
lower node, R the rotation by -90 degrees) and to the moments of sigma against
P_{k-1} in barycentric form; any basis of RT_k with normal-flux edge dofs
spans the same constrained spaces, so the estimate does not depend on it.
UNPINNED: Julia and ExtendableFEM are absent, no reference output exists.
"""
import copy
import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .basis import get_tensor_multiplication_with_ym
from .fem import triangle_rule
from .mopcontrol import add_boundary_modes, get_neighbours


def _rt_span(k, xc, h):
    """monomial spanning set of RT_k in the scaled coordinates (x - xc) / h:
    list of callables (x, y) -> (value (2,), divergence)."""
    funcs = []
    for c in range(2):
        for a in range(k + 1):
            for b in range(k + 1 - a):
                def f(x, y, c=c, a=a, b=b):
                    X, Y = (x - xc[0]) / h, (y - xc[1]) / h
                    v = np.zeros(2)
                    v[c] = X ** a * Y ** b
                    if c == 0:
                        dv = a * X ** (a - 1) * Y ** b / h if a > 0 else 0.0
                    else:
                        dv = b * X ** a * Y ** (b - 1) / h if b > 0 else 0.0
                    return v, dv
                funcs.append(f)
    for a in range(k, -1, -1):
        b = k - a

        def f(x, y, a=a, b=b):
            X, Y = (x - xc[0]) / h, (y - xc[1]) / h
            m = X ** a * Y ** b
            return np.array([X * m, Y * m]), (2 + k) * m / h
        funcs.append(f)
    return funcs


class RTSpace:
    """RT_k on the mesh: dofs = (k + 1) per face, then k (k + 1) per cell."""

    def __init__(self, mesh, k):
        self.mesh = mesh
        self.k = k
        self.nint = k * (k + 1)
        self.nb = 3 * (k + 1) + self.nint
        self.ndofs = (k + 1) * mesh.nfaces + self.nint * mesh.ncells
        gt, _ = np.polynomial.legendre.leggauss(k + 1)
        self.edge_t = (gt + 1.0) / 2.0
        self.celldofs = np.zeros((mesh.ncells, self.nb), dtype=np.int64)
        self.coef = []
        ip, iw = triangle_rule(2 * k + 2)
        for c in range(mesh.ncells):
            nodes = mesh.cells[c]
            P = mesh.coords[nodes]
            xc = P.mean(axis=0)
            span = _rt_span(k, xc, math.sqrt(mesh.cell_volumes[c]))
            D = np.zeros((self.nb, self.nb))
            r = 0
            for e in range(3):
                f = mesh.cellfaces[c, e]
                A, B = sorted(mesh.face_nodes[f])
                pa, pb = mesh.coords[A], mesh.coords[B]
                nrm = np.array([pb[1] - pa[1], -(pb[0] - pa[0])])
                for l, t in enumerate(self.edge_t):
                    x = pa + t * (pb - pa)
                    for j, fn in enumerate(span):
                        D[r, j] = fn(x[0], x[1])[0] @ nrm
                    self.celldofs[c, r] = (k + 1) * f + l
                    r += 1
            J = np.array([P[1] - P[0], P[2] - P[0]]).T
            vol = abs(np.linalg.det(J)) / 2
            tests = [lambda lam: 1.0] if k == 1 else [lambda lam, i=i: lam[i] for i in range(3)]
            for comp in range(2):
                for ti, tf in enumerate(tests):
                    for q in range(len(iw)):
                        lam = np.array([1 - ip[q, 0] - ip[q, 1], ip[q, 0], ip[q, 1]])
                        x = P[0] + J @ ip[q]
                        for j, fn in enumerate(span):
                            D[r, j] += iw[q] * vol * fn(x[0], x[1])[0][comp] * tf(lam)
                    self.celldofs[c, r] = (k + 1) * mesh.nfaces + self.nint * c + comp * len(tests) + ti
                    r += 1
            self.coef.append((np.linalg.inv(D), span))

    def eval(self, c, x):
        """values (nb, 2) and divergences (nb,) of the cell's global basis at x."""
        Cinv, span = self.coef[c]
        V = np.zeros((len(span), 2))
        dv = np.zeros(len(span))
        for j, fn in enumerate(span):
            V[j], dv[j] = fn(x[0], x[1])
        return Cinv.T @ V, Cinv.T @ dv


def estimate_equilibration(space, U, multi_indices, obt, coef, f, tail_extension=(10, 2), div_penalty=1.0e5,
                           quadorder=None):
    """Returns (eta4modes, eta4cell (ncells, P_ext), extended multi-indices)."""
    mesh = space.mesh
    nmodes = len(multi_indices)
    ext = add_boundary_modes(copy.deepcopy([list(m) for m in multi_indices]), tail_extension=tail_extension)
    M_ext = len(ext[0])
    next_ = len(ext)
    G = get_tensor_multiplication_with_ym(obt, ext)
    plus, minus = get_neighbours(ext)
    k = space.order
    RT = RTSpace(mesh, k)
    pts, wts = triangle_rule(2 * (k + 1) if quadorder is None else quadorder)
    n = space.ndofs
    nc = mesh.ncells
    nq = len(wts)
    vol = mesh.cell_volumes
    # per cell and quadrature point: x, P1 values, FE gradients, RT basis, F_j
    X = np.zeros((nc, nq, 2))
    PHI1 = np.zeros((nc, nq, 3))
    GL = np.zeros((nc, 3, 2))
    RV = np.zeros((nc, nq, RT.nb, 2))
    RD = np.zeros((nc, nq, RT.nb))
    F = np.zeros((next_, nc, nq, 2))
    for c in range(nc):
        p, J, gl = space.cell_geometry(c)
        GL[c] = gl
        cd = space.celldofs[c]
        for q in range(nq):
            lam = np.array([1 - pts[q, 0] - pts[q, 1], pts[q, 0], pts[q, 1]])
            x = p[0] + J @ pts[q]
            X[c, q] = x
            PHI1[c, q] = lam
            RV[c, q], RD[c, q] = RT.eval(c, x)
            _, g, _ = space.local_basis(lam, gl)
            am = [coef.get_am(x[0], x[1], m) for m in range(M_ext + 1)]
            for j in range(next_):
                cu = np.zeros(len(cd))
                if j < nmodes:
                    cu += U[j * n + cd] * am[0]
                for m in range(1, M_ext + 1):
                    cp = plus[m - 1][j]
                    cm = minus[m - 1][j]
                    cplus = U[(cp - 1) * n + cd] * G[(m - 1) * next_ + j, cp - 1] if 0 < cp <= nmodes else 0.0
                    cmin = U[(cm - 1) * n + cd] * G[(m - 1) * next_ + j, cm - 1] if 0 < cm <= nmodes else 0.0
                    cu = cu + (cplus + cmin) * am[m]
                F[j, c, q] = cu @ g
    fx = np.asarray(f(X[..., 0], X[..., 1]), dtype=np.float64) * np.ones((nc, nq))

    node_cells = [[] for _ in range(mesh.nnodes)]
    for c in range(nc):
        for v in mesh.cells[c]:
            node_cells[v].append(c)
    sigma = np.zeros((next_, RT.ndofs))
    for z in range(mesh.nnodes):
        cells = node_cells[z]
        inside = np.zeros(nc, dtype=bool)
        inside[cells] = True
        rows, cols, vals = [], [], []
        B = np.zeros((RT.ndofs, next_))
        for c in cells:
            loc = list(mesh.cells[c]).index(z)
            dofs = RT.celldofs[c]
            Al = np.zeros((RT.nb, RT.nb))
            bl = np.zeros((RT.nb, next_))
            for q in range(nq):
                w = wts[q] * vol[c]
                t2 = div_penalty * math.sqrt(vol[c]) * w
                r = F[:, c, q] @ GL[c, loc]
                r[0] -= fx[c, q] * PHI1[c, q, loc]
                bl += (RV[c, q] @ F[:, c, q].T) * PHI1[c, q, loc] * w
                bl += t2 * np.outer(RD[c, q], r)
                Al += (RV[c, q] @ RV[c, q].T) * w + t2 * np.outer(RD[c, q], RD[c, q])
            for i in range(RT.nb):
                B[dofs[i]] += bl[i]
                for jj in range(RT.nb):
                    rows.append(dofs[i])
                    cols.append(dofs[jj])
                    vals.append(Al[i, jj])
        A = sp.coo_matrix((vals, (rows, cols)), shape=(RT.ndofs, RT.ndofs)).tolil()
        pinned = np.zeros(RT.ndofs, dtype=bool)
        for c in np.nonzero(~inside)[0]:
            pinned[RT.celldofs[c]] = True
        for dof in np.nonzero(pinned)[0]:
            A[dof, dof] = 1.0e60
            B[dof] = 0.0
        Xz = spla.splu(A.tocsc()).solve(B)
        sigma += Xz.T

    eta4cell = np.zeros((nc, next_))
    for c in range(nc):
        cf = sigma[:, RT.celldofs[c]]                      # next x nb
        for q in range(nq):
            s = cf @ RV[c, q]                              # next x 2
            dv = cf @ RD[c, q]
            dv[0] += fx[c, q]
            d = F[:, c, q] - s
            eta4cell[c] += (np.sum(d * d, axis=1) + dv ** 2 / math.pi ** 2) * wts[q] * vol[c]
    return np.sqrt(eta4cell.sum(axis=0)), eta4cell, ext
