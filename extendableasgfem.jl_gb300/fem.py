"""Spatial finite-element layer on the host (the part ExtendableGrids /
ExtendableFEMBase / ExtendableFEM provide to the reference).

* ``unit_square_mesh(N)``: N x N squares of the unit square, each split along
  the (i,j)-(i+1,j+1) diagonal (ExtendableGrids.simplexgrid-style); faces are
  numbered in order of first appearance over cells, local faces (0,1),(1,2),(2,0).
* ``H1Pk``: continuous P1 / P2 Lagrange space; dofs are the nodes, then (P2)
  one dof per face; boundary dofs are all dofs on boundary faces
  (FES[BFaceDofs], src/modelproblems/solvers_poisson_primal.jl:136-142).
* ``triangle_rule(order)``: reference-triangle quadrature with weights summing
  to one (the ExtendableFEMBase convention used in src/estimate.jl:345-346).
* ``assemble_stiffness``: K_m = (a_m grad u, grad v) for m = 0..M on one
  shared CSR pattern (src/modelproblems/poisson_primal.jl:56-63), vectorised
  over cells; ``assemble_rhs``: b = (f, v) (poisson_primal.jl:66-68).
"""
import math

import numpy as np
import scipy.sparse as sp
from scipy.special import roots_jacobi


def triangle_rule(order):
    if order <= 1:
        return np.array([[1.0 / 3.0, 1.0 / 3.0]]), np.array([1.0])
    if order == 2:
        return (np.array([[1.0 / 6.0, 1.0 / 6.0], [2.0 / 3.0, 1.0 / 6.0], [1.0 / 6.0, 2.0 / 3.0]]),
                np.full(3, 1.0 / 3.0))
    n = int(math.ceil((order + 1) / 2.0))
    xj, wj = roots_jacobi(n, 1.0, 0.0)  # collapsed direction, weight (1 - xi)
    xl, wl = np.polynomial.legendre.leggauss(n)
    xi = (xj + 1.0) / 2.0
    t = (xl + 1.0) / 2.0
    pts = np.array([[xi[a], (1.0 - xi[a]) * t[b]] for a in range(n) for b in range(n)])
    w = np.array([wj[a] * wl[b] for a in range(n) for b in range(n)])
    return pts, w / w.sum()


def line_rule(npts):
    x, w = np.polynomial.legendre.leggauss(npts)
    return (x + 1.0) / 2.0, w / w.sum()


class Mesh:
    def __init__(self, coords, cells):
        self.coords = np.asarray(coords, dtype=np.float64)
        self.cells = np.asarray(cells, dtype=np.int64)
        self.nnodes = len(self.coords)
        self.ncells = len(self.cells)
        loc = np.array([[0, 1], [1, 2], [2, 0]])
        e = self.cells[:, loc]                       # ncells x 3 x 2
        key = np.sort(e, axis=2).reshape(-1, 2)
        code = key[:, 0] * self.nnodes + key[:, 1]
        uniq, first, inv = np.unique(code, return_index=True, return_inverse=True)
        order = np.argsort(first, kind="stable")      # number faces by first appearance
        rank = np.empty_like(order)
        rank[order] = np.arange(len(order))
        self.cellfaces = rank[inv].reshape(self.ncells, 3)
        self.nfaces = len(uniq)
        self.face_nodes = key[first[order]]
        fc = np.full((self.nfaces, 2), -1, dtype=np.int64)
        flat_faces = self.cellfaces.ravel()
        flat_cells = np.repeat(np.arange(self.ncells), 3)
        o = np.argsort(flat_faces, kind="stable")  # cells stay in traversal order per face
        ff = flat_faces[o]
        fcell = flat_cells[o]
        starts = np.searchsorted(ff, np.arange(self.nfaces))
        counts = np.bincount(ff, minlength=self.nfaces)
        fc[:, 0] = fcell[starts]
        two = counts == 2
        fc[two, 1] = fcell[starts[two] + 1]
        self.face_cells = fc
        self.bfaces = np.nonzero(fc[:, 1] < 0)[0]
        p = self.coords
        t = self.cells
        self.cell_volumes = 0.5 * np.abs((p[t[:, 1], 0] - p[t[:, 0], 0]) * (p[t[:, 2], 1] - p[t[:, 0], 1])
                                         - (p[t[:, 2], 0] - p[t[:, 0], 0]) * (p[t[:, 1], 1] - p[t[:, 0], 1]))
        fn = self.face_nodes
        self.face_volumes = np.hypot(p[fn[:, 1], 0] - p[fn[:, 0], 0], p[fn[:, 1], 1] - p[fn[:, 0], 1])
        # affine maps: x = p0 + J (xi, eta); grad lambda_i per cell
        J = np.stack([p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]]], axis=2)  # nc x 2 x 2 (columns)
        self.J = J
        Jinv = np.linalg.inv(J)
        gl = np.zeros((self.ncells, 3, 2))
        gl[:, 1] = Jinv[:, 0, :]
        gl[:, 2] = Jinv[:, 1, :]
        gl[:, 0] = -gl[:, 1] - gl[:, 2]
        self.grad_lambda = gl


def unit_square_mesh(N):
    idx = lambda i, j: j * (N + 1) + i
    xs = np.arange(N + 1) / N
    X, Y = np.meshgrid(xs, xs)
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    i, j = np.meshgrid(np.arange(N), np.arange(N))
    i = i.ravel()
    j = j.ravel()
    t1 = np.stack([idx(i, j), idx(i + 1, j), idx(i + 1, j + 1)], axis=1)
    t2 = np.stack([idx(i, j), idx(i + 1, j + 1), idx(i, j + 1)], axis=1)
    cells = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return Mesh(coords, cells)


def perturbed_unit_square_mesh(N, delta=0.2, seed=0):
    """unit_square_mesh(N) with every interior vertex moved by a uniform random
    offset of at most delta * h in each direction (h = 1/N; delta < 0.25 keeps every
    triangle positively oriented, at 0.25 two corners can meet): a non-uniform mesh
    whose dofs form no lattice, standing in for the locally refined meshes of the
    adaptive loop."""
    if not (0.0 <= delta < 0.25):
        raise ValueError("delta in [0, 0.25)")
    m = unit_square_mesh(N)
    p = m.coords.copy()
    inner = np.nonzero((p[:, 0] > 0) & (p[:, 0] < 1) & (p[:, 1] > 0) & (p[:, 1] < 1))[0]
    rng = np.random.default_rng(seed)
    p[inner] += rng.uniform(-delta / N, delta / N, size=(len(inner), 2))
    return Mesh(p, m.cells)


class H1Pk:
    def __init__(self, mesh, order):
        if order not in (1, 2):
            raise ValueError("H1Pk: order 1 or 2")
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
            self.dof_coords = np.concatenate([mesh.coords, 0.5 * (mesh.coords[fn[:, 0]] + mesh.coords[fn[:, 1]])])
        bf = mesh.bfaces
        bd = [mesh.face_nodes[bf, 0], mesh.face_nodes[bf, 1]]
        if order == 2:
            bd.append(mesh.nnodes + bf)
        self.bdofs = np.unique(np.concatenate(bd))

    @property
    def ndofs4cell(self):
        return 3 if self.order == 1 else 6

    def basis(self, lam):
        """values (nd,), gradient factors and laplacians at barycentric lam for all cells:
        returns vals (nd,), grads (nc, nd, 2), laps (nc, nd)."""
        gl = self.mesh.grad_lambda
        if self.order == 1:
            return lam.copy(), gl.copy(), np.zeros(gl.shape[:2])
        nc = gl.shape[0]
        v = np.zeros(6)
        g = np.zeros((nc, 6, 2))
        lap = np.zeros((nc, 6))
        for i in range(3):
            v[i] = lam[i] * (2 * lam[i] - 1)
            g[:, i] = (4 * lam[i] - 1) * gl[:, i]
            lap[:, i] = 4 * np.sum(gl[:, i] ** 2, axis=1)
        for e, (a, b) in enumerate(((0, 1), (1, 2), (2, 0))):
            v[3 + e] = 4 * lam[a] * lam[b]
            g[:, 3 + e] = 4 * (lam[a] * gl[:, b] + lam[b] * gl[:, a])
            lap[:, 3 + e] = 8 * np.sum(gl[:, a] * gl[:, b], axis=1)
        return v, g, lap

    def physical_points(self, pts):
        """(nc, nq, 2) physical coordinates of reference points: p0 + J xi per cell
        (broadcast products, summed as (J_i0 xi_0 + J_i1 xi_1) before adding p0)."""
        p0 = self.mesh.coords[self.mesh.cells[:, 0]]
        J = self.mesh.J
        pts = np.asarray(pts, dtype=np.float64)
        out = np.empty((len(p0), len(pts), 2))
        for i in range(2):
            out[:, :, i] = p0[:, i:i + 1] + (J[:, i, 0:1] * pts[None, :, 0] + J[:, i, 1:2] * pts[None, :, 1])
        return out

    def pattern(self):
        """CSR pattern of the cell connectivity and the scatter map cell-entry -> nnz."""
        nd = self.ndofs4cell
        cd = self.celldofs
        rows = np.repeat(cd, nd, axis=1).ravel()
        cols = np.tile(cd, (1, nd)).ravel()
        n = self.ndofs
        code = rows * n + cols
        uniq, inv = np.unique(code, return_inverse=True)
        r = uniq // n
        c = uniq % n
        indptr = np.zeros(n + 1, dtype=np.int64)
        np.add.at(indptr, r + 1, 1)
        indptr = np.cumsum(indptr)
        return indptr, c, inv


def assemble_stiffness(space, coef, ms, quadorder):
    """[K_m for m in ms] as CSR matrices sharing one pattern."""
    pts, wts = triangle_rule(quadorder)
    X = space.physical_points(pts)  # nc x nq x 2
    vol = space.mesh.cell_volumes
    nd = space.ndofs4cell
    nc = space.mesh.ncells
    GG = []
    for q in range(len(wts)):
        lam = np.array([1 - pts[q, 0] - pts[q, 1], pts[q, 0], pts[q, 1]])
        _, g, _ = space.basis(lam)
        GG.append(np.einsum("cik,cjk->cij", g, g))
    indptr, col, inv = space.pattern()
    n = space.ndofs
    out = []
    for m in ms:
        a = coef.get_am(X[..., 0], X[..., 1], m)  # nc x nq
        loc = np.zeros((nc, nd, nd))
        for q in range(len(wts)):
            loc += (wts[q] * vol * a[:, q])[:, None, None] * GG[q]
        data = np.bincount(inv, weights=loc.ravel(), minlength=len(col))
        out.append(sp.csr_matrix((data, col, indptr), shape=(n, n)))
    return out


def assemble_rhs(space, f, quadorder):
    pts, wts = triangle_rule(quadorder)
    X = space.physical_points(pts)
    vol = space.mesh.cell_volumes
    b = np.zeros(space.ndofs)
    fx = np.broadcast_to(np.asarray(f(X[..., 0], X[..., 1]), dtype=np.float64), X.shape[:2])
    for q in range(len(wts)):
        lam = np.array([1 - pts[q, 0] - pts[q, 1], pts[q, 0], pts[q, 1]])
        v, _, _ = space.basis(lam)
        np.add.at(b, space.celldofs, (wts[q] * vol * fx[:, q])[:, None] * v[None, :])
    return b


def assemble_laplacian(space, quadorder=None):
    """A = (grad u, grad v) (logpoisson_primal.jl:97-99)."""
    class _One:
        mean_value = 1.0

        @staticmethod
        def get_am(x1, x2, m):
            return np.ones(np.shape(x1))
    q = 2 * (space.order - 1) if quadorder is None else quadorder
    return assemble_stiffness(space, _One, [0], q)[0]


def assemble_convection(space, coef, ms, quadorder):
    """[N_m for m in ms], N_m[i, j] = -(grad a_m . grad phi_j, phi_i) on the shared
    CSR pattern (logpoisson_primal.jl:101-107: test function id, ansatz grad)."""
    pts, wts = triangle_rule(quadorder)
    X = space.physical_points(pts)
    vol = space.mesh.cell_volumes
    nd = space.ndofs4cell
    nc = space.mesh.ncells
    VG = []
    for q in range(len(wts)):
        lam = np.array([1 - pts[q, 0] - pts[q, 1], pts[q, 0], pts[q, 1]])
        v, g, _ = space.basis(lam)
        VG.append((v, g))
    indptr, col, inv = space.pattern()
    n = space.ndofs
    out = []
    for m in ms:
        gx, gy = coef.get_gradam(X[..., 0], X[..., 1], m)  # nc x nq
        loc = np.zeros((nc, nd, nd))
        for q in range(len(wts)):
            v, g = VG[q]
            conv = gx[:, q, None] * g[:, :, 0] + gy[:, q, None] * g[:, :, 1]  # nc x nd (ansatz j)
            loc -= (wts[q] * vol)[:, None, None] * v[None, :, None] * conv[:, None, :]
        data = np.bincount(inv, weights=loc.ravel(), minlength=len(col))
        out.append(sp.csr_matrix((data, col, indptr), shape=(n, n)))
    return out


def pce_lambda(coef, multi_indices, x1, x2, factor=-1.0, N_truncate=None):
    """lambda_mu(x) of exp(factor * a) = sum_mu lambda_mu H_mu (coefficients.jl:219-260):
    exp(sum_{m<=N} a_m^2 / 2) exp(factor a_0) prod_d a_d^mu_d / (sqrt(prod mu_d!) factor^|mu|).
    Returns (P,) + x1.shape."""
    N = coef.maxm() if N_truncate is None else N_truncate
    x1 = np.asarray(x1, dtype=np.float64)
    x2 = np.asarray(x2, dtype=np.float64)
    s = np.zeros(x1.shape)
    for m in range(1, N + 1):
        s = s + coef.get_am(x1, x2, m) ** 2
    s = np.exp(s / 2) * math.exp(coef.meanvalue() * factor)
    M = max(len(mi) for mi in multi_indices)
    am = [coef.get_am(x1, x2, d) for d in range(1, M + 1)]
    out = np.empty((len(multi_indices),) + x1.shape)
    for k, mi in enumerate(multi_indices):
        a = np.ones(x1.shape)
        fac = 1
        for d, e in enumerate(mi):
            a = a * am[d] ** e
            fac *= math.factorial(e)
        out[k] = a / (math.sqrt(fac) * factor ** sum(mi)) * s
    return out


def assemble_pce_rhs(space, coef, multi_indices, f, quadorder, factor=-1.0, N_truncate=None):
    """b_mu = (lambda_mu f, v) for every multi-index (logpoisson_primal.jl:109-131);
    returns the n x P blocks flattened mode-major (SGFEVector layout)."""
    pts, wts = triangle_rule(quadorder)
    X = space.physical_points(pts)
    vol = space.mesh.cell_volumes
    lam_mu = pce_lambda(coef, multi_indices, X[..., 0], X[..., 1], factor, N_truncate)  # P x nc x nq
    fx = np.broadcast_to(np.asarray(f(X[..., 0], X[..., 1]), dtype=np.float64), X.shape[:2])
    P = len(multi_indices)
    n = space.ndofs
    b = np.zeros((P, n))
    for q in range(len(wts)):
        lam = np.array([1 - pts[q, 0] - pts[q, 1], pts[q, 0], pts[q, 1]])
        v, _, _ = space.basis(lam)
        for k in range(P):
            np.add.at(b[k], space.celldofs, (wts[q] * vol * lam_mu[k][:, q] * fx[:, q])[:, None] * v[None, :])
    return b.ravel()


def assemble_stiffness_nodal_mean(space, alpha, quadorder):
    """K_0(alpha) = (a_0 grad u, grad v) with the nodal P1 mean field
    a_0 = sum_i alpha_i phi_i (alpha: one value per mesh node); alpha = 1
    gives the constant mean 1."""
    alpha = np.asarray(alpha, dtype=np.float64)
    mesh = space.mesh
    if alpha.shape != (mesh.nnodes,):
        raise ValueError("alpha needs one value per mesh node")
    pts, wts = triangle_rule(quadorder)
    vol = mesh.cell_volumes
    nd = space.ndofs4cell
    nc = mesh.ncells
    av = alpha[mesh.cells]  # nc x 3
    loc = np.zeros((nc, nd, nd))
    for q in range(len(wts)):
        lam = np.array([1 - pts[q, 0] - pts[q, 1], pts[q, 0], pts[q, 1]])
        _, g, _ = space.basis(lam)
        a0 = av @ lam
        loc += (wts[q] * vol * a0)[:, None, None] * np.einsum("cik,cjk->cij", g, g)
    indptr, col, inv = space.pattern()
    data = np.bincount(inv, weights=loc.ravel(), minlength=len(col))
    n = space.ndofs
    return sp.csr_matrix((data, col, indptr), shape=(n, n))


def box_functional(space, box, quadorder=None):
    """l_i = int_box phi_i for an axis-aligned box (x0, x1, y0, y1) whose edges
    lie on mesh lines (the indicator is evaluated at interior quadrature points)."""
    x0, x1, y0, y1 = box
    ind = lambda x, y: ((x >= x0) & (x <= x1) & (y >= y0) & (y <= y1)).astype(np.float64)
    return assemble_rhs(space, ind, space.order + 1 if quadorder is None else quadorder)


def _bilinear_gpu(entry, space, coef, ms, quadorder, device, ctx):
    import ctypes
    from . import _lib
    from .estimate import _Cosine, _Quad, _mesh_struct, _ptr
    from .sampling_error import _FESpace
    ms = list(ms)
    m0, m1 = ms[0], ms[-1]
    if ms != list(range(m0, m1 + 1)):
        raise ValueError(f"{entry}: terms must be a contiguous range")
    pts, wts = triangle_rule(quadorder)
    indptr, col, _ = space.pattern()
    n = space.ndofs
    colptr = np.ascontiguousarray(indptr + 1, dtype=np.int64)   # the pattern is symmetric: CSR = CSC
    rowval = np.ascontiguousarray(col + 1, dtype=np.int64)
    nnz = len(col)
    mesh, keep = _mesh_struct(space)
    xref = np.ascontiguousarray(pts, dtype=np.float64)
    w = np.ascontiguousarray(wts, dtype=np.float64)
    q = _Quad(len(w), _ptr(xref), _ptr(w), 0, None, None)
    dfac = np.ascontiguousarray(coef.decay_factors, dtype=np.float64)
    b1 = np.ascontiguousarray(coef.b1, dtype=np.int64)
    b2 = np.ascontiguousarray(coef.b2, dtype=np.int64)
    c = _Cosine(coef.maxm(), coef.mean_value, coef.freq, _ptr(dfac), _ptr(b1), _ptr(b2))
    cd = np.ascontiguousarray(space.celldofs + 1, dtype=np.int64)
    fs = _FESpace(space.order, n, cd.ctypes.data)
    vals = np.zeros((m1 - m0 + 1, nnz))
    _with_ctx(device, ctx, lambda cx: getattr(cx.lib, entry)(
        cx.h, ctypes.byref(mesh), ctypes.byref(fs), ctypes.byref(c), m0, m1, ctypes.byref(q), nnz,
        _lib._i64p(colptr), _lib._i64p(rowval), _lib._dp(vals)))
    # values[k] is the entry (rowval[k], column) of the CSC pattern
    return [sp.csc_matrix((vals[i], col, indptr), shape=(n, n)).tocsr() for i in range(m1 - m0 + 1)]


def assemble_stiffness_gpu(space, coef, ms, quadorder, device=0, ctx=None):
    """assemble_stiffness on the GPU (sgfem_assemble_stiffness): the same CSR
    matrices (pattern of `space.pattern()`, values summed cell by cell), with the
    quadrature-point work and the per-nonzero sums on the device.  `ms` must be a
    contiguous range of terms."""
    return _bilinear_gpu("sgfem_assemble_stiffness", space, coef, ms, quadorder, device, ctx)


def assemble_convection_gpu(space, coef, ms, quadorder, device=0, ctx=None):
    """assemble_convection on the GPU (sgfem_assemble_convection):
    N_m[i, j] = -(grad a_m . grad phi_j, phi_i) for a contiguous range of terms."""
    return _bilinear_gpu("sgfem_assemble_convection", space, coef, ms, quadorder, device, ctx)


class _UnitMean:
    """a = 1: the coefficient of the Laplacian A = (grad u, grad v)."""
    mean_value = 1.0
    freq = 1.0
    decay_factors = b1 = b2 = ()

    @staticmethod
    def maxm():
        return 0


def assemble_laplacian_gpu(space, quadorder=None, device=0, ctx=None):
    """assemble_laplacian on the GPU (sgfem_assemble_stiffness with a = 1)."""
    q = 2 * (space.order - 1) if quadorder is None else quadorder
    return assemble_stiffness_gpu(space, _UnitMean, [0], q, device, ctx)[0]


def _gpu_rhs_args(space, f, quadorder):
    from .estimate import _Quad, _mesh_struct, _ptr
    from .sampling_error import _FESpace
    pts, wts = triangle_rule(quadorder)
    X = space.physical_points(pts)
    fqp = np.ascontiguousarray(np.broadcast_to(np.asarray(f(X[..., 0], X[..., 1]), dtype=np.float64), X.shape[:2]))
    mesh, keep = _mesh_struct(space)
    xref = np.ascontiguousarray(pts, dtype=np.float64)
    w = np.ascontiguousarray(wts, dtype=np.float64)
    q = _Quad(len(w), _ptr(xref), _ptr(w), 0, None, None)
    cd = np.ascontiguousarray(space.celldofs + 1, dtype=np.int64)
    fs = _FESpace(space.order, space.ndofs, cd.ctypes.data)
    return mesh, q, fs, fqp, (keep, xref, w, cd)


def _with_ctx(device, ctx, call):
    from . import _lib
    own = ctx is None
    ctx = _lib.Context(device) if own else ctx
    try:
        ctx._check(call(ctx))
    finally:
        if own:
            ctx.close()


def assemble_rhs_gpu(space, f, quadorder, device=0, ctx=None):
    """assemble_rhs on the GPU (sgfem_assemble_rhs): b = (f, v) with f evaluated
    on the host at the quadrature points and the cell sums on the device."""
    import ctypes
    from . import _lib
    mesh, q, fs, fqp, keep = _gpu_rhs_args(space, f, quadorder)
    b = np.zeros(space.ndofs)
    _with_ctx(device, ctx, lambda c: c.lib.sgfem_assemble_rhs(c.h, ctypes.byref(mesh), ctypes.byref(fs),
                                                              ctypes.byref(q), _lib._dp(fqp), _lib._dp(b)))
    return b


def assemble_pce_rhs_gpu(space, coef, multi_indices, f, quadorder, factor=-1.0, N_truncate=None, device=0, ctx=None):
    """assemble_pce_rhs on the GPU (sgfem_assemble_pce_rhs): b_mu = (lambda_mu f, v)
    for every multi-index, flattened mode-major (SGFEVector layout)."""
    import ctypes
    from . import _lib
    from .estimate import _Cosine, _ptr
    mesh, q, fs, fqp, keep = _gpu_rhs_args(space, f, quadorder)
    P = len(multi_indices)
    M = max(len(mi) for mi in multi_indices)
    mis = np.zeros((P, M), dtype=np.int32)
    for k, mi in enumerate(multi_indices):
        mis[k, :len(mi)] = mi
    N = coef.maxm() if N_truncate is None else N_truncate
    dfac = np.ascontiguousarray(coef.decay_factors, dtype=np.float64)
    b1 = np.ascontiguousarray(coef.b1, dtype=np.int64)
    b2 = np.ascontiguousarray(coef.b2, dtype=np.int64)
    c = _Cosine(coef.maxm(), coef.meanvalue(), coef.freq, _ptr(dfac), _ptr(b1), _ptr(b2))
    b = np.zeros((P, space.ndofs))
    _with_ctx(device, ctx, lambda cx: cx.lib.sgfem_assemble_pce_rhs(
        cx.h, ctypes.byref(mesh), ctypes.byref(fs), ctypes.byref(q), _lib._dp(fqp), ctypes.byref(c), M, P,
        mis.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), float(factor), int(N), _lib._dp(b)))
    return b.ravel()
