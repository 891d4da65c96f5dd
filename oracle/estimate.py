"""Oracle restatement of the residual error estimator for PoissonProblemPrimal.

Test infrastructure only (see ``oracle/__init__.py``).

Follows src/estimate.jl:260-418 literally:
  * extended multi-index set via add_boundary_modes (mopcontrol.jl:60-132),
    coupling G of the extended set (tensorizedbasis.jl:193-218), neighbour
    tables (estimate.jl:1-22);
  * volume term (estimate.jl:308-366): f for j == 1 plus, for order > 1,
    a_0 Laplace(u_j) (active j) and sum_m a_m Laplace(G-coupled active
    neighbours); squared, quadrature-weighted, scaled by |T|^3 (active j) or
    |T| (inactive j);
  * jump term (estimate.jl:370-415): for each extended mode j the face
    function sum_{m=0..M_ext} a_m [[grad w_{j,m}]] with w_{j,0} = u_j (active
    j) and w_{j,m} = sum_{+/-} G u_{neighbour} (active neighbours), squared
    and integrated over each face, boundary faces set to 0, scaled by |F|
    (active j) or 1/|F| (inactive j), added to both adjacent cells and to
    eta4modes.
UNPINNED: ExtendableFEM's FaceInterpolator projects the face function onto a
face space before the L2 norm is taken; here the face function is integrated
with a Gauss-Legendre rule given by the caller (``face_points``).
"""
import copy

import numpy as np

from .basis import get_tensor_multiplication_with_ym
from .fem import triangle_rule, line_rule
from .mopcontrol import add_boundary_modes, get_neighbours


def _cell_data(space, pts):
    mesh = space.mesh
    nc = mesh.ncells
    nq = len(pts)
    nd = space.ndofs4cell()
    X = np.zeros((nc, nq, 2))
    LAP = np.zeros((nc, nd))
    for c in range(nc):
        p, J, gl = space.cell_geometry(c)
        for q in range(nq):
            xi, eta = pts[q]
            X[c, q] = p[0] + J @ np.array([xi, eta])
            lam = np.array([1 - xi - eta, xi, eta])
            _, _, lap = space.local_basis(lam, gl)
            LAP[c] = lap
    return X, LAP


def _face_jump_grads(space, U, modes, tq):
    """[[grad u_nu]] at face points for the given (active) modes:
    array (len(modes), nfaces, nqf, 2); interior faces only (boundary faces 0)."""
    mesh = space.mesh
    nf = mesh.nfaces
    nqf = len(tq)
    n = space.ndofs
    out = np.zeros((len(modes), nf, nqf, 2))
    XF = np.zeros((nf, nqf, 2))
    for f in range(nf):
        a, b = mesh.face_nodes[f]
        pa, pb = mesh.coords[a], mesh.coords[b]
        pts = pa[None, :] + tq[:, None] * (pb - pa)[None, :]
        XF[f] = pts
        c0, c1 = mesh.face_cells[f]
        if c1 < 0:
            continue
        grads = []
        for c in (c0, c1):
            p, J, gl = space.cell_geometry(c)
            Jinv = np.linalg.inv(J)
            g = np.zeros((nqf, space.ndofs4cell(), 2))
            for q in range(nqf):
                xe = Jinv @ (pts[q] - p[0])
                lam = np.array([1 - xe[0] - xe[1], xe[0], xe[1]])
                _, gq, _ = space.local_basis(lam, gl)
                g[q] = gq
            grads.append((space.celldofs[c], g))
        for i, nu in enumerate(modes):
            u = U[nu * n:(nu + 1) * n]
            g0 = np.einsum("d,qdk->qk", u[grads[0][0]], grads[0][1])
            g1 = np.einsum("d,qdk->qk", u[grads[1][0]], grads[1][1])
            out[i, f] = g0 - g1
    return out, XF


def estimate_primal(space, U, multi_indices, obt, coef, f, bonus_quadorder=1,
                    tail_extension=(10, 2), face_points=None):
    """estimate(::Type{PoissonProblemPrimal}, sol, C; rhs, bonus_quadorder, tail_extension).

    U: column-major n x P entries.  Returns (eta4modes, eta4cell, ext).
    """
    mesh = space.mesh
    nmodes = len(multi_indices)
    ext = add_boundary_modes(copy.deepcopy([list(m) for m in multi_indices]),
                             tail_extension=tail_extension)
    M_ext = len(ext[0])
    next_ = len(ext)
    G = get_tensor_multiplication_with_ym(obt, ext)
    plus, minus = get_neighbours(ext)
    order = space.order
    quadorder = 2 * (order - 1) + bonus_quadorder
    pts, wts = triangle_rule(quadorder)
    n = space.ndofs
    nc = mesh.ncells
    vol = mesh.cell_volumes
    X, LAP = _cell_data(space, pts)
    am = np.stack([coef.get_am(X[..., 0], X[..., 1], m) for m in range(M_ext + 1)])  # (M+1, nc, nq)
    fx = f(X[..., 0], X[..., 1]) * np.ones(X.shape[:2])
    cd = space.celldofs

    def lap_mode(k):  # Laplace(u_k) per cell (constant), k 0-based active mode
        return np.sum(U[k * n:(k + 1) * n][cd] * LAP, axis=1)

    lapU = [lap_mode(k) for k in range(nmodes)] if order > 1 else None

    eta4cell = np.zeros((nc, next_))
    for j in range(next_):
        ft = np.zeros((nc, len(wts)))
        if j == 0:
            ft += fx
        if order > 1:
            if j < nmodes:
                ft += am[0] * lapU[j][:, None]
            for m in range(1, M_ext + 1):
                cp = plus[m - 1][j]
                cm = minus[m - 1][j]
                acc = np.zeros(nc)
                if 0 < cp <= nmodes:
                    acc += G[(m - 1) * next_ + j, cp - 1] * lapU[cp - 1]
                if 0 < cm <= nmodes:
                    acc += G[(m - 1) * next_ + j, cm - 1] * lapU[cm - 1]
                ft += am[m] * acc[:, None]
        eta4cell[:, j] = np.sum(ft ** 2 * wts[None, :], axis=1)
        eta4cell[:, j] *= vol ** 3 if j < nmodes else vol
    eta4modes = np.sqrt(eta4cell.sum(axis=0))

    if face_points is None:
        face_points = quadorder + 1
    tq, tw = line_rule(face_points)
    JG, XF = _face_jump_grads(space, U, list(range(nmodes)), tq)
    amf = np.stack([coef.get_am(XF[..., 0], XF[..., 1], m) for m in range(M_ext + 1)])  # (M+1, nf, nqf)
    fvol = mesh.face_volumes
    bmask = np.zeros(mesh.nfaces, dtype=bool)
    bmask[mesh.bfaces] = True
    for j in range(next_):
        val = np.zeros((mesh.nfaces, len(tq), 2))
        for m in range(0, M_ext + 1):
            w = np.zeros((mesh.nfaces, len(tq), 2))
            used = False
            if m == 0 and j < nmodes:
                w += JG[j]
                used = True
            elif m > 0:
                cp = plus[m - 1][j]
                cm = minus[m - 1][j]
                if 0 < cp <= nmodes:
                    w += JG[cp - 1] * G[(m - 1) * next_ + j, cp - 1]
                    used = True
                if 0 < cm <= nmodes:
                    w += JG[cm - 1] * G[(m - 1) * next_ + j, cm - 1]
                    used = True
            if used:
                val += amf[m][..., None] * w
        jumps = fvol * np.sum(tw[None, :] * np.sum(val ** 2, axis=2), axis=1)
        jumps[bmask] = 0.0
        if j < nmodes:
            jumps *= fvol
        else:
            jumps /= fvol
        eta4cell[:, j] += jumps[mesh.cellfaces].sum(axis=1)
        eta4modes[j] = np.sqrt(eta4modes[j] ** 2 + jumps.sum())
    return eta4modes, eta4cell, ext


def estimate_logpoisson(space, U, multi_indices, obt, coef, f, bonus_quadorder=1, tail_extension=(10, 2),
                        face_points=None):
    """estimate(::Type{LogTransformedPoissonProblemPrimal}, sol, C; rhs, bonus_quadorder,
    tail_extension), src/estimate.jl:70-257, by element loops.

    * lambda_j (the Hermite chaos coefficients of exp(-a), expa_PCE_mop with
      factor -1, coefficients.jl:219-260) interpolated into the Lagrange space
      of degree quadorder = 2 (order - 1) + bonus_quadorder (:102-114), here by
      nodal values (the reference's interpolate! is nodal for P1; its
      higher-order dofs are UNPINNED);
    * volume term (:130-214): per cell and extended mode j and quadrature point,
      f lambda_j (+ Laplace(u_j) for P2 and active j) + sum_m grad a_m . grad of the
      G-coupled active neighbours, squared and weighted, times |T|^2 (active j)
      or |T| (inactive j);
    * data term zeta = zeta1 - zeta2 (:139-156, :248-254);
    * jumps (:231-246): for active j, int_F |[[grad u_j]]|^2 times |F| on interior
      faces, added to the adjacent cells; eta4modes[j] += sqrt(eta4modes[j]^2 + sum)
      (the reference's own update).
    Returns (eta4modes, eta4cell, ext, zeta).
    """
    from .coefficient import pce_lambda
    from .fem import LagrangeSpace
    if isinstance(tail_extension, (int, np.integer)):
        raise TypeError("tail_extension must hold two entries (add_boundary_modes reads tail_extension[2])")
    mesh = space.mesh
    nmodes = len(multi_indices)
    ext = add_boundary_modes(copy.deepcopy([list(m) for m in multi_indices]), tail_extension=tail_extension)
    M_ext = len(ext[0])
    next_ = len(ext)
    G = get_tensor_multiplication_with_ym(obt, ext)
    plus, minus = get_neighbours(ext)
    order = space.order
    quadorder = 2 * (order - 1) + bonus_quadorder
    if quadorder > 2:
        raise NotImplementedError("interpolation degree above 2")
    pts, wts = triangle_rule(quadorder)
    n = space.ndofs
    nc = mesh.ncells
    vol = mesh.cell_volumes
    Vi = LagrangeSpace(mesh, max(quadorder, 1))
    lam_nodes = np.zeros((next_, Vi.ndofs))
    for j in range(next_):
        for d in range(Vi.ndofs):
            x, y = Vi.dof_coords[d]
            lam_nodes[j, d] = pce_lambda(coef, ext[j], x, y, factor=-1.0)
    Mcoeff = coef.maxm()
    eta4cell = np.zeros((nc, next_))
    zeta1 = 0.0
    zeta2 = 0.0
    for c in range(nc):
        p, J, gl = space.cell_geometry(c)
        _, _, gli = Vi.cell_geometry(c)
        dofs = space.celldofs[c]
        idofs = Vi.celldofs[c]
        lamq = np.zeros((next_, len(wts)))
        X = []
        for q, (xi, eta) in enumerate(pts):
            x = p[0] + J @ np.array([xi, eta])
            X.append(x)
            lam = np.array([1 - xi - eta, xi, eta])
            iv, _, _ = Vi.local_basis(lam, gli)
            lamq[:, q] = lam_nodes[:, idofs] @ iv
            kmL2 = sum(float(coef.get_am(x[0], x[1], m)) ** 2 for m in range(1, Mcoeff + 1))
            fq = f(x[0], x[1])
            zeta1 += fq ** 2 * np.exp(2 * kmL2) * wts[q] * vol[c]
            zeta2 += np.sum(lamq[:, q] ** 2) * fq ** 2 * wts[q] * vol[c]
        for j in range(next_):
            acc = 0.0
            for q, (xi, eta) in enumerate(pts):
                x = X[q]
                lam = np.array([1 - xi - eta, xi, eta])
                _, g, lap = space.local_basis(lam, gl)
                ft = lamq[j, q] * f(x[0], x[1])
                if order > 1 and j < nmodes:
                    ft += U[j * n + dofs] @ lap
                sig = 0.0
                for m in range(1, M_ext + 1):
                    ga = np.array([float(t) for t in coef.get_gradam(x[0], x[1], m)])
                    cv = np.zeros(len(dofs))
                    cp, cm = plus[m - 1][j], minus[m - 1][j]
                    if 0 < cp <= nmodes:
                        cv += U[(cp - 1) * n + dofs] * G[(m - 1) * next_ + j, cp - 1]
                    if 0 < cm <= nmodes:
                        cv += U[(cm - 1) * n + dofs] * G[(m - 1) * next_ + j, cm - 1]
                    sig += cv @ (g @ ga)
                acc += (ft + sig) ** 2 * wts[q]
            eta4cell[c, j] = acc * (vol[c] ** 2 if j < nmodes else vol[c])
    eta4modes = np.sqrt(eta4cell.sum(axis=0))
    tq, tw = line_rule(face_points if face_points is not None else order)
    JG, _ = _face_jump_grads(space, U, list(range(nmodes)), tq)
    fvol = mesh.face_volumes
    for j in range(nmodes):
        jumps = fvol * np.sum(tw[None, :] * np.sum(JG[j] ** 2, axis=2), axis=1) * fvol
        eta4cell[:, j] += jumps[mesh.cellfaces].sum(axis=1)
        eta4modes[j] += np.sqrt(eta4modes[j] ** 2 + jumps.sum())
    return eta4modes, eta4cell, ext, zeta1 - zeta2
