"""Oracle restatement of the SG evaluation at samples and the sampling error.

Test infrastructure only (see ``oracle/__init__.py``).

Follows
  src/sgfevector.jl:43-69         set_sample!: u(y) = sum_k H_k(y) U[:, k]
  src/tensorizedbasis.jl:226-252  set_sample!/evaluate (dims beyond len(y): p_0=1, p_k=0)
  src/sampling_error.jl:84-219    calculate_sampling_error (dimensionwise, energy norm)
  src/modelproblems/poisson_primal.jl:14-35  deterministic_problem
The sample matrix is an input: the reference draws it with Julia's
Random.seed!(123) stream (tensorizedbasis.jl:84-91), which is not restated.
The deterministic operator is assembled as K_0 + sum_m y_m K_m with the same
quadrature as a direct assembly of a(y) (equal up to rounding, since the
bilinear form is linear in a).
"""
import numpy as np
import scipy.sparse.linalg as spla

from .fem import triangle_rule


def sg_evaluate(U, n, TB, y):
    """sgfevector.jl:43-69 (one unknown)."""
    TB.set_sample(list(y))
    out = np.zeros(n)
    for k in range(TB.nmodes):
        r = TB.evaluate(k)
        if r != 0:
            out += r * U[k * n:(k + 1) * n]
    return out


def deterministic_solve(Kdet, bdet, bdofs, y):
    """poisson_primal.jl:14-35 + ExtendableFEM.solve: -div(a(y) grad u) = f,
    homogeneous Dirichlet data on all boundary dofs."""
    K = Kdet[0].copy()
    for m in range(1, len(Kdet)):
        if m - 1 < len(y):
            K = K + y[m - 1] * Kdet[m]
    n = K.shape[0]
    inner = np.setdiff1d(np.arange(n), bdofs)
    u = np.zeros(n)
    Kii = K[inner][:, inner].tocsc()
    u[inner] = spla.spsolve(Kii, bdet[inner])
    return u


_QP_CACHE = {}


def _qp_values(space, pts):
    """Basis values and gradients at reference points per cell: (nc, nq, nd), (nc, nq, nd, 2)
    (they depend on the space and the rule only, so they are kept per pair)."""
    key = (id(space), np.asarray(pts).tobytes())
    hit = _QP_CACHE.get(key)
    if hit is not None and hit[0] is space:
        return hit[1]
    out = _qp_values_uncached(space, pts)
    _QP_CACHE[key] = (space, out)
    return out


def _qp_values_uncached(space, pts):
    nc = space.mesh.ncells
    nd = space.ndofs4cell()
    V = np.zeros((nc, len(pts), nd))
    Gr = np.zeros((nc, len(pts), nd, 2))
    for c in range(nc):
        _, _, gl = space.cell_geometry(c)
        for q, (xi, eta) in enumerate(pts):
            lam = np.array([1 - xi - eta, xi, eta])
            v, g, _ = space.local_basis(lam, gl)
            V[c, q] = v
            Gr[c, q] = g
    return V, Gr


def error_integrals(space_det, u_det, space_sg, u_sg, quadorder):
    """sampling_error.jl:2-44 kernels integrated over all cells:
    (sum_T int |grad(u_det - u_sg)|^2, sum_T int (u_det - u_sg)^2)."""
    pts, wts = triangle_rule(quadorder)
    Vd, Gd = _qp_values(space_det, pts)
    Vs, Gs = _qp_values(space_sg, pts)
    vol = space_det.mesh.cell_volumes
    ud = u_det[space_det.celldofs]
    us = u_sg[space_sg.celldofs]
    e = np.einsum("cqd,cd->cq", Vd, ud) - np.einsum("cqd,cd->cq", Vs, us)
    ge = np.einsum("cqdk,cd->cqk", Gd, ud) - np.einsum("cqdk,cd->cqk", Gs, us)
    h1 = np.sum(vol[:, None] * wts[None, :] * np.sum(ge ** 2, axis=2))
    l2 = np.sum(vol[:, None] * wts[None, :] * e ** 2)
    return h1, l2


def calculate_sampling_error(U, TB, space_sg, space_det, Kdet, bdet, samples, weights,
                             order, dimensionwise_error=True):
    """sampling_error.jl:84-219 with the sample matrix and weights given.

    samples: (Msamples, S).  Returns the four (M+1) arrays
    (stress_weighted, u_weighted, stress_uniform, u_uniform).
    """
    M = TB.maxlength_multiindices()
    S = samples.shape[1]
    n = space_sg.ndofs
    errH1 = np.zeros((M + 1, S))
    errL2 = np.zeros((M + 1, S))
    M0 = 0 if dimensionwise_error else M
    for s in range(S):
        y = samples[:, s]
        ud = deterministic_solve(Kdet, bdet, space_det.bdofs, y)
        for m in range(M0, M + 1):
            us = sg_evaluate(U, n, TB, y[:m])
            h1, l2 = error_integrals(space_det, ud, space_sg, us, 2 * order)
            errH1[m, s] = h1
            errL2[m, s] = l2
    wsum = np.sum(weights)
    return (errH1 @ weights / wsum, errL2 @ weights / wsum, errH1.sum(axis=1) / S, errL2.sum(axis=1) / S)
