"""Residual error estimator for PoissonProblemPrimal (host side of K4).

Mirrors estimate(::Type{PoissonProblemPrimal}, sol, C; rhs, bonus_quadorder,
tail_extension) of src/estimate.jl:260-418.  The integer work of the
reference runs here (extended multi-index set, add_boundary_modes,
mopcontrol.jl:60-132; neighbour tables, estimate.jl:1-22; the coupling tensor
of the extended set, tensorizedbasis.jl:193-218) and is reduced to one list
per extended mode j of its couplings to active modes; the per-cell and
per-face arithmetic runs in libsgfem (sgfem_estimate_primal).
Returns (eta4modes, eta4cell, multi_indices_extended) like the reference,
eta4cell with shape (ncells, P_ext).
"""
import copy
import ctypes

import numpy as np
import scipy.sparse as sp

from . import _lib
from .fem import line_rule, triangle_rule
from .modelproblems import LogTransformedPoissonProblemPrimal, PoissonProblemPrimal
from .mopcontrol import add_boundary_modes


class _Mesh(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("nnodes", ctypes.c_int64), ("ncells", ctypes.c_int64),
                ("nfaces", ctypes.c_int64), ("coords", ctypes.c_void_p), ("cell_nodes", ctypes.c_void_p),
                ("cell_dofs", ctypes.c_void_p), ("face_nodes", ctypes.c_void_p), ("face_cells", ctypes.c_void_p),
                ("cell_faces", ctypes.c_void_p), ("cell_volumes", ctypes.c_void_p),
                ("face_volumes", ctypes.c_void_p)]


class _Quad(ctypes.Structure):
    _fields_ = [("nq", ctypes.c_int), ("xref", ctypes.c_void_p), ("w", ctypes.c_void_p), ("nqf", ctypes.c_int),
                ("tref", ctypes.c_void_p), ("wf", ctypes.c_void_p)]


class _Cosine(ctypes.Structure):
    _fields_ = [("maxm", ctypes.c_int), ("mean", ctypes.c_double), ("freq", ctypes.c_double),
                ("decay_factors", ctypes.c_void_p), ("b1", ctypes.c_void_p), ("b2", ctypes.c_void_p)]


class _Interp(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("ndofs", ctypes.c_int64), ("cell_dofs", ctypes.c_void_p),
                ("values", ctypes.c_void_p)]


class _Ext(ctypes.Structure):
    _fields_ = [("P_ext", ctypes.c_int64), ("M_ext", ctypes.c_int64), ("ptr", ctypes.c_void_p),
                ("m", ctypes.c_void_p), ("nu", ctypes.c_void_p), ("g", ctypes.c_void_p)]


def _ptr(a):
    return a.ctypes.data


def extension_couplings(multi_indices, basis, tail_extension=(10, 2)):
    """Extended set and, per extended mode j, its couplings to active modes:
    (0, j, 1) if j is active, (m, nu, G_ext[(m-1)P_ext + j, nu]) for active
    neighbours nu = j +/- e_m (estimate.jl:343-353, :385-393), in that order
    (m ascending, the j + e_m neighbour before j - e_m).  G_ext at a neighbour is
    the up / down value of the one-dimensional coupling at degree ext[j][m-1]
    (the entry coupling_matrix stores); neighbours are found by mixed-radix keys
    (the last of equal multi-indices wins, as in get_neighbours)."""
    nmodes = len(multi_indices)
    ext = add_boundary_modes(copy.deepcopy([list(m) for m in multi_indices]), tail_extension=tail_extension)
    P_ext = len(ext)
    M_ext = len(ext[0])
    A = np.asarray(ext, dtype=np.int64)                    # P_ext x M_ext degrees
    radix = [int(r) + 2 for r in A.max(axis=0)]            # per dimension: a degree + 1 stays below it
    w_py = [1] * M_ext
    for d in range(M_ext - 2, -1, -1):
        w_py[d] = w_py[d + 1] * radix[d + 1]
    exact = w_py[0] * radix[0] < 2 ** 62
    w = np.array(w_py, dtype=np.int64 if exact else object)  # object ints only if int64 would overflow
    keys = (A.astype(object) if not exact else A) @ w
    # last occurrence of each key -> its 1-based index
    order = np.argsort(keys, kind="stable")
    sk = keys[order]
    last = np.r_[sk[1:] != sk[:-1], True]
    uk, ui = sk[last], order[last] + 1
    def lookup(q):
        pos = np.searchsorted(uk, q)
        pos_c = np.minimum(pos, len(uk) - 1)
        hit = (pos < len(uk)) & (uk[pos_c] == q)
        return np.where(hit, ui[pos_c], 0)
    wm = np.asarray(w)[None, :]
    plus = lookup(keys[:, None] + wm)                       # P_ext x M_ext, 1-based, 0: none
    minus = np.where(A > 0, lookup(keys[:, None] - wm), 0)
    maxdeg = int(A.max())
    tab = np.array([basis.coupling(k) for k in range(maxdeg + 1)], dtype=np.float64)  # (up, down) per degree
    up, down = tab[A, 0], tab[A, 1]
    # per mode j: the self term, then for m = 1..M_ext the plus and the minus neighbour
    act_self = np.arange(P_ext) < nmodes
    valid = np.zeros((P_ext, 1 + 2 * M_ext), dtype=bool)
    mcol = np.zeros((P_ext, 1 + 2 * M_ext), dtype=np.int32)
    nucol = np.zeros((P_ext, 1 + 2 * M_ext), dtype=np.int64)
    gcol = np.zeros((P_ext, 1 + 2 * M_ext), dtype=np.float64)
    valid[:, 0] = act_self
    nucol[:, 0] = np.arange(P_ext)
    gcol[:, 0] = 1.0
    mm = np.arange(1, M_ext + 1, dtype=np.int32)[None, :]
    valid[:, 1::2] = (plus > 0) & (plus <= nmodes)
    valid[:, 2::2] = (minus > 0) & (minus <= nmodes)
    mcol[:, 1::2] = mm
    mcol[:, 2::2] = mm
    nucol[:, 1::2] = plus - 1
    nucol[:, 2::2] = minus - 1
    gcol[:, 1::2] = up
    gcol[:, 2::2] = down
    ptr = np.r_[0, np.cumsum(valid.sum(axis=1))].astype(np.int64)
    flat = valid.ravel()
    ms = mcol.ravel()[flat].astype(np.int32)
    nus = nucol.ravel()[flat].astype(np.int32)
    gs = gcol.ravel()[flat].astype(np.float64)
    return ext, (ptr, ms, nus, gs)


def _light_context(FES, TB, device):
    """A context that carries only the dof/mode layout (identity blocks)."""
    n = FES.ndofs
    I = sp.identity(n, format="csr")
    M = TB.maxlength_multiindices()
    ctx = _lib.Context(device)
    for m in range(M + 1):
        ctx.set_spatial_matrix(m, I)
    ctx.set_coupling(TB.G, TB.nmodes, M)
    ctx.set_boundary_dofs(FES.bdofs)
    ctx.set_dof_coordinates(FES.dof_coords)
    ctx.finalize()
    return ctx


def estimate(problem, sol, C, rhs=None, bonus_quadorder=1, tail_extension=(10, 2), face_points=None, device=0,
             op=None):
    """estimate(PoissonProblemPrimal, sol, C; rhs, bonus_quadorder, tail_extension) on the GPU.

    ``op``: an SGOperator of the same space and basis to reuse its context.
    ``face_points``: Gauss points per face for the jump term (default quadorder + 1).
    """
    if problem is LogTransformedPoissonProblemPrimal:
        return _estimate_log(sol, C, rhs, bonus_quadorder, tail_extension, face_points, device, op)
    if problem is not PoissonProblemPrimal:
        raise NotImplementedError(f"no estimator for {problem}")
    if rhs is None:
        raise ValueError("need right-hand side")
    FES = sol.FES_space[0]
    mesh = FES.mesh
    TB = sol.TB
    ext, (ptr, ms, nus, gs) = extension_couplings(TB.multi_indices, TB.basis, tail_extension)
    P_ext, M_ext = len(ext), len(ext[0])
    if C.maxm() < M_ext:
        raise ValueError(f"coefficient maxm = {C.maxm()} < extended length {M_ext}")
    order = FES.order
    quadorder = 2 * (order - 1) + bonus_quadorder
    pts, wts = triangle_rule(quadorder)
    tq, tw = line_rule(face_points if face_points is not None else quadorder + 1)
    X = FES.physical_points(pts)
    fq = np.ascontiguousarray(np.broadcast_to(np.asarray(rhs(X[..., 0], X[..., 1]), dtype=np.float64), X.shape[:2]))

    coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    cell_nodes = np.ascontiguousarray(mesh.cells + 1, dtype=np.int64)
    cell_dofs = np.ascontiguousarray(FES.celldofs + 1, dtype=np.int64)
    face_nodes = np.ascontiguousarray(mesh.face_nodes + 1, dtype=np.int64)
    face_cells = np.ascontiguousarray(np.where(mesh.face_cells >= 0, mesh.face_cells + 1, 0), dtype=np.int64)
    cell_faces = np.ascontiguousarray(mesh.cellfaces + 1, dtype=np.int64)
    cvol = np.ascontiguousarray(mesh.cell_volumes, dtype=np.float64)
    fvol = np.ascontiguousarray(mesh.face_volumes, dtype=np.float64)
    m = _Mesh(order, mesh.nnodes, mesh.ncells, mesh.nfaces, _ptr(coords), _ptr(cell_nodes), _ptr(cell_dofs),
              _ptr(face_nodes), _ptr(face_cells), _ptr(cell_faces), _ptr(cvol), _ptr(fvol))
    xref = np.ascontiguousarray(pts, dtype=np.float64)
    w = np.ascontiguousarray(wts, dtype=np.float64)
    tq = np.ascontiguousarray(tq, dtype=np.float64)
    tw = np.ascontiguousarray(tw, dtype=np.float64)
    q = _Quad(len(w), _ptr(xref), _ptr(w), len(tw), _ptr(tq), _ptr(tw))
    dfac = np.ascontiguousarray(C.decay_factors, dtype=np.float64)
    b1 = np.ascontiguousarray(C.b1, dtype=np.int64)
    b2 = np.ascontiguousarray(C.b2, dtype=np.int64)
    c = _Cosine(C.maxm(), C.mean_value, C.freq, _ptr(dfac), _ptr(b1), _ptr(b2))
    e = _Ext(P_ext, M_ext, _ptr(ptr), _ptr(ms), _ptr(nus), _ptr(gs))
    eta4modes = np.zeros(P_ext)
    eta4cell = np.zeros((P_ext, mesh.ncells))
    ctx = op.ctx if op is not None else _light_context(FES, TB, device)
    try:
        solv = np.ascontiguousarray(sol.entries, dtype=np.float64)
        lib = _lib.load()
        rc = lib.sgfem_estimate_primal(ctx.h, solv.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(m),
                                       ctypes.byref(q), fq.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       ctypes.byref(c), ctypes.byref(e),
                                       eta4modes.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       eta4cell.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        ctx._check(rc)
    finally:
        if op is None:
            ctx.close()
    return eta4modes, eta4cell.T, ext


def _mesh_struct(FES, order=None):
    mesh = FES.mesh
    keep = dict(
        coords=np.ascontiguousarray(mesh.coords, dtype=np.float64),
        cell_nodes=np.ascontiguousarray(mesh.cells + 1, dtype=np.int64),
        cell_dofs=np.ascontiguousarray(FES.celldofs + 1, dtype=np.int64),
        face_nodes=np.ascontiguousarray(mesh.face_nodes + 1, dtype=np.int64),
        face_cells=np.ascontiguousarray(np.where(mesh.face_cells >= 0, mesh.face_cells + 1, 0), dtype=np.int64),
        cell_faces=np.ascontiguousarray(mesh.cellfaces + 1, dtype=np.int64),
        cvol=np.ascontiguousarray(mesh.cell_volumes, dtype=np.float64),
        fvol=np.ascontiguousarray(mesh.face_volumes, dtype=np.float64))
    m = _Mesh(FES.order if order is None else order, mesh.nnodes, mesh.ncells, mesh.nfaces, _ptr(keep["coords"]),
              _ptr(keep["cell_nodes"]), _ptr(keep["cell_dofs"]), _ptr(keep["face_nodes"]), _ptr(keep["face_cells"]),
              _ptr(keep["cell_faces"]), _ptr(keep["cvol"]), _ptr(keep["fvol"]))
    return m, keep


def _estimate_log(sol, C, rhs, bonus_quadorder, tail_extension, face_points, device, op):
    """estimate(LogTransformedPoissonProblemPrimal, sol, C; rhs, bonus_quadorder,
    tail_extension), src/estimate.jl:70-257: (eta4modes, eta4cell, ext, zeta).
    lambda_j is interpolated nodally into the H1Pk space of degree
    quadorder = 2 (order - 1) + bonus_quadorder (1 or 2)."""
    from .fem import H1Pk, pce_lambda
    if rhs is None:
        raise ValueError("need right-hand side")
    if isinstance(tail_extension, (int, np.integer)):
        raise TypeError("tail_extension needs two entries (add_boundary_modes reads tail_extension[2])")
    FES = sol.FES_space[0]
    mesh = FES.mesh
    TB = sol.TB
    ext, (ptr, ms, nus, gs) = extension_couplings(TB.multi_indices, TB.basis, tail_extension)
    P_ext, M_ext = len(ext), len(ext[0])
    if C.maxm() < M_ext:
        raise ValueError(f"coefficient maxm = {C.maxm()} < extended length {M_ext}")
    order = FES.order
    quadorder = 2 * (order - 1) + bonus_quadorder
    if quadorder not in (1, 2):
        raise NotImplementedError("interpolation degree 1 or 2 (2 (order - 1) + bonus_quadorder)")
    pts, wts = triangle_rule(quadorder)
    tq, tw = line_rule(face_points if face_points is not None else order)
    X = FES.physical_points(pts)
    fq = np.ascontiguousarray(np.broadcast_to(np.asarray(rhs(X[..., 0], X[..., 1]), dtype=np.float64), X.shape[:2]))
    Vi = H1Pk(mesh, quadorder)
    lamv = np.ascontiguousarray(pce_lambda(C, ext, Vi.dof_coords[:, 0], Vi.dof_coords[:, 1], factor=-1.0))
    idofs = np.ascontiguousarray(Vi.celldofs + 1, dtype=np.int64)
    interp = _Interp(quadorder, Vi.ndofs, _ptr(idofs), _ptr(lamv))
    m, keep = _mesh_struct(FES)
    xref = np.ascontiguousarray(pts, dtype=np.float64)
    w = np.ascontiguousarray(wts, dtype=np.float64)
    tq = np.ascontiguousarray(tq, dtype=np.float64)
    tw = np.ascontiguousarray(tw, dtype=np.float64)
    q = _Quad(len(w), _ptr(xref), _ptr(w), len(tw), _ptr(tq), _ptr(tw))
    dfac = np.ascontiguousarray(C.decay_factors, dtype=np.float64)
    b1 = np.ascontiguousarray(C.b1, dtype=np.int64)
    b2 = np.ascontiguousarray(C.b2, dtype=np.int64)
    c = _Cosine(C.maxm(), C.mean_value, C.freq, _ptr(dfac), _ptr(b1), _ptr(b2))
    e = _Ext(P_ext, M_ext, _ptr(ptr), _ptr(ms), _ptr(nus), _ptr(gs))
    eta4modes = np.zeros(P_ext)
    eta4cell = np.zeros((P_ext, mesh.ncells))
    zeta = np.zeros(2)
    ctx = op.ctx if op is not None else _light_context(FES, TB, device)
    try:
        solv = np.ascontiguousarray(sol.entries, dtype=np.float64)
        lib = _lib.load()
        dp = lambda a_: a_.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        rc = lib.sgfem_estimate_logpoisson(ctx.h, dp(solv), ctypes.byref(m), ctypes.byref(q), dp(fq),
                                           ctypes.byref(c), ctypes.byref(e), ctypes.byref(interp), dp(eta4modes),
                                           dp(eta4cell), dp(zeta))
        ctx._check(rc)
    finally:
        if op is None:
            ctx.close()
    del keep
    return eta4modes, eta4cell.T, ext, float(zeta[0] - zeta[1])


def estimate_equilibration(problem, sol, C, rhs=None, tail_extension=(10, 2), bonus_quadorder=0, FETypeDual=None,
                           div_penalty=1.0e5, quadorder=None, device=0, op=None):
    """estimate_equilibration(PoissonProblemPrimal, sol, C; rhs, tail_extension)
    (src/estimate.jl:607-954) on the GPU (sgfem_estimate_equilibration): local
    RT_k flux equilibration on every node patch, k the order of the space.
    Returns (eta4modes, eta4cell, multi_indices_extended), eta4cell (ncells, P_ext).
    The cell rule has order 2 (k + 1) like the reference's (``quadorder``
    overrides it); ``bonus_quadorder`` is accepted and unused, as in the reference.
    The reference's default tail_extension = 5 cannot reach add_boundary_modes,
    which reads tail_extension[2]; a pair is required."""
    if problem is not PoissonProblemPrimal:
        raise NotImplementedError(f"no equilibration estimator for {problem}")
    if rhs is None:
        raise ValueError("need right-hand side")
    if FETypeDual is not None:
        raise NotImplementedError("the flux space is RT_k with k the order of the H1Pk space")
    if isinstance(tail_extension, (int, np.integer)):
        raise TypeError("tail_extension needs two entries (add_boundary_modes reads tail_extension[2])")
    FES = sol.FES_space[0]
    mesh = FES.mesh
    TB = sol.TB
    ext, (ptr, ms, nus, gs) = extension_couplings(TB.multi_indices, TB.basis, tail_extension)
    P_ext, M_ext = len(ext), len(ext[0])
    if C.maxm() < M_ext:
        raise ValueError(f"coefficient maxm = {C.maxm()} < extended length {M_ext}")
    pts, wts = triangle_rule(2 * (FES.order + 1) if quadorder is None else quadorder)
    X = FES.physical_points(pts)
    fq = np.ascontiguousarray(np.broadcast_to(np.asarray(rhs(X[..., 0], X[..., 1]), dtype=np.float64), X.shape[:2]))
    m, keep = _mesh_struct(FES)
    xref = np.ascontiguousarray(pts, dtype=np.float64)
    w = np.ascontiguousarray(wts, dtype=np.float64)
    q = _Quad(len(w), _ptr(xref), _ptr(w), 0, None, None)
    dfac = np.ascontiguousarray(C.decay_factors, dtype=np.float64)
    b1 = np.ascontiguousarray(C.b1, dtype=np.int64)
    b2 = np.ascontiguousarray(C.b2, dtype=np.int64)
    c = _Cosine(C.maxm(), C.mean_value, C.freq, _ptr(dfac), _ptr(b1), _ptr(b2))
    e = _Ext(P_ext, M_ext, _ptr(ptr), _ptr(ms), _ptr(nus), _ptr(gs))
    eta4modes = np.zeros(P_ext)
    eta4cell = np.zeros((P_ext, mesh.ncells))
    ctx = op.ctx if op is not None else _light_context(FES, TB, device)
    try:
        solv = np.ascontiguousarray(sol.entries, dtype=np.float64)
        dp = lambda a_: a_.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        rc = _lib.load().sgfem_estimate_equilibration(ctx.h, dp(solv), ctypes.byref(m), ctypes.byref(q), dp(fq),
                                                      ctypes.byref(c), ctypes.byref(e), float(div_penalty),
                                                      dp(eta4modes), dp(eta4cell))
        ctx._check(rc)
    finally:
        if op is None:
            ctx.close()
    del keep
    return eta4modes, eta4cell.T, ext
