"""Sampling error and the evaluation of SG solutions at samples (host side of K5).

Mirrors src/sampling_error.jl:84-219 (calculate_sampling_error) and
src/sgfevector.jl:43-69 (set_sample!) of ExtendableASGFEM.jl:
  SampleProblems            deterministic_problem + ExtendableFEM.solve for a
                            batch of samples (poisson_primal.jl:14-35,
                            sampling_error.jl:118-128): one block-diagonal
                            operator K_0 + sum_m y_{s,m} K_m on the GPU, solved
                            by the device PCG, every sample to rtol.
  evaluate_samples          set_sample!(sol, y_s[1:m]) for a batch of samples:
                            U Psi on the GPU (sgfem_evaluate_samples).
  calculate_sampling_error  the reference driver: samples and pdf weights
                            (sample_distribution, tensorizedbasis.jl:84-91),
                            batched deterministic solves, and the error
                            integrals for the truncations m = 0..M on the GPU
                            (sgfem_sampling_error); the weighted and uniform
                            means are formed here in sample order.
"""
import ctypes

import numpy as np

from . import _lib
from .estimate import _Mesh, _Quad
from .fem import H1Pk, assemble_rhs_gpu, assemble_stiffness_gpu, triangle_rule
from .modelproblems import PoissonProblemPrimal


class _SGBasis(ctypes.Structure):
    _fields_ = [("P", ctypes.c_int64), ("M", ctypes.c_int64), ("multi_indices", ctypes.c_void_p),
                ("maxorder", ctypes.c_int32), ("recurrence", ctypes.c_void_p), ("norms", ctypes.c_void_p)]


class _FESpace(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("ndofs", ctypes.c_int64), ("cell_dofs", ctypes.c_void_p)]


def _basis_struct(TB, modes):
    """sgfem_sg_basis of the given modes of TB; returns (struct, arrays kept alive)."""
    M = TB.maxlength_multiindices()
    P = len(modes)
    mi = np.zeros((P, M), dtype=np.int32)
    for j, k in enumerate(modes):
        v = TB.multi_indices[k]
        mi[j, :len(v)] = v
    maxorder = int(mi.max()) if mi.size else 0
    rec = np.ascontiguousarray(np.array([TB.basis.recurrence_coefficients(k) for k in range(maxorder)],
                                        dtype=np.float64).reshape(maxorder, 3))
    norms = np.ascontiguousarray(TB.ONB.norms[:maxorder + 1], dtype=np.float64)
    if len(norms) < maxorder + 1:
        raise ValueError("ONBasis maxorder below the multi-index degree")
    keep = (mi, rec, norms)
    b = _SGBasis(P, M, mi.ctypes.data, maxorder, rec.ctypes.data if maxorder else None, norms.ctypes.data)
    return b, keep


def evaluate_samples(sol, samples, m=None, device=0, ctx=None):
    """set_sample!(sol, y_s[1:m]) for every column y_s of samples (Ms x S):
    the n x S matrix of SG solution values.  m defaults to min(Ms, M)."""
    samples = np.asarray(samples, dtype=np.float64)
    if samples.ndim == 1:
        samples = samples[:, None]
    Ms, S = samples.shape
    TB = sol.TB
    m = min(Ms, TB.maxlength_multiindices()) if m is None else int(m)
    n = sol.ndofs
    b, keep = _basis_struct(TB, sol.active_modes)
    y = np.ascontiguousarray(samples.T)
    U = np.ascontiguousarray(sol.entries, dtype=np.float64)
    out = np.zeros((S, n))
    own = ctx is None
    if own:
        ctx = _light_samples_context(sol.FES_space[0], device)
    try:
        lib = _lib.load()
        ctx._check(lib.sgfem_evaluate_samples(ctx.h, _lib._dp(U), n, ctypes.byref(b), _lib._dp(y), Ms, S, m,
                                              _lib._dp(out)))
    finally:
        if own:
            ctx.close()
    del keep
    return out.T


def _light_samples_context(FES, device):
    """A finalized context (identity operator, one sample) that carries a device and stream."""
    import scipy.sparse as sp
    ctx = _lib.Context(device)
    ctx.set_spatial_matrix(0, sp.identity(FES.ndofs, format="csr"))
    ctx.set_samples(np.zeros((0, 1)))
    ctx.set_boundary_dofs(FES.bdofs)
    ctx.finalize()
    return ctx


class SampleProblems:
    """S deterministic problems -div(a(y_s) grad u_s) = f on one finite-element space."""

    def __init__(self, FES, Ks, samples, device=0):
        self.FES = FES
        self.n = FES.ndofs
        samples = np.asarray(samples, dtype=np.float64)
        self.M, self.S = samples.shape
        if len(Ks) < self.M + 1:
            raise ValueError("need K_0..K_M for M sample dimensions")
        self.ctx = _lib.Context(device)
        for m in range(self.M + 1):
            self.ctx.set_spatial_matrix(m, Ks[m])
        self.ctx.set_samples(samples)
        self.ctx.set_boundary_dofs(FES.bdofs)
        self.ctx.set_dof_coordinates(FES.dof_coords)
        self.ctx.finalize()

    def set_samples(self, samples):
        """Next batch of the same shape."""
        samples = np.asarray(samples, dtype=np.float64)
        if samples.shape != (self.M, self.S):
            raise ValueError("batch shape differs")
        self.ctx.set_samples(samples)

    def options(self, rtol=1e-10, precision=_lib.MIXED, maxit=5000, check_every=4):
        prec = _lib.PREC_LATTICE if self.ctx.has_lattice else _lib.PREC_CHOLESKY
        return self.ctx.default_options(precision=precision, preconditioner=prec, rtol=rtol, maxit=maxit,
                                        reference_rhs=0, check_every=check_every)

    def solve(self, b0, rtol=1e-10, precision=_lib.MIXED, maxit=5000, check_every=4, keep_on_device=False):
        """Solutions as an (n, S) array (None with keep_on_device: they stay in the
        context for sampling_error)."""
        o = self.options(rtol, precision, maxit, check_every)
        if keep_on_device:
            st = self.ctx.solve_samples(b0, None, o)
            self.stats = st.as_dict()
            return None
        x = np.zeros(self.n * self.S)
        st = self.ctx.solve_samples(b0, x, o)
        self.stats = st.as_dict()
        return x.reshape(self.S, self.n).T

    def sampling_error(self, sol, quadorder, det_solutions=None):
        """Error integrals (errH1, errL2), each (M_sg + 1) x S, of the SG solution
        sol against the solutions of the current samples."""
        V = self.FES
        mesh = V.mesh
        Vs = sol.FES_space[0]
        if Vs.mesh is not mesh and (Vs.mesh.ncells != mesh.ncells or not np.array_equal(Vs.mesh.cells, mesh.cells)):
            raise ValueError("SG and deterministic spaces must live on the same cells")
        TB = sol.TB
        b, keep = _basis_struct(TB, sol.active_modes)
        Msg = TB.maxlength_multiindices()
        pts, wts = triangle_rule(quadorder)
        coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
        cell_nodes = np.ascontiguousarray(mesh.cells + 1, dtype=np.int64)
        ddofs = np.ascontiguousarray(V.celldofs + 1, dtype=np.int64)
        sdofs = np.ascontiguousarray(Vs.celldofs + 1, dtype=np.int64)
        cvol = np.ascontiguousarray(mesh.cell_volumes, dtype=np.float64)
        mstruct = _Mesh(V.order, mesh.nnodes, mesh.ncells, mesh.nfaces, coords.ctypes.data, cell_nodes.ctypes.data,
                        ddofs.ctypes.data, None, None, None, cvol.ctypes.data, None)
        fs = _FESpace(Vs.order, Vs.ndofs, sdofs.ctypes.data)
        xref = np.ascontiguousarray(pts, dtype=np.float64)
        w = np.ascontiguousarray(wts, dtype=np.float64)
        q = _Quad(len(w), xref.ctypes.data, w.ctypes.data, 0, None, None)
        U = np.ascontiguousarray(sol.entries, dtype=np.float64)
        eh = np.zeros((self.S, Msg + 1))
        el = np.zeros((self.S, Msg + 1))
        D = None
        if det_solutions is not None:
            D = np.ascontiguousarray(np.asarray(det_solutions, dtype=np.float64).T)  # (S, n) == n x S column-major
        lib = _lib.load()
        self.ctx._check(lib.sgfem_sampling_error(self.ctx.h, _lib._dp(D) if D is not None else None,
                                                 ctypes.byref(mstruct), ctypes.byref(fs), _lib._dp(U), ctypes.byref(b),
                                                 ctypes.byref(q), _lib._dp(eh), _lib._dp(el)))
        del keep
        return eh.T, el.T

    def close(self):
        self.ctx.close()


def calculate_sampling_error(sol, C, problem=PoissonProblemPrimal, bonus_quadorder_a=10, bonus_quadorder_f=0,
                             order=2, rhs=None, Msamples=None, dimensionwise_error=True, energy_norm=True,
                             nsamples=100, samples=None, weights=None, batch=512, rtol=1e-12,
                             precision=_lib.FP64, device=0, return_per_sample=False):
    """calculate_sampling_error(sol, C; problem, order, rhs, Msamples, nsamples, ...)
    (src/sampling_error.jl:84-219) on the GPU.

    Returns (stress_weighted, u_weighted, stress_uniform, u_uniform), arrays
    of length M+1 (entry m: the SG solution truncated to y[1:m]).  The sample
    matrix (Msamples x nsamples) and pdf weights come from
    sol.TB.sample_distribution unless given.  The deterministic problems are
    solved by the device PCG to rtol (the reference uses a direct solver).
    energy_norm selects nothing here: the reference's two stress components
    are equal for this problem (sampling_error.jl:2-14).
    """
    if problem is not PoissonProblemPrimal:
        raise NotImplementedError(f"sampling error for {problem}")
    if rhs is None:
        raise ValueError("need right-hand side")
    FES = sol.FES_space[0]
    TB = sol.TB
    M = TB.maxlength_multiindices()
    Ms = C.maxm() if Msamples is None else int(Msamples)
    if samples is None:
        samples, w = TB.sample_distribution(nsamples, M=Ms, Mweights=Ms)
        weights = w if weights is None else weights
    samples = np.asarray(samples, dtype=np.float64)
    Ms, S = samples.shape
    if weights is None:
        weights = np.prod(TB.basis.pdf(samples), axis=0)
    weights = np.asarray(weights, dtype=np.float64)
    if Ms < M:
        raise ValueError("Msamples below the multi-index length")
    Vd = H1Pk(FES.mesh, order)
    qa = 2 * (order - 1) + bonus_quadorder_a
    Kd = assemble_stiffness_gpu(Vd, C, list(range(Ms + 1)), qa, device=device)
    bd = assemble_rhs_gpu(Vd, rhs, order + bonus_quadorder_f, device=device)
    B = min(batch, S)
    errH1 = np.zeros((M + 1, S))
    errL2 = np.zeros((M + 1, S))
    sp_ = None
    try:
        for s0 in range(0, S, B):
            cols = np.arange(s0, min(s0 + B, S))
            Y = samples[:, cols]
            if len(cols) < B:  # pad the last batch with copies of its last sample
                Y = np.concatenate([Y, np.repeat(Y[:, -1:], B - len(cols), axis=1)], axis=1)
            if sp_ is None:
                sp_ = SampleProblems(Vd, Kd, Y, device=device)
            else:
                sp_.set_samples(Y)
            sp_.solve(bd, rtol=rtol, precision=precision, keep_on_device=True)
            eh, el = sp_.sampling_error(sol, 2 * order)
            errH1[:, cols] = eh[:, :len(cols)]
            errL2[:, cols] = el[:, :len(cols)]
    finally:
        if sp_ is not None:
            sp_.close()
    if not dimensionwise_error:
        errH1[:M] = 0.0
        errL2[:M] = 0.0
    wsum = np.sum(weights)
    out = (errH1 @ weights / wsum, errL2 @ weights / wsum, errH1.sum(axis=1) / S, errL2.sum(axis=1) / S)
    if return_per_sample:
        return out, (errH1, errL2)
    return out
