"""Model problems and the GPU stochastic-Galerkin solve (host side).

Mirrors src/modelproblems/ of ExtendableASGFEM.jl:
  AbstractModelProblem / solve        modelproblems.jl:1-31
  PoissonProblemPrimal / solve        poisson_primal.jl:38-81: assemble K_0..K_M
                                      (M = maxlength_multiindices(TB)) and b = (f, v),
                                      then solve_primal!
  SGOperator                          solvers_poisson_primal.jl:14-124 (MySystemPrimal
                                      + MyPreconditionerPrimal), backed by one libsgfem
                                      context on the GPU: mul / ldiv / solve_primal
  LogTransformedPoissonProblemPrimal  logpoisson_primal.jl:85-153: A = (grad u, grad v),
                                      N_m = -(grad a_m . grad u, v), b_mu = (lambda_mu f, v);
                                      MySystemLogPrimal (solvers_logpoisson_primal.jl:14-127)
                                      is the same SGOperator with K_0 = A, K_m = N_m, solved
                                      by solve_logpoisson (device GMRES)
All arithmetic of mul!, ldiv! and the Krylov solve runs in the CUDA library;
this module only assembles the spatial blocks (the caller's side of the
boundary, ExtendableFEM in the reference) and moves arrays across the C ABI.
"""
import numpy as np

from . import _lib
from .fem import (assemble_convection, assemble_laplacian, assemble_pce_rhs, assemble_rhs, assemble_stiffness,
                  assemble_stiffness_gpu, assemble_rhs_gpu, assemble_pce_rhs_gpu, assemble_laplacian_gpu,
                  assemble_convection_gpu)


class AbstractModelProblem:
    pass


class PoissonProblemPrimal(AbstractModelProblem):
    """-div(a(y, x) grad u) = f with the affine coefficient a = a_0 + sum_m y_m a_m."""


class LogTransformedPoissonProblemPrimal(AbstractModelProblem):
    """-div(exp(a) grad u) = f, solved in the transformed form
    -Laplace u - grad a . grad u = exp(-a) f (logpoisson_primal.jl:1-13), a = sum_m y_m a_m."""


class SGOperator:
    """The SG operator S and the mean-based preconditioner on one GPU."""

    def __init__(self, FES, TB, Ks, device=0):
        self.FES = FES
        self.TB = TB
        self.n = FES.ndofs
        self.P = TB.nmodes
        self.M = len(Ks) - 1
        if TB.G.shape != (self.M * self.P, self.P):
            raise ValueError("G must be (M*P) x P with M = len(Ks) - 1")
        self.ctx = _lib.Context(device)
        for m, K in enumerate(Ks):
            self.ctx.set_spatial_matrix(m, K)
        self.ctx.set_coupling(TB.G, self.P, self.M)
        self.bdofs = np.asarray(FES.bdofs, dtype=np.int64)
        self.ctx.set_boundary_dofs(self.bdofs)
        self.ctx.set_dof_coordinates(FES.dof_coords)
        self.ctx.finalize()

    @property
    def has_lattice(self):
        return self.ctx.has_lattice

    @property
    def mean_preconditioner(self):
        """The exact mean-based preconditioner (the reference's LU(K_0) solve): the
        sine-transform form on power-of-two dof lattices, the sparse Cholesky of K_0
        on every other mesh."""
        return _lib.PREC_LATTICE if self.has_lattice else _lib.PREC_CHOLESKY

    def update_basis(self, TB):
        """The adaptive loop appended modes: switch to the TensorizedBasis TB (same
        spatial blocks; TB's multi-index length may not exceed len(Ks) - 1).  The
        K_m, the dof numbering and the lattice preconditioner stay on the GPU."""
        M = TB.maxlength_multiindices()
        if M > self.M:
            raise ValueError("update_basis: TB needs more KLE terms than this operator holds")
        G = TB.G
        if G.shape != (M * TB.nmodes, TB.nmodes):
            raise ValueError("G must be (M*P) x P")
        self.ctx.update_coupling(G, TB.nmodes, M)
        self.TB = TB
        self.P = TB.nmodes

    def mul(self, x, precision=_lib.FP64):
        """mul!(Ax, S, x) on SGFEVector.entries."""
        return self.ctx.apply(x, precision)

    def ldiv(self, b, kind=None, precision=_lib.FP64):
        """ldiv!(y, P, b): mean-based preconditioner on every mode."""
        if kind is None:
            kind = self.mean_preconditioner
        return self.ctx.precondition(b, kind, precision)

    def solve_primal(self, b0, x, rtol=1e-12, precision=_lib.MIXED, preconditioner=None, maxit=5000,
                     inner_rtol=1e-4, reference_rhs=True, check_every=4, allow_maxit=False):
        """solve_primal!: x (SGFEVector.entries) is the warm start and receives the solution."""
        if preconditioner is None:
            preconditioner = self.mean_preconditioner
        o = self.ctx.default_options(precision=precision, preconditioner=preconditioner, rtol=rtol, maxit=maxit,
                                     inner_rtol=inner_rtol, reference_rhs=1 if reference_rhs else 0,
                                     check_every=check_every)
        return self.ctx.solve(b0, x, o, allow_maxit=allow_maxit).as_dict()

    def solve_logpoisson(self, b_full, x, rtol=1e-12, precision=_lib.FP64, preconditioner=None, maxit=5000,
                         inner_rtol=1e-5, reference_rhs=True, restart=20, allow_maxit=False):
        """solve_logpoisson_primal!: GMRES for the non-symmetric operator; b_full holds
        the n x P right-hand side blocks, x the warm start (receives the solution)."""
        if preconditioner is None:
            preconditioner = self.mean_preconditioner
        o = self.ctx.default_options(precision=precision, preconditioner=preconditioner, rtol=rtol, maxit=maxit,
                                     inner_rtol=inner_rtol, reference_rhs=1 if reference_rhs else 0)
        return self.ctx.solve_gmres(b_full, x, o, restart=restart, allow_maxit=allow_maxit).as_dict()

    def close(self):
        self.ctx.close()


def assemble(problem, sol, C, rhs, bonus_quadorder_a=2, bonus_quadorder_f=0, device=None):
    """Spatial blocks: poisson_primal.jl:55-68 ([K_0..K_M], b = (f, v)) or
    logpoisson_primal.jl:97-131 ([A, N_1..N_M], b_mu = (lambda_mu f, v) for all modes).
    device=k assembles on GPU k: the K_m (sgfem_assemble_stiffness), b (sgfem_assemble_rhs),
    and A, N_m, b_mu of the lognormal problem (sgfem_assemble_stiffness with a = 1,
    sgfem_assemble_convection, sgfem_assemble_pce_rhs)."""
    if problem is not PoissonProblemPrimal and problem is not LogTransformedPoissonProblemPrimal:
        raise NotImplementedError(f"no assembly for {problem}")
    if rhs is None:
        raise ValueError("need right-hand side")
    FES = sol.FES_space[0]
    p = FES.order
    M = sol.TB.maxlength_multiindices()
    if problem is LogTransformedPoissonProblemPrimal:
        mis = [sol.TB.multi_indices[k] for k in sol.active_modes]
        qa = p + (p - 1) + bonus_quadorder_a
        if device is None:
            A = assemble_laplacian(FES)
            Ns = assemble_convection(FES, C, list(range(1, M + 1)), qa)
            b = assemble_pce_rhs(FES, C, mis, rhs, p + bonus_quadorder_f)
        else:
            A = assemble_laplacian_gpu(FES, device=device)
            Ns = assemble_convection_gpu(FES, C, list(range(1, M + 1)), qa, device=device)
            b = assemble_pce_rhs_gpu(FES, C, mis, rhs, p + bonus_quadorder_f, device=device)
        return [A] + Ns, b
    if device is None:
        Ks = assemble_stiffness(FES, C, list(range(M + 1)), 2 * (p - 1) + bonus_quadorder_a)
    else:
        Ks = assemble_stiffness_gpu(FES, C, list(range(M + 1)), 2 * (p - 1) + bonus_quadorder_a, device=device)
    if device is None:
        b0 = assemble_rhs(FES, rhs, p + bonus_quadorder_f)
    else:
        b0 = assemble_rhs_gpu(FES, rhs, p + bonus_quadorder_f, device=device)
    return Ks, b0


def solve(problem, sol, C, rhs=None, bonus_quadorder_a=2, bonus_quadorder_f=0, use_iterative_solver=True,
          device=0, **solver_kwargs):
    """solve!(problem, sol, C; rhs, ...): assembles (poisson_primal.jl:55-68) and
    solves on GPU ``device``, writes sol.entries, returns the (0-based) boundary
    dofs like the reference returns bdofs.
    ``solver_kwargs`` go to SGOperator.solve_primal (rtol, precision, ...)."""
    if not issubclass(problem, AbstractModelProblem) or problem is AbstractModelProblem:
        raise NotImplementedError("This model problem seems to have no solver implemented!")
    if not use_iterative_solver:
        raise NotImplementedError("the GPU path has no assembled Kronecker solver; use_iterative_solver=True")
    Ks, b0 = assemble(problem, sol, C, rhs, bonus_quadorder_a, bonus_quadorder_f, device=device)
    op = SGOperator(sol.FES_space[0], sol.TB, Ks, device=device)
    try:
        if problem is LogTransformedPoissonProblemPrimal:
            stats = op.solve_logpoisson(b0, sol.entries, **solver_kwargs)
        else:
            stats = op.solve_primal(b0, sol.entries, **solver_kwargs)
    finally:
        op.close()
    sol.solve_stats = stats
    return op.bdofs
