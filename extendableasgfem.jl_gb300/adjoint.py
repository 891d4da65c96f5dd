"""Adjoint gradient of a mean quantity of interest (host side of K6).

No counterpart in the reference package: this differentiates its
PoissonProblemPrimal SG solve (src/modelproblems/poisson_primal.jl:38-81,
solvers_poisson_primal.jl:86-169).  With the parametrised operator
  S(theta, alpha) = I (x) K_0(alpha) + sum_m theta_m G_m (x) K_m,
K_0(alpha) = (a_0 grad u, grad v) for the nodal P1 mean field a_0 = sum_i alpha_i phi_i
(alpha = 1 reproduces a_0 = 1) and K_m the KLE blocks, the quantity of interest is
  J(theta, alpha) = int_box E[u] dx = l . U_0,   S U = e_1 (x) (f, v).
The gradient needs one adjoint solve S Lambda = e_1 (x) l (S is symmetric, the
same device PCG) and two device contractions (sgfem_adjoint_gradient):
  dJ/dtheta_m = -Lambda^T (G_m (x) K_m) U,   dJ/dalpha_i = -sum_mu Lambda_mu^T K_0^(i) U_mu.
``MeanQoI.rrule`` returns (J, pullback) like ChainRulesCore.rrule;
``MeanQoIFunction`` wraps the same as a torch.autograd.Function.
"""
import ctypes

import numpy as np

from . import _lib
from .estimate import _Mesh
from .fem import assemble_rhs_gpu, assemble_stiffness_gpu, assemble_stiffness_nodal_mean, box_functional
from .modelproblems import SGOperator


class MeanQoI:
    def __init__(self, FES, TB, C, rhs, box=(0.25, 0.75, 0.25, 0.75), bonus_quadorder_a=2, bonus_quadorder_f=0,
                 device=0):
        if FES.order != 1:
            raise NotImplementedError("the mean-field gradient is defined for the P1 space")
        self.FES, self.TB, self.C, self.device = FES, TB, C, device
        self.M = TB.maxlength_multiindices()
        self.n = FES.ndofs
        p = FES.order
        self.quadorder_a = 2 * (p - 1) + bonus_quadorder_a
        self.Km = assemble_stiffness_gpu(FES, C, list(range(1, self.M + 1)), self.quadorder_a, device=device)
        self.b0 = assemble_rhs_gpu(FES, rhs, p + bonus_quadorder_f, device=device)
        self.l = box_functional(FES, box)
        mesh = FES.mesh
        self._coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
        self._cells = np.ascontiguousarray(mesh.cells + 1, dtype=np.int64)
        self._vol = np.ascontiguousarray(mesh.cell_volumes, dtype=np.float64)
        self._mesh = _Mesh(1, mesh.nnodes, mesh.ncells, mesh.nfaces, self._coords.ctypes.data,
                           self._cells.ctypes.data, self._cells.ctypes.data, None, None, None,
                           self._vol.ctypes.data, None)

    def operator(self, theta, alpha):
        theta = np.asarray(theta, dtype=np.float64)
        if theta.shape != (self.M,):
            raise ValueError(f"theta needs {self.M} values")
        K0 = assemble_stiffness_nodal_mean(self.FES, alpha, self.quadorder_a)
        return SGOperator(self.FES, self.TB, [K0] + [t * K for t, K in zip(theta, self.Km)], device=self.device)

    def _solve(self, op, rhs, rtol, precision):
        x = np.zeros(self.n * op.P)
        st = op.solve_primal(rhs, x, rtol=rtol, precision=precision, reference_rhs=False)
        return x, st

    def value(self, theta, alpha, rtol=1e-12, precision=_lib.FP64):
        op = self.operator(theta, alpha)
        try:
            U, _ = self._solve(op, self.b0, rtol, precision)
        finally:
            op.close()
        return float(self.l @ U[:self.n])

    def value_and_gradient(self, theta, alpha, rtol=1e-12, precision=_lib.FP64):
        """(J, dJ/dtheta, dJ/dalpha, stats); theta_m must be nonzero (the context
        holds theta_m K_m and the contraction gives theta_m dJ/dtheta_m)."""
        theta = np.asarray(theta, dtype=np.float64)
        if np.any(theta == 0.0):
            raise ValueError("theta_m = 0: the block is absent from the operator")
        op = self.operator(theta, alpha)
        try:
            U, st_f = self._solve(op, self.b0, rtol, precision)
            Lam, st_a = self._solve(op, self.l, rtol, precision)
            dblocks = np.zeros(self.M)
            dalpha = np.zeros(self.FES.mesh.nnodes)
            lib = _lib.load()
            op.ctx._check(lib.sgfem_adjoint_gradient(op.ctx.h, _lib._dp(np.ascontiguousarray(U)),
                                                     _lib._dp(np.ascontiguousarray(Lam)), _lib._dp(dblocks),
                                                     ctypes.byref(self._mesh), _lib._dp(dalpha)))
        finally:
            op.close()
        J = float(self.l @ U[:self.n])
        stats = {"forward": st_f, "adjoint": st_a}
        return J, dblocks / theta, dalpha, stats

    def rrule(self, theta, alpha, **kw):
        """(J, pullback): pullback(dJ) -> (dJ * dJ/dtheta, dJ * dJ/dalpha)."""
        J, gt, ga, _ = self.value_and_gradient(theta, alpha, **kw)
        return J, (lambda dJ: (dJ * gt, dJ * ga))


def _torch_function():
    import torch

    class MeanQoIFunction(torch.autograd.Function):
        """J = MeanQoIFunction.apply(theta, alpha, qoi): float64 tensors, CPU."""

        @staticmethod
        def forward(fctx, theta, alpha, qoi):
            J, gt, ga, _ = qoi.value_and_gradient(theta.detach().cpu().numpy(), alpha.detach().cpu().numpy())
            fctx.save_for_backward(torch.from_numpy(gt), torch.from_numpy(ga))
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(fctx, gJ):
            gt, ga = fctx.saved_tensors
            return gJ * gt, gJ * ga, None

    return MeanQoIFunction


def __getattr__(name):
    if name == "MeanQoIFunction":
        return _torch_function()
    raise AttributeError(name)
