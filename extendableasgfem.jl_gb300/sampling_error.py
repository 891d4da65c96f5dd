"""Sampling error (host side of the sample kernels).

Mirrors src/sampling_error.jl:84-219 (calculate_sampling_error) and the
evaluation of an SGFEVector at samples, src/sgfevector.jl:43-69:
  SampleProblems        deterministic_problem + ExtendableFEM.solve for a batch of
                        samples (poisson_primal.jl:14-35, sampling_error.jl:118-128):
                        one block-diagonal operator K_0 + sum_m y_{s,m} K_m on the
                        GPU, solved by the device PCG (mean preconditioner, mixed
                        precision), every sample to rtol.
"""
import numpy as np

from . import _lib


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

    def solve(self, b0, rtol=1e-10, precision=_lib.MIXED, maxit=5000, check_every=8):
        """Solutions as an (n, S) array."""
        prec = _lib.PREC_LATTICE if self.ctx.has_lattice else _lib.PREC_JACOBI
        o = self.ctx.default_options(precision=precision, preconditioner=prec, rtol=rtol, maxit=maxit,
                                     reference_rhs=0, check_every=check_every)
        x = np.zeros(self.n * self.S)
        st = self.ctx.solve_samples(b0, x, o)
        self.stats = st.as_dict()
        return x.reshape(self.S, self.n).T

    def close(self):
        self.ctx.close()
