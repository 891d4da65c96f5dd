"""SGFEVector: the stochastic-Galerkin coefficient vector (host side).

Mirrors src/sgfevector.jl of ExtendableASGFEM.jl (one unknown): ``entries``
is a flat Float64 vector holding the column-major n x P block matrix, mode mu
at entries[mu*n:(mu+1)*n] (sgfevector.jl:86-106).  ``set_sample`` evaluates
sum_k H_k(y) U[:, k] (sgfevector.jl:43-69) on the GPU: the batched evaluation
``evaluate_samples`` (sampling_error.py, sgfem_evaluate_samples) with one
sample, on a light context the vector keeps for later samples.
"""
import numpy as np


class SGFEVector:
    def __init__(self, FES, TB, active_modes=None):
        self.FES_space = [FES]
        self.TB = TB
        self.active_modes = list(range(TB.nmodes)) if active_modes is None else list(active_modes)
        n = FES.ndofs
        P = len(self.active_modes)
        self.length4modes = [k * n for k in range(P + 1)]
        self.entries = np.zeros(n * P)
        self.last_sample = np.zeros(TB.maxlength_multiindices())
        self.FEV = np.zeros(n)
        self._eval_ctx = None  # device context of set_sample (created at the first call)

    @property
    def ndofs(self):
        return self.FES_space[0].ndofs

    def num_multiindices(self):
        return len(self.active_modes)

    def __len__(self):
        return len(self.entries)

    def __getitem__(self, i):
        """View of mode i (0-based)."""
        n = self.ndofs
        return self.entries[i * n:(i + 1) * n]

    def modes(self):
        """n x P column view of the entries."""
        return self.entries.reshape(self.num_multiindices(), self.ndofs).T

    def set_sample(self, S, device=0):
        """set_sample!(SolutionSGFEM, S) (sgfevector.jl:43-69): keeps S, sets the
        basis sample (tensorizedbasis.jl:226-252; dimensions beyond len(S) take
        p_0 = 1, p_k = 0) and evaluates FEV = sum_k H_k(S) U[:, k] on the GPU."""
        from .sampling_error import _light_samples_context, evaluate_samples
        S = np.asarray(S, dtype=np.float64).ravel()
        self.last_sample[:] = 0.0
        k = min(len(S), len(self.last_sample))
        self.last_sample[:k] = S[:k]
        x = S[:len(self.TB.vals)]
        self.TB.set_sample(x, normalize=True)
        if self._eval_ctx is None:
            self._eval_ctx = _light_samples_context(self.FES_space[0], device)
        self.FEV[:] = evaluate_samples(self, x[:, None], m=len(x), ctx=self._eval_ctx)[:, 0]
        return self.FEV

    def norms(self, p=2):
        return np.array([np.linalg.norm(self[j], p) for j in range(self.num_multiindices())])
