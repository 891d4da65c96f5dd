"""Tensorised orthonormal basis and its coupling tensor G (host side).

Mirrors src/tensorizedbasis.jl of ExtendableASGFEM.jl:
  TensorizedBasis                  :28-34, ctor :165-181
  G (get_tensor_multiplication_with_ym)  :193-218, stored as the sparse
      (M*P) x P matrix G[(m-1)P + j, k] = <y_m H_j H_k>, nonzero only for
      k = j +/- e_m with values 1/b' and c'/b' of the normalised recurrence
  set_sample / evaluate            :226-252
  sample_distribution              :84-91 (the sample matrix is drawn with
      NumPy here; Julia's Random.seed!(123) stream is not reproduced)
"""
import numpy as np
import scipy.sparse as sp

from .mopcontrol import generate_multiindices
from .orthopolys import ONBasis


class TensorizedBasis:
    def __init__(self, basis, M, order, maxorder, maxquadorder=None, multi_indices="full"):
        assert order <= maxorder
        self.basis = basis
        self.ONB = ONBasis(basis, maxorder, maxquadorder if maxquadorder is not None else 2 * maxorder)
        self.vals = [np.zeros(maxorder + 1) for _ in range(M)]
        if isinstance(multi_indices, str) and multi_indices == "full":
            multi_indices = generate_multiindices(M, order)
        self.multi_indices = [list(mi) for mi in multi_indices]
        self.nmodes = len(self.multi_indices)
        self.G = coupling_matrix(basis, self.multi_indices)

    def maxlength_multiindices(self):
        return max(len(mi) for mi in self.multi_indices)

    def num_multiindices(self):
        return self.nmodes

    def get_coupling_coefficient(self, m, j, k):
        """<y_m H_j H_k>, m 1-based, j, k 0-based."""
        return self.G[(m - 1) * self.nmodes + j, k]

    def triple_product(self, j, k, l, normalize=True):
        val = 1.0
        for d in range(self.maxlength_multiindices()):
            val *= self.ONB.triple_product(self.multi_indices[j][d], self.multi_indices[k][d],
                                           self.multi_indices[l][d], normalize=normalize)
        return val

    def set_sample(self, x, normalize=True):
        for j in range(len(x)):
            self.vals[j] = self.ONB.evaluate(x[j], normalize=normalize)
        for j in range(len(x), len(self.vals)):
            v = np.zeros(len(self.vals[j]))
            v[0] = 1.0
            self.vals[j] = v
        return self.vals

    def evaluate(self, j):
        prod = 1.0
        for m, k in enumerate(self.multi_indices[j]):
            prod *= self.vals[m][k]
        return prod

    def sample_distribution(self, nsamples, M=None, Mweights=None, seed=123):
        M = self.maxlength_multiindices() if M is None else M
        Mweights = M if Mweights is None else Mweights
        rng = np.random.default_rng(seed)
        if self.basis.name == "legendre":
            S = rng.uniform(-1.0, 1.0, size=(M, nsamples))
        else:
            S = rng.standard_normal(size=(M, nsamples))
        w = np.prod(self.basis.pdf(S[:Mweights]), axis=0)
        return S, w


def coupling_matrix(basis, multi_indices):
    """Sparse (M*P) x P coupling matrix in CSC form."""
    M = max(len(mi) for mi in multi_indices)
    P = len(multi_indices)
    index = {tuple(mi): k for k, mi in enumerate(multi_indices)}
    rows, cols, vals = [], [], []
    for j, mi in enumerate(multi_indices):
        for m in range(M):
            up, down = basis.coupling(mi[m])
            mu = list(mi)
            mu[m] += 1
            k = index.get(tuple(mu))
            if k is not None:
                rows.append(m * P + j)
                cols.append(k)
                vals.append(up)
            if mi[m] > 0:
                mu = list(mi)
                mu[m] -= 1
                k = index.get(tuple(mu))
                if k is not None:
                    rows.append(m * P + j)
                    cols.append(k)
                    vals.append(down)
    return sp.csc_matrix((vals, (rows, cols)), shape=(M * P, P))
