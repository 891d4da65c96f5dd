"""Orthogonal polynomials and the one-dimensional orthonormal basis (host side).

Mirrors src/orthogonal_polynomials/*.jl and src/onbasis.jl of ExtendableASGFEM.jl:
  recurrence_coefficients   Hermite_normal.jl:20-21, Legendre_uniform.jl:20-21
  norms                     Hermite_normal.jl:32, Legendre_uniform.jl:32
  evaluate                  orthogonal_polynomials.jl:63-133
  gauss_rule                orthogonal_polynomials.jl:162-192 (Golub-Welsch)
  normalise_recurrence_coefficients  orthogonal_polynomials.jl:211-221
  ONBasis                   onbasis.jl:13-207
"""
import math

import numpy as np


class HermitePolynomials:
    """Orthogonal w.r.t. the standard normal distribution (Hermite_normal.jl)."""
    name = "hermite"

    @staticmethod
    def recurrence_coefficients(k):
        return 0.0, 1.0, float(k)

    @staticmethod
    def norms(k):
        return math.sqrt(math.factorial(k))

    @staticmethod
    def coupling(k):
        """(G[j, j+e_m], G[j, j-e_m]) for mu_j[m] = k: 1/b', c'/b' of the
        normalised recurrence; the reference evaluates them in BigFloat."""
        return math.sqrt(k + 1), math.sqrt(k)

    @staticmethod
    def pdf(y):
        return np.exp(-0.5 * np.asarray(y) ** 2) / math.sqrt(2 * math.pi)


class LegendrePolynomials:
    """Orthogonal w.r.t. the uniform distribution on [-1, 1] (Legendre_uniform.jl)."""
    name = "legendre"

    @staticmethod
    def recurrence_coefficients(k):
        return 0.0, (2 * k + 1) / (k + 1), k / (k + 1)

    @staticmethod
    def norms(k):
        return math.sqrt(2.0 / (2 * k + 1))

    @staticmethod
    def coupling(k):
        # Float64 evaluation order of normalise_recurrence_coefficients: (b*h1)/h2, (c*h0)/h2
        _, b, c = LegendrePolynomials.recurrence_coefficients(k)
        h2 = LegendrePolynomials.norms(k + 1)
        h1 = LegendrePolynomials.norms(k)
        h0 = LegendrePolynomials.norms(k - 1) if k > 0 else 0.0
        bp = b * h1 / h2
        cp = c * h0 / h2
        return 1.0 / bp, cp / bp

    @staticmethod
    def pdf(y):
        y = np.asarray(y)
        return np.where(np.abs(y) <= 1.0, 0.5, 0.0)


def evaluate(basis, n, x):
    """p_0..p_n at x (scalar or array); returns shape x.shape + (n+1,)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.ones(x.shape + (n + 1,))
    for k in range(n):
        a, b, c = basis.recurrence_coefficients(k)
        y[..., k + 1] = (a + b * x) * y[..., k]
        if k > 0:
            y[..., k + 1] -= c * y[..., k - 1]
    return y


def gauss_rule(basis, n):
    """n-point Gauss rule of the basis' weight, weights summing to one."""
    alpha = np.zeros(n)
    beta = np.zeros(max(n - 1, 0))
    rc = [basis.recurrence_coefficients(k) for k in range(n)]
    for k in range(n):
        alpha[k] = -rc[k][0] / rc[k][1]
    for k in range(1, n):
        beta[k - 1] = rc[k][2] / (rc[k - 1][1] * rc[k][1])
    J = np.diag(alpha)
    if n > 1:
        J += np.diag(np.sqrt(beta), 1) + np.diag(np.sqrt(beta), -1)
    x, V = np.linalg.eigh(J)
    w = V[0, :] ** 2
    return x, w / w.sum()


class ONBasis:
    """One-dimensional orthonormal basis (onbasis.jl:13-18, :89-105)."""

    def __init__(self, basis, maxorder, maxquadorder=None):
        self.basis = basis
        self.maxorder = maxorder
        qp, qw = gauss_rule(basis, maxquadorder if maxquadorder is not None else 2 * maxorder)
        self.gauss_rule = (qp, qw)
        self.vals4xref = evaluate(basis, maxorder, qp)
        self.norms = np.sqrt((self.vals4xref ** 2 * qw[:, None]).sum(axis=0))

    def norm4poly(self, p):
        return self.norms[p]

    def evaluate(self, x, normalize=True):
        v = evaluate(self.basis, self.maxorder, x)
        return v / self.norms if normalize else v

    def integral(self, j, normalize=True):
        v = float(self.vals4xref[:, j] @ self.gauss_rule[1])
        return v / self.norms[j] if normalize else v

    def scalar_product(self, j, k, normalize=True):
        v = float((self.vals4xref[:, j] * self.vals4xref[:, k]) @ self.gauss_rule[1])
        return v / (self.norms[j] * self.norms[k]) if normalize else v

    def triple_product(self, j, k, l, normalize=True):
        v = float((self.vals4xref[:, j] * self.vals4xref[:, k] * self.vals4xref[:, l]) @ self.gauss_rule[1])
        return v / (self.norms[j] * self.norms[k] * self.norms[l]) if normalize else v
