"""Oracle restatement of the orthogonal-polynomial layer and the tensorised basis.

Test infrastructure only (see ``oracle/__init__.py``).

Follows
  src/orthogonal_polynomials/orthogonal_polynomials.jl   (evaluate!, gauss_rule,
                                                           normalise_recurrence_coefficients)
  src/orthogonal_polynomials/Hermite_normal.jl:20-39      (Hermite recurrence / norms)
  src/orthogonal_polynomials/Legendre_uniform.jl:20-39    (Legendre recurrence / norms)
  src/onbasis.jl:89-207                                  (ONBasis, products, evaluate)
  src/tensorizedbasis.jl:84-252                          (TensorizedBasis, G, set_sample!, evaluate)
"""
import math
from fractions import Fraction

import numpy as np

HERMITE = "hermite"
LEGENDRE = "legendre"


def recurrence_coefficients(obt, k):
    """(a, b, c) with p_{k+1} = (a + b x) p_k - c p_{k-1}.

    Hermite_normal.jl:20-21 -> (0, 1, k); Legendre_uniform.jl:20-21 ->
    (0, (2k+1)//(k+1), k//(k+1)).  Rationals are kept exact here and rounded
    to float64 where the reference does (Rational * Float64 promotes).
    """
    if obt == HERMITE:
        return Fraction(0), Fraction(1), Fraction(k)
    if obt == LEGENDRE:
        return Fraction(0), Fraction(2 * k + 1, k + 1), Fraction(k, k + 1)
    raise ValueError(obt)


def poly_norm(obt, k):
    """Closed-form norms: Hermite sqrt(k!) (Hermite_normal.jl:32, BigFloat),
    Legendre sqrt(2/(2k+1)) (Legendre_uniform.jl:32, Float64)."""
    if obt == HERMITE:
        return math.sqrt(math.factorial(k))
    return math.sqrt(2.0 / (2 * k + 1))


def evaluate_polys(obt, n, x):
    """Values p_0..p_n at scalar or array x (orthogonal_polynomials.jl:63-73, :96-133)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.ones(x.shape + (n + 1,), dtype=np.float64)
    for k in range(n):
        a, b, c = recurrence_coefficients(obt, k)
        y[..., k + 1] = (float(a) + float(b) * x) * y[..., k]
        if k > 0:
            y[..., k + 1] = y[..., k + 1] - float(c) * y[..., k - 1]
    return y


def rc_array_monic(obt, n):
    """orthogonal_polynomials.jl:30-43 (monic recurrence alpha, beta)."""
    rc = [recurrence_coefficients(obt, k) for k in range(n + 1)]
    a = [-r[0] for r in rc]
    bcoef = [r[2] for r in rc][1:]
    c = [r[1] for r in rc]
    alpha = [float(a[k] / c[k]) for k in range(n + 1)]
    beta = [float(bcoef[k] / (c[k] * c[k + 1])) for k in range(n)]
    return np.array(alpha), np.array(beta)


def gauss_rule(obt, n):
    """Golub-Welsch rule with n points (orthogonal_polynomials.jl:162-192).

    The reference's symmetrisation branch tests ``all(alpha == 0)`` which is
    never true in Julia (vector == scalar is false), so no symmetrisation.
    Weights are normalised to sum 1 (probability measure).
    """
    alpha, beta = rc_array_monic(obt, n - 1)
    J = np.diag(alpha) + np.diag(np.sqrt(beta), 1) + np.diag(np.sqrt(beta), -1)
    x, V = np.linalg.eigh(J)
    w = V[0, :] ** 2
    w = w / np.sum(w)
    return x, w


class ONBasis:
    """onbasis.jl:13-18, ctor :89-105."""

    def __init__(self, obt, maxorder, maxquadorder=None):
        if maxquadorder is None:
            maxquadorder = 2 * maxorder
        self.obt = obt
        self.maxorder = maxorder
        self.qp, self.qw = gauss_rule(obt, maxquadorder)
        self.vals4xref = evaluate_polys(obt, maxorder, self.qp)  # nq x (maxorder+1)
        norms = np.zeros(maxorder + 1)
        for m in range(maxorder + 1):
            for k in range(len(self.qw)):
                norms[m] += self.vals4xref[k, m] ** 2 * self.qw[k]
        self.norms = np.sqrt(norms)

    def norm4poly(self, p):
        return self.norms[p]

    def integral(self, j, normalize=True):
        v = 0.0
        for q in range(len(self.qw)):
            v += self.vals4xref[q, j] * self.qw[q]
        return v / self.norms[j] if normalize else v

    def scalar_product(self, j, k, normalize=True):
        v = 0.0
        for q in range(len(self.qw)):
            v += self.vals4xref[q, j] * self.vals4xref[q, k] * self.qw[q]
        return v / self.norms[j] / self.norms[k] if normalize else v

    def triple_product(self, j, k, l, normalize=True):
        """onbasis.jl:110-127."""
        v = 0.0
        for q in range(len(self.qw)):
            v += self.vals4xref[q, j] * self.vals4xref[q, k] * self.vals4xref[q, l] * self.qw[q]
        if normalize:
            return v / self.norms[j] / self.norms[k] / self.norms[l]
        return v

    def evaluate(self, x, normalize=True):
        """onbasis.jl:201-207."""
        v = evaluate_polys(self.obt, self.maxorder, x)
        return v / self.norms if normalize else v


def normalise_recurrence_coefficients(obt, k):
    """orthogonal_polynomials.jl:211-221, with the reference's float arithmetic.

    Hermite norms are BigFloat in the reference, so the ratios are exact up to
    the final rounding; Legendre norms are Float64 and the products are
    evaluated left to right as ``b * h1 / h2``.
    """
    a, b, c = recurrence_coefficients(obt, k)
    if obt == HERMITE:
        # exact: h1/h2 = 1/sqrt(k+1), h0/h2 = 1/sqrt(k(k+1))
        return None
    h2 = poly_norm(obt, k + 1)
    h1 = poly_norm(obt, k)
    h0 = poly_norm(obt, k - 1) if k > 0 else 0.0
    return (float(a) * h1 / h2, float(b) * h1 / h2, float(c) * h0 / h2)


def coupling_values(obt, n):
    """(G[j, j+e_m], G[j, j-e_m]) for mu_j[m] = n (tensorizedbasis.jl:204-214):
    1/b' and c'/b' of the normalised recurrence."""
    if obt == HERMITE:
        # BigFloat evaluation rounded once: sqrt(n+1), sqrt(n)
        return math.sqrt(n + 1), math.sqrt(n)
    _, bp, cp = normalise_recurrence_coefficients(obt, n)
    return 1.0 / bp, cp / bp


def maxlength(multi_indices):
    return max(len(mi) for mi in multi_indices)


def get_tensor_multiplication_with_ym(obt, multi_indices):
    """G as a dense (M*P) x P array, G[(m-1)P + j, k] (tensorizedbasis.jl:193-218).

    Literal O(P^2 M) search, as in the reference.
    """
    M = maxlength(multi_indices)
    P = len(multi_indices)
    G = np.zeros((M * P, P))
    for j in range(P):
        for m in range(M):
            up, down = coupling_values(obt, multi_indices[j][m])
            mu1 = list(multi_indices[j])
            mu2 = list(multi_indices[j])
            mu1[m] += 1
            mu2[m] -= 1
            for k in range(P):
                if list(multi_indices[k]) == mu1:
                    G[m * P + j, k] = up
                elif list(multi_indices[k]) == mu2:
                    G[m * P + j, k] = down
    return G


class TensorizedBasis:
    """tensorizedbasis.jl:28-34, ctor :165-181."""

    def __init__(self, obt, M, order, maxorder, maxquadorder=None, multi_indices="full"):
        from .mopcontrol import generate_multiindices
        assert order <= maxorder
        self.ONB = ONBasis(obt, maxorder, maxquadorder if maxquadorder is not None else 2 * maxorder)
        self.obt = obt
        self.vals = [np.zeros(maxorder + 1) for _ in range(M)]
        if isinstance(multi_indices, str) and multi_indices == "full":
            multi_indices = generate_multiindices(M, order)
        self.multi_indices = [list(mi) for mi in multi_indices]
        self.nmodes = len(self.multi_indices)
        self.G = get_tensor_multiplication_with_ym(obt, self.multi_indices)

    def maxlength_multiindices(self):
        return maxlength(self.multi_indices)

    def get_coupling_coefficient(self, m, j, k):
        """tensorizedbasis.jl:74 (1-based m, 0-based j, k here)."""
        return self.G[(m - 1) * self.nmodes + j, k]

    def triple_product(self, j, k, l, normalize=True):
        """tensorizedbasis.jl:183-191."""
        val = 1.0
        for d in range(self.maxlength_multiindices()):
            val *= self.ONB.triple_product(self.multi_indices[j][d], self.multi_indices[k][d],
                                           self.multi_indices[l][d], normalize=normalize)
        return val

    def set_sample(self, x, normalize=True):
        """tensorizedbasis.jl:226-236."""
        for j in range(len(x)):
            self.vals[j] = self.ONB.evaluate(x[j], normalize=normalize).copy()
        for j in range(len(x), len(self.vals)):
            v = np.zeros_like(self.vals[j])
            v[0] = 1.0
            self.vals[j] = v
        return self.vals

    def evaluate(self, j):
        """tensorizedbasis.jl:244-252."""
        prod = 1.0
        mi = self.multi_indices[j]
        for m in range(len(mi)):
            prod *= self.vals[m][mi[m]]
        return prod


def hermite_triple_closed_form(j, k, l):
    """Normalised Hermite triple product (test/runtests.jl:80-93)."""
    if (j + k + l) % 2 == 0 and min(j + k - l, k + l - j, l + j - k) >= 0:
        v = math.factorial(l) * math.factorial(j) * math.factorial(k) / (
            math.factorial((j + k - l) // 2) * math.factorial((k + l - j) // 2)
            * math.factorial((j + l - k) // 2))
        return v / (poly_norm(HERMITE, j) * poly_norm(HERMITE, k) * poly_norm(HERMITE, l))
    return 0.0
