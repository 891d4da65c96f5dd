"""Generate the golden fixtures for the basis layer from closed forms.

The reference's own tests (test/runtests.jl:51-127 of ExtendableASGFEM.jl)
check the Hermite ONBasis and TensorizedBasis against closed-form integrals,
norms and triple products; this script evaluates those closed forms exactly
(rational arithmetic, one final rounding) and writes them to JSON.  The
Legendre coupling values beta_n = n / sqrt(4n^2 - 1) are added for the
Legendre coupling tensor.  Run: python tests/golden/make_golden.py
"""
import json
import math
import os
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))


def hermite_triple(j, k, l):
    """<H_j H_k H_l> / (||H_j|| ||H_k|| ||H_l||) for probabilists' Hermite."""
    if (j + k + l) % 2 or min(j + k - l, k + l - j, l + j - k) < 0:
        return 0.0
    s = (j + k + l) // 2
    num = Fraction(math.factorial(j) * math.factorial(k) * math.factorial(l),
                   math.factorial(s - j) * math.factorial(s - k) * math.factorial(s - l))
    # divide by sqrt(j! k! l!) exactly: value = num / sqrt(j!k!l!)
    den2 = math.factorial(j) * math.factorial(k) * math.factorial(l)
    return float(num) / math.sqrt(den2)


def main():
    out = {}
    order = 6
    out["hermite_1d_order"] = order
    out["hermite_1d_triple"] = [[j, k, l, hermite_triple(j, k, l)]
                                for j in range(order + 1) for k in range(j, order + 1) for l in range(k, order + 1)]
    out["hermite_norms"] = [[j, math.sqrt(math.factorial(j))] for j in range(order + 1)]
    # TensorizedBasis(HermitePolynomials, 3, 3, 6): full set {0..3}^3, triple products
    mis = [[a, b, c] for a in range(4) for b in range(4) for c in range(4)]
    trip = []
    for j in range(0, len(mis), 9):
        for k in range(0, len(mis), 7):
            for l in range(len(mis)):
                v = 1.0
                for d in range(3):
                    v *= hermite_triple(mis[j][d], mis[k][d], mis[l][d])
                trip.append([j, k, l, v])
    out["hermite_tensor_M3_order3_triple_sample"] = trip
    out["legendre_beta"] = [[nn, nn / math.sqrt(4 * nn * nn - 1)] for nn in range(1, 16)]
    out["hermite_beta"] = [[nn, math.sqrt(nn)] for nn in range(1, 16)]
    with open(os.path.join(HERE, "basis_closed_forms.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
