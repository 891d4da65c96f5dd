"""Oracle restatement of the cosine KLE coefficient.

Test infrastructure only (see ``oracle/__init__.py``).

Follows src/coefficients/cosinus.jl:32-76 (constructor, get_am!, get_gradam!)
and src/coefficients/coefficients.jl:31-42 (get_a!).
"""
import math

import numpy as np
from scipy.special import zeta


class StochasticCoefficientCosinus:
    """a(x, y) = mean + sum_m y_m d_m cos(pi b1_m x1) cos(pi b2_m x2).

    ``freq`` multiplies pi; the reference uses 1 (cosinus.jl:62).
    """

    def __init__(self, tau=1.0, start=2, decay=2.0, mean=0.0, maxm=100, freq=1.0):
        self.decay = float(decay)
        self.mean_value = float(mean)
        self.freq = float(freq)
        d = np.zeros(maxm)
        b1 = np.zeros(maxm, dtype=np.int64)
        b2 = np.zeros(maxm, dtype=np.int64)
        k = 0
        j = 0
        for m in range(1, maxm + 2):  # cosinus.jl:37-51
            if m > 1:
                d[m - 2] = float(m - 2 + start) ** (-decay)
                b1[m - 2] = j
                b2[m - 2] = k
            if k > 0:
                j += 1
                k -= 1
            else:
                k = (j + k) + 1
                j = 0
        amp = tau / zeta(decay, start)  # Hurwitz zeta
        self.decay_factors = d * amp
        self.b1 = b1
        self.b2 = b2

    def maxm(self):
        return len(self.decay_factors)

    def get_am(self, x1, x2, m):
        """cosinus.jl:58-65 (vectorised over points)."""
        x1 = np.asarray(x1, dtype=np.float64)
        if m == 0:
            return np.full(x1.shape, self.mean_value)
        pi = math.pi * self.freq
        return self.decay_factors[m - 1] * np.cos(pi * self.b1[m - 1] * x1) * np.cos(pi * self.b2[m - 1] * np.asarray(x2))

    def get_gradam(self, x1, x2, m):
        """cosinus.jl:67-76."""
        x1 = np.asarray(x1, dtype=np.float64)
        x2 = np.asarray(x2, dtype=np.float64)
        if m == 0:
            return np.zeros(x1.shape), np.zeros(x1.shape)
        pi = math.pi * self.freq
        b1 = self.b1[m - 1]
        b2 = self.b2[m - 1]
        d = self.decay_factors[m - 1]
        g1 = -b1 * pi * np.sin(b1 * pi * x1) * np.cos(b2 * pi * x2)
        g2 = -b2 * pi * np.cos(b1 * pi * x1) * np.sin(b2 * pi * x2)
        return d * g1, d * g2

    def get_a(self, x1, x2, y):
        """coefficients.jl:31-42."""
        r = np.full(np.shape(x1), self.mean_value)
        for m in range(1, len(y) + 1):
            r = r + y[m - 1] * self.get_am(x1, x2, m)
        return r


def pce_lambda(coef, mu, x1, x2, factor=-1.0, N_truncate=None):
    """lambda_mu(x) of expa_PCE_mop (src/coefficients/coefficients.jl:219-260), one
    point, one multi-index: the Hermite chaos coefficient of exp(factor a(x, y)),
    exp(sum_{m<=N} a_m(x)^2 / 2) exp(a_0 factor) prod_d a_d(x)^mu_d / (sqrt(prod_d mu_d!) factor^|mu|)."""
    N = coef.maxm() if N_truncate is None else N_truncate
    s = 0.0
    for m in range(1, N + 1):
        s += float(coef.get_am(x1, x2, m)) ** 2
    s = math.exp(s / 2) * math.exp(coef.mean_value * factor)
    amu = 1.0
    fac = 1
    for d, e in enumerate(mu):
        amu *= float(coef.get_am(x1, x2, d + 1)) ** e
        fac *= math.factorial(e)
    amu /= math.sqrt(fac) * factor ** sum(mu)
    return amu * s
