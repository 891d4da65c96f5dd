"""Stochastic coefficients (host side).

Mirrors src/coefficients/cosinus.jl and src/coefficients/coefficients.jl of
ExtendableASGFEM.jl:
  StochasticCoefficientCosinus   cosinus.jl:11-55 (a_m = d_m cos(pi b1 x) cos(pi b2 y),
                                 d_m = tau (m-1+start)^-decay / zeta(decay, start))
  get_am / get_gradam            cosinus.jl:58-76
  get_a                          coefficients.jl:31-42
``freq`` scales pi in the cosines (1 in the reference; 2 gives the cos(2 pi b x)
variant written in some workload descriptions).
"""
import math

import numpy as np
from scipy.special import zeta


class StochasticCoefficientCosinus:
    def __init__(self, tau=1.0, start=2, decay=2.0, mean=0.0, maxm=100, freq=1.0):
        self.decay = float(decay)
        self.mean_value = float(mean)
        self.freq = float(freq)
        m = np.arange(1, maxm + 1)
        # anti-diagonal walk (0,1),(1,0),(0,2),(1,1),(2,0),(0,3),...
        b1 = np.zeros(maxm, dtype=np.int64)
        b2 = np.zeros(maxm, dtype=np.int64)
        k = 0
        i = 0
        s = 1
        while k < maxm:
            for j in range(s + 1):
                if k >= maxm:
                    break
                b1[k] = j
                b2[k] = s - j
                k += 1
            s += 1
        self.b1 = b1
        self.b2 = b2
        self.decay_factors = (m - 1 + start).astype(np.float64) ** (-self.decay) * (tau / zeta(self.decay, start))

    def maxm(self):
        return len(self.decay_factors)

    def meanvalue(self):
        return self.mean_value

    def get_am(self, x1, x2, m):
        x1 = np.asarray(x1, dtype=np.float64)
        if m == 0:
            return np.full(x1.shape, self.mean_value)
        w = math.pi * self.freq
        return self.decay_factors[m - 1] * np.cos(w * self.b1[m - 1] * x1) * np.cos(w * self.b2[m - 1] * np.asarray(x2))

    def get_gradam(self, x1, x2, m):
        x1 = np.asarray(x1, dtype=np.float64)
        x2 = np.asarray(x2, dtype=np.float64)
        if m == 0:
            return np.zeros(x1.shape), np.zeros(x1.shape)
        w = math.pi * self.freq
        b1, b2, d = self.b1[m - 1], self.b2[m - 1], self.decay_factors[m - 1]
        return (-d * b1 * w * np.sin(b1 * w * x1) * np.cos(b2 * w * x2),
                -d * b2 * w * np.cos(b1 * w * x1) * np.sin(b2 * w * x2))

    def get_a(self, x1, x2, y):
        r = np.full(np.shape(x1), self.mean_value)
        for m in range(1, len(y) + 1):
            r = r + y[m - 1] * self.get_am(x1, x2, m)
        return r
