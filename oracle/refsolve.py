"""The reference's solve_primal! on the host cores, timed as the CPU baseline.

Test infrastructure only (see oracle/__init__.py): bench.py's reference arm and
CPU-baseline leg time it, tests check it against the pure-Python oracle.

Follows src/modelproblems/solvers_poisson_primal.jl:
  MyPreconditionerPrimal :23-44   K_0 with 1e60 on the boundary diagonals,
                                  factored once (SuperLU through SciPy, as a
                                  library; the reference uses UMFPACK);
  ldiv!                  :47-78   one LU solve per mode (oracle_lu_solve_modes:
                                  the triangular solves in C, modes split over
                                  the host threads);
  mul!                   :86-124  oracle_sg_mul (one SpMV per nonzero of G);
  solve_primal!          :130-169 b = x0 + e_1 (x) b0 with boundary rows zeroed,
                                  left-preconditioned GMRES without restarts
                                  (Krylov.jl gmres, M = P, ldiv = true), modified
                                  Gram-Schmidt and Givens rotations.
The reference stops at atol = rtol = 1e-14 on the preconditioned residual; the
measured metric is the time to a true relative residual ||b - A x|| <= rtol ||b||,
so once the preconditioned residual estimate has fallen below rtol times its
start value the solution is formed and its true residual checked after every
further iteration.
"""
import ctypes
import os
import time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import cbuild

PD = ctypes.POINTER(ctypes.c_double)
PI = ctypes.POINTER(ctypes.c_int64)


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


class ReferenceSolver:
    def __init__(self, Ks, G, bdofs, P, nthreads=None, permc_spec="MMD_AT_PLUS_A"):
        self.lib = cbuild.load()
        self.lib.oracle_dot.restype = ctypes.c_double
        self.n = Ks[0].shape[0]
        self.P = P
        self.bdofs = np.asarray(bdofs, dtype=np.int64)
        self.nthreads = int(nthreads or os.cpu_count())
        self.op = cbuild.COperator(Ks, G, bdofs, P)
        t = time.perf_counter()
        A = sp.csc_matrix(Ks[0], dtype=np.float64, copy=True)
        A = A.tolil()
        for d in self.bdofs:
            A[d, d] = 1.0e60
        lu = spla.splu(sp.csc_matrix(A), permc_spec=permc_spec)
        L, U = lu.L.tocsc(), lu.U.tocsc()
        L.sort_indices()
        U.sort_indices()
        self.f = (_i64(L.indptr), _i64(L.indices), np.ascontiguousarray(L.data),
                  _i64(U.indptr), _i64(U.indices), np.ascontiguousarray(U.data),
                  _i64(lu.perm_r), _i64(lu.perm_c))
        self.t_factor = time.perf_counter() - t
        self.factor_nnz = int(L.nnz + U.nnz)

    # ---------------------------------------------------------------- kernels
    def mul(self, x):
        return self.op.mul(x, nthreads=self.nthreads)

    def ldiv(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty_like(b)
        Lp, Li, Lx, Up, Ui, Ux, pr, pc = self.f
        self.lib.oracle_lu_solve_modes(ctypes.c_int64(self.n), ctypes.c_int64(self.P), Lp.ctypes.data_as(PI),
                                       Li.ctypes.data_as(PI), Lx.ctypes.data_as(PD), Up.ctypes.data_as(PI),
                                       Ui.ctypes.data_as(PI), Ux.ctypes.data_as(PD), pr.ctypes.data_as(PI),
                                       pc.ctypes.data_as(PI), b.ctypes.data_as(PD), x.ctypes.data_as(PD),
                                       ctypes.c_int(self.nthreads))
        return x

    def _dot(self, x, y):
        return self.lib.oracle_dot(ctypes.c_int64(len(x)), x.ctypes.data_as(PD), y.ctypes.data_as(PD),
                                   ctypes.c_int(self.nthreads))

    def _axpy(self, a, x, y):
        self.lib.oracle_axpy(ctypes.c_int64(len(x)), ctypes.c_double(a), x.ctypes.data_as(PD), y.ctypes.data_as(PD),
                             ctypes.c_int(self.nthreads))

    def _scale(self, a, x, out):
        self.lib.oracle_scale_copy(ctypes.c_int64(len(x)), ctypes.c_double(a), x.ctypes.data_as(PD),
                                   out.ctypes.data_as(PD), ctypes.c_int(self.nthreads))

    # ---------------------------------------------------------------- solve
    def rhs(self, b0, x0):
        n, P = self.n, self.P
        b = x0.copy()
        b[:n] += b0
        for mu in range(P):
            b[mu * n + self.bdofs] = 0.0
        return b

    def solve(self, b0, x0=None, rtol=1e-8, itmax=300):
        """x, stats: iterations, true relative residual, time split."""
        n, P = self.n, self.P
        N = n * P
        x0 = np.zeros(N) if x0 is None else np.asarray(x0, dtype=np.float64)
        tm = dict(mul=0.0, ldiv=0.0, orth=0.0, check=0.0)
        t_all = time.perf_counter()
        b = self.rhs(b0, x0)
        nb = np.sqrt(self._dot(b, b))

        def timed(key, fn, *a):
            t = time.perf_counter()
            r = fn(*a)
            tm[key] += time.perf_counter() - t
            return r

        r0 = b - timed("mul", self.mul, x0)
        q = timed("ldiv", self.ldiv, r0)
        beta = np.sqrt(self._dot(q, q))
        V = [np.empty(N)]
        self._scale(1.0 / beta, q, V[0])
        R = np.zeros((itmax + 1, itmax + 1))
        cs = np.zeros(itmax)
        sn = np.zeros(itmax)
        z = np.zeros(itmax + 1)
        z[0] = beta
        x = x0.copy()
        relres = np.inf
        k = 0
        armed = False
        for k in range(itmax):
            w = timed("ldiv", self.ldiv, timed("mul", self.mul, V[k]))
            t = time.perf_counter()
            for i in range(k + 1):  # modified Gram-Schmidt
                R[i, k] = self._dot(V[i], w)
                self._axpy(-R[i, k], V[i], w)
            hbis = np.sqrt(self._dot(w, w))
            for i in range(k):
                a = cs[i] * R[i, k] + sn[i] * R[i + 1, k]
                R[i + 1, k] = -sn[i] * R[i, k] + cs[i] * R[i + 1, k]
                R[i, k] = a
            d = np.hypot(R[k, k], hbis)
            cs[k], sn[k] = R[k, k] / d, hbis / d
            R[k, k] = d
            z[k + 1] = -sn[k] * z[k]
            z[k] = cs[k] * z[k]
            tm["orth"] += time.perf_counter() - t
            armed = armed or abs(z[k + 1]) <= rtol * beta
            if armed or hbis == 0.0:
                t = time.perf_counter()
                y = np.linalg.solve(np.triu(R[:k + 1, :k + 1]), z[:k + 1])
                x = x0.copy()
                for i in range(k + 1):
                    self._axpy(y[i], V[i], x)
                tm["check"] += time.perf_counter() - t
                res = b - timed("mul", self.mul, x)
                relres = np.sqrt(self._dot(res, res)) / nb
                if relres <= rtol or hbis == 0.0:
                    break
            V.append(np.empty(N))
            self._scale(1.0 / hbis, w, V[k + 1])
        total = time.perf_counter() - t_all
        return x, dict(iterations=k + 1, relres=float(relres), time_s=total, split_s=tm, threads=self.nthreads)
