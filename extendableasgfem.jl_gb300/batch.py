"""Batches of independent SG problems on one GPU (host side of the batched solver).

The reference solves one problem per solve! call (src/modelproblems/
poisson_primal.jl:38-81).  ``SGBatch`` hands many PoissonProblemPrimal systems
to the library at once (sgfem_batch_*): one preconditioned CG runs all of them
in lock step, each phase one launch over every problem, iterations replayed
from a captured CUDA graph; the apply's form (column slots or pair passes) and
launch shape are timed at finalize and cached on disk.  P1 problems on the
unit-square lattice get the mean-based preconditioner (sine transforms), the
others Jacobi.  ``host_apply_column_slots`` and ``host_sine_transform`` evaluate
the column-slot schedule and the split sine tables on the host (checks, no
GPU).  ``config4_problems`` draws the problem shapes from a SplitMix64 stream
(seed = problem index): n = 16 + r % 113 (n x n P1 mesh), M = 4 + r % 13,
total degree 1 + r % 3.
"""
import ctypes

import numpy as np
import scipy.sparse as sp

from . import _lib

_MASK64 = (1 << 64) - 1


def splitmix64(x):
    """One output of SplitMix64 for the state x (Steele, Lea, Flood 2014)."""
    z = (x + 0x9E3779B97F4A7C15) & _MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
    return z ^ (z >> 31)


def config4_problems(count=256, n_lo=16, n_span=113, m_lo=4, m_span=13, deg_span=3):
    """[(N, M, degree)] for problem indices 0..count-1."""
    out = []
    for i in range(count):
        r = splitmix64(i)
        out.append((n_lo + r % n_span, m_lo + r % m_span, 1 + r % deg_span))
    return out


def _shared_pattern_values(Ks):
    """CSC pattern of K_0 and the (M+1) x nnz values of every K_m on it."""
    K0 = sp.csc_matrix(Ks[0])
    K0.sort_indices()
    vals = np.zeros((len(Ks), K0.nnz))
    for m, K in enumerate(Ks):
        Kc = sp.csc_matrix(K)
        Kc.sort_indices()
        if Kc.nnz == K0.nnz and np.array_equal(Kc.indptr, K0.indptr) and np.array_equal(Kc.indices, K0.indices):
            vals[m] = Kc.data
        else:  # values on K_0's pattern (entries outside it would be lost: refuse)
            extra = abs(Kc) - abs(Kc).multiply(K0 != 0)
            if extra.nnz and abs(extra).max() > 0:
                raise ValueError("K_m has entries outside the pattern of K_0")
            vals[m] = _take(Kc, K0)
    return K0, vals


def _take(Kc, K0):
    out = np.zeros(K0.nnz)
    for j in range(K0.shape[1]):
        rows = K0.indices[K0.indptr[j]:K0.indptr[j + 1]]
        col = Kc[:, j].toarray().ravel()
        out[K0.indptr[j]:K0.indptr[j + 1]] = col[rows]
    return out


def _lattice_size(FES):
    """nl if the dofs are the (nl+1)^2 points of a uniform lattice of the unit square in
    x-fastest order (P1 on unit_square_mesh), else 0."""
    if getattr(FES, "order", 0) != 1:
        return 0
    n = FES.ndofs
    nl = int(round(np.sqrt(n))) - 1
    if nl < 2 or nl > 128 or (nl + 1) ** 2 != n:
        return 0
    i = np.arange(n) % (nl + 1)
    j = np.arange(n) // (nl + 1)
    expect = np.stack([i / nl, j / nl], axis=1)
    return nl if np.allclose(FES.dof_coords, expect, atol=1e-12) else 0


def host_apply_column_slots(Ks, TB, bdofs, x, precision=1):
    """sgfem_batch_host_apply: Y = S X through the column-slot schedule of the batch
    apply, evaluated on the host (precision 1: the FP32 kernel's passes, 0: the FP64
    kernel's); x and the result in the SGFEVector layout.  Returns (y, summary)."""
    lib = _lib.load()
    K0, vals = _shared_pattern_values(Ks)
    n = K0.shape[0]
    M = len(Ks) - 1
    P = TB.nmodes
    colptr = np.ascontiguousarray(K0.indptr.astype(np.int64) + 1)
    rowval = np.ascontiguousarray(K0.indices.astype(np.int64) + 1)
    vals = np.ascontiguousarray(vals)
    G = sp.csc_matrix(TB.G)
    G.sort_indices()
    gcp = np.ascontiguousarray(G.indptr.astype(np.int64) + 1)
    grv = np.ascontiguousarray(G.indices.astype(np.int64) + 1)
    gv = np.ascontiguousarray(G.data.astype(np.float64))
    bd = np.ascontiguousarray(np.asarray(bdofs, dtype=np.int64) + 1)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(n * P)
    msg = ctypes.create_string_buffer(256)
    i64 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    rc = lib.sgfem_batch_host_apply(n, M, P, i64(colptr), i64(rowval), _lib._dp(vals), i64(gcp), i64(grv),
                                    _lib._dp(gv), len(bd), i64(bd), int(precision), _lib._dp(x), _lib._dp(y), msg, 256)
    if rc != _lib.OK:
        raise _lib.SGError(rc, msg.value.decode())
    return y, msg.value.decode()


def host_sine_transform(nl, x):
    """sgfem_batch_host_dst: S x for the columns of x ((nl-1) x ncols), S_ik =
    sin(pi i k / nl), through the batch preconditioner's split tables, on the host."""
    lib = _lib.load()
    x = np.asfortranarray(np.asarray(x, dtype=np.float64).reshape(nl - 1, -1))
    y = np.zeros_like(x, order="F")
    rc = lib.sgfem_batch_host_dst(int(nl), x.shape[1], _lib._dp(x), _lib._dp(y))
    if rc != _lib.OK:
        raise _lib.SGError(rc, "sgfem_batch_host_dst failed")
    return y


class SGBatch:
    def __init__(self, device=0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        rc = self.lib.sgfem_batch_create(ctypes.byref(h), int(device))
        if rc != _lib.OK:
            raise _lib.SGError(rc, "sgfem_batch_create failed")
        self.h = h
        self.shapes = []

    def _check(self, rc, allow=()):
        if rc != _lib.OK and rc not in allow:
            raise _lib.SGError(rc, self.lib.sgfem_batch_last_error(self.h).decode())

    def add(self, FES, TB, Ks, b0):
        """One PoissonProblemPrimal system: K_0..K_M (shared pattern), TB.G, FES boundary dofs, b0."""
        K0, vals = _shared_pattern_values(Ks)
        n = K0.shape[0]
        M = len(Ks) - 1
        P = TB.nmodes
        colptr = np.ascontiguousarray(K0.indptr.astype(np.int64) + 1)
        rowval = np.ascontiguousarray(K0.indices.astype(np.int64) + 1)
        vals = np.ascontiguousarray(vals)
        G = sp.csc_matrix(TB.G)
        G.sort_indices()
        gcp = np.ascontiguousarray(G.indptr.astype(np.int64) + 1)
        grv = np.ascontiguousarray(G.indices.astype(np.int64) + 1)
        gv = np.ascontiguousarray(G.data.astype(np.float64))
        bd = np.ascontiguousarray(np.asarray(FES.bdofs, dtype=np.int64) + 1)
        b0 = np.ascontiguousarray(b0, dtype=np.float64)
        i64 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        self._check(self.lib.sgfem_batch_add(self.h, n, M, P, i64(colptr), i64(rowval), _lib._dp(vals), i64(gcp),
                                             i64(grv), _lib._dp(gv), len(bd), i64(bd), _lib._dp(b0)))
        self.shapes.append((n, P))
        i = len(self.shapes) - 1
        nl = _lattice_size(FES)
        if nl:
            self._check(self.lib.sgfem_batch_set_lattice(self.h, i, nl))
        return i

    def finalize(self):
        self._check(self.lib.sgfem_batch_finalize(self.h))

    @property
    def tuning(self):
        return self.lib.sgfem_batch_tuning(self.h).decode()

    def solve(self, rtol=1e-8, maxit=20000, check_every=16, allow_maxit=False, want_solutions=True):
        """Solutions (list of n*P arrays, SGFEVector entries layout) and stats."""
        total = sum(n * P for n, P in self.shapes)
        x = np.zeros(total) if want_solutions else None
        st = _lib.BatchStats()
        self._check(self.lib.sgfem_batch_solve(self.h, float(rtol), int(maxit), int(check_every),
                                               _lib._dp(x) if x is not None else None, ctypes.byref(st)),
                    allow=(_lib.ERR_MAXIT,) if allow_maxit else ())
        out = []
        if x is not None:
            off = 0
            for n, P in self.shapes:
                out.append(x[off:off + n * P])
                off += n * P
        return out, st.as_dict()

    def problem_stats(self, i):
        it = ctypes.c_int()
        rr = ctypes.c_double()
        self._check(self.lib.sgfem_batch_problem_stats(self.h, int(i), ctypes.byref(it), ctypes.byref(rr)))
        return it.value, rr.value

    def close(self):
        if self.h:
            self.lib.sgfem_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
