"""Build recipe and ctypes binding of the oracle's C restatement (sg_mul.c).

Test infrastructure only (see oracle/__init__.py).  Compiles with gcc into
oracle/liboracle_sg.so (git-ignored, rebuilt on each machine).  The reference
itself is Julia and has no C sources, so there is no oracle/_ref build.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sg_mul.c")
LIB = os.path.join(HERE, "liboracle_sg.so")
_lib = None


def build(force=False):
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp"
        cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", SRC, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed: " + r.stderr)
        os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        lib.oracle_sg_mul.restype = None
        lib.oracle_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


class COperator:
    """The reference mul! in C on CSC matrices (K_0..K_M), dense G, bdofs."""

    def __init__(self, Ks, G, bdofs, P):
        self.lib = load()
        self.n = Ks[0].shape[0]
        self.P = P
        self.M = len(Ks) - 1
        self.mats = []
        for K in Ks:
            K = K.tocsc()
            K.sort_indices()
            self.mats.append((np.ascontiguousarray(K.indptr, dtype=np.int64),
                              np.ascontiguousarray(K.indices, dtype=np.int64),
                              np.ascontiguousarray(K.data, dtype=np.float64)))
        PI = ctypes.POINTER(ctypes.c_int64)
        PD = ctypes.POINTER(ctypes.c_double)
        self._cp = (PI * len(self.mats))(*[m[0].ctypes.data_as(PI) for m in self.mats])
        self._rv = (PI * len(self.mats))(*[m[1].ctypes.data_as(PI) for m in self.mats])
        self._nz = (PD * len(self.mats))(*[m[2].ctypes.data_as(PD) for m in self.mats])
        self.G = np.ascontiguousarray(G, dtype=np.float64)
        self.bdofs = np.ascontiguousarray(bdofs, dtype=np.int64)

    def mul(self, x, nthreads=1):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        PD = ctypes.POINTER(ctypes.c_double)
        PI = ctypes.POINTER(ctypes.c_int64)
        self.lib.oracle_sg_mul(ctypes.c_int64(self.n), ctypes.c_int64(self.P), ctypes.c_int64(self.M),
                               self._cp, self._rv, self._nz, self.G.ctypes.data_as(PD),
                               ctypes.c_int64(len(self.bdofs)), self.bdofs.ctypes.data_as(PI),
                               x.ctypes.data_as(PD), y.ctypes.data_as(PD), ctypes.c_int(int(nthreads)))
        return y

    @staticmethod
    def max_threads():
        return load().oracle_max_threads()
