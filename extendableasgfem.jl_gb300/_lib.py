"""ctypes binding of libsgfem.so (the C ABI declared in include/sgfem.h).

The library is the only compute path: if it is missing, importing this module
raises, and no operation falls back to CPU code.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsgfem.so")

OK = 0
ERR_ARGUMENT = 1
ERR_STATE = 2
ERR_CUDA = 3
ERR_NONFINITE = 4
ERR_BREAKDOWN = 5
ERR_MAXIT = 6
ERR_UNSUPPORTED = 7

FP64 = 0
FP32 = 1
MIXED = 2

PREC_NONE = 0
PREC_LATTICE = 1
PREC_JACOBI = 2
PREC_CHOLESKY = 3

_P = ctypes.c_void_p
_I64P = ctypes.POINTER(ctypes.c_int64)
_DP = ctypes.POINTER(ctypes.c_double)


class SolveOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("preconditioner", ctypes.c_int), ("rtol", ctypes.c_double),
                ("maxit", ctypes.c_int), ("inner_rtol", ctypes.c_double), ("reference_rhs", ctypes.c_int),
                ("check_every", ctypes.c_int)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("outer_iterations", ctypes.c_int), ("fp64_applies", ctypes.c_int),
                ("relres", ctypes.c_double), ("time_ms", ctypes.c_double), ("apply_ms", ctypes.c_double),
                ("precond_ms", ctypes.c_double), ("kernel_launches", ctypes.c_longlong)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


# name -> (restype, argtypes); every symbol declared in include/sgfem.h
class BatchStats(ctypes.Structure):
    _fields_ = [("iterations_max", ctypes.c_int), ("converged", ctypes.c_int), ("graph_replays", ctypes.c_int),
                ("relres_max", ctypes.c_double), ("time_ms", ctypes.c_double), ("kernel_launches", ctypes.c_longlong)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}



SIGNATURES = {
    "sgfem_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int]),
    "sgfem_destroy": (ctypes.c_int, [_P]),
    "sgfem_last_error": (ctypes.c_char_p, [_P]),
    "sgfem_version": (ctypes.c_int, []),
    "sgfem_set_spatial_matrix": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int64, _I64P, _I64P, _DP]),
    "sgfem_set_coupling": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int64, _I64P, _I64P, _DP]),
    "sgfem_set_boundary_dofs": (ctypes.c_int, [_P, ctypes.c_int64, _I64P]),
    "sgfem_set_dof_coordinates": (ctypes.c_int, [_P, ctypes.c_int64, _DP]),
    "sgfem_finalize": (ctypes.c_int, [_P]),
    "sgfem_has_lattice": (ctypes.c_int, [_P]),
    "sgfem_update_coupling": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int64, _I64P, _I64P, _DP]),
    "sgfem_lattice_log": (ctypes.c_char_p, [_P]),
    "sgfem_cholesky_log": (ctypes.c_char_p, [_P]),
    "sgfem_small_solve_log": (ctypes.c_char_p, [_P]),
    "sgfem_sampling_error_log": (ctypes.c_char_p, [_P]),
    "sgfem_cholesky_host_solve": (ctypes.c_int, [ctypes.c_int64, _I64P, _I64P, _DP, ctypes.c_int64, _I64P,
                                                 ctypes.c_int64, _DP, _DP, ctypes.c_char_p, ctypes.c_int]),
    "sgfem_apply": (ctypes.c_int, [_P, _DP, _DP, ctypes.c_int]),
    "sgfem_precondition": (ctypes.c_int, [_P, _DP, _DP, ctypes.c_int, ctypes.c_int]),
    "sgfem_solve": (ctypes.c_int, [_P, _DP, _DP, ctypes.POINTER(SolveOptions), ctypes.POINTER(SolveStats)]),
    "sgfem_default_options": (None, [ctypes.POINTER(SolveOptions)]),
    "sgfem_device_layout": (ctypes.c_int, [_P, _I64P, _I64P]),
    "sgfem_apply_device": (ctypes.c_int, [_P, _P, _P, ctypes.c_int]),
    "sgfem_to_device_layout": (ctypes.c_int, [_P, _DP, _P, ctypes.c_int]),
    "sgfem_from_device_layout": (ctypes.c_int, [_P, _P, _DP, ctypes.c_int]),
    "sgfem_solve_device": (ctypes.c_int, [_P, _DP, _P, ctypes.POINTER(SolveOptions), ctypes.POINTER(SolveStats)]),
    "sgfem_time_apply": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _DP]),
    "sgfem_time_residual": (ctypes.c_int, [_P, ctypes.c_int, _DP, ctypes.POINTER(ctypes.c_int)]),
    "sgfem_kernel_launches": (ctypes.c_longlong, [_P]),
    "sgfem_time_precondition": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _DP]),
    "sgfem_estimate_primal": (ctypes.c_int, [_P, _DP, _P, _P, _DP, _P, _P, _DP, _DP]),
    "sgfem_assemble_stiffness": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int64,
                                                _I64P, _I64P, _DP]),
    "sgfem_assemble_convection": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int64,
                                                 _I64P, _I64P, _DP]),
    "sgfem_assemble_rhs": (ctypes.c_int, [_P, _P, _P, _P, _DP, _DP]),
    "sgfem_assemble_pce_rhs": (ctypes.c_int, [_P, _P, _P, _P, _DP, _P, ctypes.c_int64, ctypes.c_int64,
                                              ctypes.POINTER(ctypes.c_int32), ctypes.c_double, ctypes.c_int64, _DP]),
    "sgfem_estimate_logpoisson": (ctypes.c_int, [_P, _DP, _P, _P, _DP, _P, _P, _P, _DP, _DP, _DP]),
    "sgfem_estimate_equilibration": (ctypes.c_int, [_P, _DP, _P, _P, _DP, _P, _P, ctypes.c_double, _DP, _DP]),
    "sgfem_rt_reference_basis": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _DP, _DP, _DP]),
    "sgfem_set_samples": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int64, _DP]),
    "sgfem_solve_samples": (ctypes.c_int, [_P, _DP, _DP, ctypes.POINTER(SolveOptions), ctypes.POINTER(SolveStats)]),
    "sgfem_solve_gmres": (ctypes.c_int, [_P, _DP, _DP, ctypes.POINTER(SolveOptions), ctypes.c_int,
                                         ctypes.POINTER(SolveStats)]),
    "sgfem_adjoint_gradient": (ctypes.c_int, [_P, _DP, _DP, _DP, _P, _DP]),
    "sgfem_batch_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int]),
    "sgfem_batch_destroy": (ctypes.c_int, [_P]),
    "sgfem_batch_last_error": (ctypes.c_char_p, [_P]),
    "sgfem_batch_add": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _I64P, _I64P, _DP, _I64P,
                                       _I64P, _DP, ctypes.c_int64, _I64P, _DP]),
    "sgfem_batch_count": (ctypes.c_int, [_P]),
    "sgfem_batch_host_dst": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, _DP, _DP]),
    "sgfem_batch_host_apply": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _I64P, _I64P, _DP,
                                              _I64P, _I64P, _DP, ctypes.c_int64, _I64P, ctypes.c_int, _DP, _DP,
                                              ctypes.c_char_p, ctypes.c_int]),
    "sgfem_batch_set_lattice": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int64]),
    "sgfem_batch_finalize": (ctypes.c_int, [_P]),
    "sgfem_batch_tuning": (ctypes.c_char_p, [_P]),
    "sgfem_batch_solve": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_int, ctypes.c_int, _DP,
                                         ctypes.POINTER(BatchStats)]),
    "sgfem_batch_problem_stats": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                                 ctypes.POINTER(ctypes.c_double)]),
    "sgfem_evaluate_samples": (ctypes.c_int, [_P, _DP, ctypes.c_int64, _P, _DP, ctypes.c_int64, ctypes.c_int64,
                                              ctypes.c_int64, _DP]),
    "sgfem_sampling_error": (ctypes.c_int, [_P, _DP, _P, _P, _DP, _P, _P, _DP, _DP]),
    "sgfem_precondition_device_static": (ctypes.c_int, [_P, _P, _P, ctypes.c_int]),
    "sgfem_apply_variant": (ctypes.c_int, [_P]),
    "sgfem_apply_variant_log": (ctypes.c_char_p, [_P]),
}

_lib = None


def load():
    """Load libsgfem.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} not found: build the CUDA library first "
                          "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class SGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libsgfem error {code}: {msg}")
        self.code = code


def _dp(a):
    return a.ctypes.data_as(_DP)


def _i64p(a):
    return a.ctypes.data_as(_I64P)


def cholesky_host_solve(K0, bdofs, B):
    """sgfem_cholesky_host_solve: K_0^-1 B (B column-major n x P, SGFEVector layout) by
    the SGFEM_PREC_CHOLESKY factorisation and schedule, on the host; returns (Z, summary)."""
    lib = load()
    n = K0.shape[0]
    B = np.ascontiguousarray(B, dtype=np.float64)
    P = len(B) // n
    cp, rv, nz = _csc_arrays(K0)
    bd = np.ascontiguousarray(np.asarray(bdofs, dtype=np.int64) + 1)
    Z = np.zeros_like(B)
    msg = ctypes.create_string_buffer(512)
    rc = lib.sgfem_cholesky_host_solve(n, _i64p(cp), _i64p(rv), _dp(nz), len(bd), _i64p(bd), P, _dp(B), _dp(Z),
                                       msg, 512)
    if rc != OK:
        raise SGError(rc, msg.value.decode())
    return Z, msg.value.decode()


def _csc_arrays(A):
    """1-based int64 colptr / rowval and float64 nzval of a SciPy sparse matrix
    (Julia SparseMatrixCSC{Float64,Int64} convention)."""
    A = A.tocsc()
    A.sort_indices()
    colptr = np.ascontiguousarray(A.indptr.astype(np.int64) + 1)
    rowval = np.ascontiguousarray(A.indices.astype(np.int64) + 1)
    nzval = np.ascontiguousarray(A.data.astype(np.float64))
    return colptr, rowval, nzval


class Context:
    """One libsgfem context (device memory for one SG operator)."""

    def __init__(self, device=0):
        self.lib = load()
        h = _P()
        rc = self.lib.sgfem_create(ctypes.byref(h), int(device))
        self.h = h
        if rc != OK:
            msg = self.lib.sgfem_last_error(h).decode() if h else "sgfem_create failed"
            self.lib.sgfem_destroy(h)
            self.h = None
            raise SGError(rc, msg)
        self.n = None
        self.P = None

    def _check(self, rc, allow=()):
        if rc != OK and rc not in allow:
            raise SGError(rc, self.lib.sgfem_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.sgfem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- setup
    def set_spatial_matrix(self, m, A):
        colptr, rowval, nzval = _csc_arrays(A)
        self._check(self.lib.sgfem_set_spatial_matrix(self.h, int(m), int(A.shape[0]), _i64p(colptr),
                                                       _i64p(rowval), _dp(nzval)))
        self.n = A.shape[0]

    def set_coupling(self, G, P, M):
        colptr, rowval, nzval = _csc_arrays(G)
        self._check(self.lib.sgfem_set_coupling(self.h, int(P), int(M), _i64p(colptr), _i64p(rowval), _dp(nzval)))
        self.P = P

    def update_coupling(self, G, P, M):
        """New modes on a finalized context (sgfem_update_coupling)."""
        colptr, rowval, nzval = _csc_arrays(G)
        self._check(self.lib.sgfem_update_coupling(self.h, int(P), int(M), _i64p(colptr), _i64p(rowval),
                                                   _dp(nzval)))
        self.P = P

    def set_samples(self, y):
        """y: (M, S) sample matrix (Julia M x S column-major == NumPy (S, M) C-order)."""
        y = np.asarray(y, dtype=np.float64)
        M, S = y.shape
        yc = np.ascontiguousarray(y.T)
        self._check(self.lib.sgfem_set_samples(self.h, int(S), int(M), _dp(yc)))
        self.P = S

    def solve_samples(self, b0, x_inout, options=None, allow_maxit=False):
        """x_inout None: zero start, solutions stay on the device."""
        b0 = np.ascontiguousarray(b0, dtype=np.float64)
        if x_inout is not None:
            assert x_inout.dtype == np.float64 and x_inout.flags.c_contiguous
        o = options if options is not None else self.default_options()
        st = SolveStats()
        xp = _dp(x_inout) if x_inout is not None else None
        self._check(self.lib.sgfem_solve_samples(self.h, _dp(b0), xp, ctypes.byref(o), ctypes.byref(st)),
                    allow=(ERR_MAXIT,) if allow_maxit else ())
        return st

    def set_boundary_dofs(self, bdofs0):
        b = np.ascontiguousarray(np.asarray(bdofs0, dtype=np.int64) + 1)
        self._check(self.lib.sgfem_set_boundary_dofs(self.h, len(b), _i64p(b)))

    def set_dof_coordinates(self, xy):
        xy = np.ascontiguousarray(np.asarray(xy, dtype=np.float64))  # n x 2 == Julia 2 x n column-major
        self._check(self.lib.sgfem_set_dof_coordinates(self.h, xy.shape[0], _dp(xy)))

    def finalize(self):
        self._check(self.lib.sgfem_finalize(self.h))

    @property
    def has_lattice(self):
        return bool(self.lib.sgfem_has_lattice(self.h))

    @property
    def sampling_error_log(self):
        """The form of the last sampling-error call: quadratic forms or quadrature points."""
        return self.lib.sgfem_sampling_error_log(self.h).decode()

    @property
    def small_solve_log(self):
        """Whether mixed solves run the inner FP32 PCG as one cluster launch, or why not."""
        return self.lib.sgfem_small_solve_log(self.h).decode()

    @property
    def cholesky_log(self):
        """The sparse-Cholesky mean preconditioner: its factor size, or 'not factored yet'."""
        return self.lib.sgfem_cholesky_log(self.h).decode()

    @property
    def lattice_log(self):
        """Which mean-based lattice preconditioner is in use (exact block form or Laplacian), and why."""
        return self.lib.sgfem_lattice_log(self.h).decode()

    def device_layout(self):
        n = ctypes.c_int64()
        ld = ctypes.c_int64()
        self._check(self.lib.sgfem_device_layout(self.h, ctypes.byref(n), ctypes.byref(ld)))
        return n.value, ld.value

    # ---- operations on host vectors (SGFEVector.entries layout)
    def apply(self, x, precision=FP64):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self._check(self.lib.sgfem_apply(self.h, _dp(x), _dp(y), int(precision)))
        return y

    def precondition(self, b, kind=PREC_LATTICE, precision=FP64):
        b = np.ascontiguousarray(b, dtype=np.float64)
        y = np.empty_like(b)
        self._check(self.lib.sgfem_precondition(self.h, _dp(b), _dp(y), int(kind), int(precision)))
        return y

    @staticmethod
    def default_options(**kw):
        o = SolveOptions()
        load().sgfem_default_options(ctypes.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    def solve(self, b0, x_inout, options=None, allow_maxit=False):
        """solve_primal!: x_inout (SGFEVector.entries) is the warm start and is overwritten."""
        b0 = np.ascontiguousarray(b0, dtype=np.float64)
        assert x_inout.dtype == np.float64 and x_inout.flags.c_contiguous
        o = options if options is not None else self.default_options()
        st = SolveStats()
        self._check(self.lib.sgfem_solve(self.h, _dp(b0), _dp(x_inout), ctypes.byref(o), ctypes.byref(st)),
                    allow=(ERR_MAXIT,) if allow_maxit else ())
        return st

    # ---- device-resident operations (pointers are integers, e.g. torch tensor.data_ptr())
    def solve_gmres(self, b0_full, x_inout, options=None, restart=20, allow_maxit=False):
        """b0_full: n*P right-hand side blocks (mode-major), x_inout: warm start / solution."""
        b0 = np.ascontiguousarray(b0_full, dtype=np.float64)
        assert x_inout.dtype == np.float64 and x_inout.flags.c_contiguous
        o = options if options is not None else self.default_options()
        st = SolveStats()
        self._check(self.lib.sgfem_solve_gmres(self.h, _dp(b0), _dp(x_inout), ctypes.byref(o), int(restart),
                                               ctypes.byref(st)),
                    allow=(ERR_MAXIT,) if allow_maxit else ())
        return st

    def apply_device(self, x_ptr, y_ptr, precision=FP64):
        self._check(self.lib.sgfem_apply_device(self.h, _P(x_ptr), _P(y_ptr), int(precision)))

    def to_device_layout(self, x, dst_ptr, precision=FP64):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._check(self.lib.sgfem_to_device_layout(self.h, _dp(x), _P(dst_ptr), int(precision)))

    def from_device_layout(self, src_ptr, out, precision=FP64):
        self._check(self.lib.sgfem_from_device_layout(self.h, _P(src_ptr), _dp(out), int(precision)))
        return out

    def solve_device(self, b0, x_ptr, options=None, allow_maxit=False):
        b0 = np.ascontiguousarray(b0, dtype=np.float64)
        o = options if options is not None else self.default_options()
        st = SolveStats()
        self._check(self.lib.sgfem_solve_device(self.h, _dp(b0), _P(x_ptr), ctypes.byref(o), ctypes.byref(st)),
                    allow=(ERR_MAXIT,) if allow_maxit else ())
        return st

    def precondition_device_static(self, r_ptr, z_ptr, precision=FP64):
        """Lattice preconditioner on device-layout vectors using the library's
        static scratch array (no device allocation; see include/sgfem.h)."""
        self._check(self.lib.sgfem_precondition_device_static(self.h, _P(r_ptr), _P(z_ptr), int(precision)))

    @property
    def apply_variant(self):
        """(1 if the FP32 apply is specialised to this coupling structure else 0, log)."""
        return int(self.lib.sgfem_apply_variant(self.h)), self.lib.sgfem_apply_variant_log(self.h).decode()

    def kernel_launches(self):
        return int(self.lib.sgfem_kernel_launches(self.h))

    def time_precondition(self, precision=FP64, reps=10):
        ms = ctypes.c_double()
        self._check(self.lib.sgfem_time_precondition(self.h, int(precision), int(reps), ctypes.byref(ms)))
        return ms.value

    def time_residual(self, reps=10):
        """(ms per refinement residual, 'double-FP32' or 'FP64')."""
        ms = ctypes.c_double()
        kind = ctypes.c_int()
        self._check(self.lib.sgfem_time_residual(self.h, int(reps), ctypes.byref(ms), ctypes.byref(kind)))
        return ms.value, ("double-FP32" if kind.value else "FP64")

    def time_apply(self, precision=FP64, reps=10):
        ms = ctypes.c_double()
        self._check(self.lib.sgfem_time_apply(self.h, int(precision), int(reps), ctypes.byref(ms)))
        return ms.value
