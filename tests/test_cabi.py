"""The C ABI library (CPU-side checks, no GPU calls): it builds, loads, and
exports every entry point declared in include/sgfem.h; the ctypes binding
covers every declaration; pure host entry points behave."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "sgfem.h")).read()
    return sorted(set(re.findall(r"SGFEM_API\s+[\w\s\*]*?\b(sgfem_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib(built_pkg):
    return built_pkg._lib.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "sgfem_apply" in syms and "sgfem_solve" in syms and len(syms) >= 20


def test_library_exports_every_declared_symbol(lib, built_pkg):
    path = built_pkg._lib.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    for s in declared_symbols():
        assert hasattr(lib, s)


def test_binding_covers_header(built_pkg):
    assert sorted(built_pkg._lib.SIGNATURES) == declared_symbols()


def test_host_only_entry_points(lib, built_pkg):
    assert lib.sgfem_version() >= 10000
    o = built_pkg._lib.SolveOptions()
    lib.sgfem_default_options(ctypes.byref(o))
    assert o.precision == built_pkg.MIXED and o.preconditioner == built_pkg.PREC_LATTICE
    assert o.rtol == 1e-8 and o.reference_rhs == 1
    assert lib.sgfem_last_error(None) == b"null context"
    assert lib.sgfem_destroy(None) == 0
    assert lib.sgfem_has_lattice(None) == 0


@pytest.mark.parametrize("k", [1, 2])
def test_rt_reference_basis_is_dual_to_its_moments(lib, k):
    """sgfem_rt_reference_basis (the RT_k basis the equilibration estimator maps to
    every cell): its Legendre edge moments and interior moments form the identity,
    and the divergence integrates to the total outward flux (host only)."""
    import numpy as np
    from oracle import fem as of
    nb = 8 if k == 1 else 15

    def basis(pts):
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        vals = np.zeros((len(pts), nb, 2))
        divs = np.zeros((len(pts), nb))
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        assert lib.sgfem_rt_reference_basis(k, len(pts), dp(pts), dp(vals), dp(divs)) == 0
        return vals, divs

    V = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    t, w = np.polynomial.legendre.leggauss(6)
    t, w = (t + 1) / 2, w / 2
    leg = [np.ones_like(t), 2 * t - 1, 0.5 * (3 * (2 * t - 1) ** 2 - 1)]
    D = np.zeros((nb, nb))
    flux = np.zeros(nb)
    for e in range(3):
        a, b = V[e], V[(e + 1) % 3]
        d = b - a
        nrm = np.array([d[1], -d[0]])
        vals, _ = basis(a[None, :] + t[:, None] * d[None, :])
        fl = vals @ nrm                                    # points x nb
        for l in range(k + 1):
            D[e * (k + 1) + l] = (w * leg[l]) @ fl
        flux += w @ fl
    pts, wq = of.triangle_rule(8)
    vals, divs = basis(pts)
    tests = [np.ones(len(pts))] if k == 1 else [np.ones(len(pts)), pts[:, 0], pts[:, 1]]
    r = 3 * (k + 1)
    for c in range(2):
        for q in tests:
            D[r] = (0.5 * wq * q) @ vals[:, :, c]
            r += 1
    assert np.abs(D - np.eye(nb)).max() <= 1e-12
    assert np.abs((0.5 * wq) @ divs - flux).max() <= 1e-12
    assert lib.sgfem_rt_reference_basis(3, 1, None, None, None) != 0
