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
