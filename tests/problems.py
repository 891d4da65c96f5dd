"""Shared test problems built with the package's host layer (assembly is
the caller's side of the boundary) plus the matching oracle objects."""
from types import SimpleNamespace

import numpy as np

import __graft_entry__ as ge


def build(N, order, M, mis, basis="legendre", mean=1.0, tau=0.9, freq=1.0, maxm=150):
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=tau, start=1, decay=2, mean=mean, maxm=maxm, freq=freq)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), order)
    B = pkg.LegendrePolynomials if basis == "legendre" else pkg.HermitePolynomials
    maxdeg = max(max(mi) for mi in mis)
    TB = pkg.TensorizedBasis(B, M, maxdeg, maxdeg + 4, multi_indices=mis)
    sol = pkg.SGFEVector(V, TB)
    Ks, b0 = pkg.assemble(pkg.PoissonProblemPrimal, sol, C, rhs=lambda x, y: np.ones_like(x))
    return SimpleNamespace(pkg=pkg, C=C, V=V, TB=TB, sol=sol, Ks=Ks[1:], K0=Ks[0], Kall=Ks, b0=b0,
                           G=TB.G.toarray(), bdofs=V.bdofs, n=V.ndofs, P=TB.nmodes, M=M, mis=mis)


def config1_like(N=32, M=5, deg=2, order=1, basis="legendre"):
    """Config 1 of the workload list at N=32, M=5, deg=2 (P1, total degree set)."""
    pkg = ge.load_package()
    mis = pkg.total_degree_multiindices(M, deg)
    return build(N, order, M, mis, basis=basis)
