"""Pins of the oracle's basis layer against the reference's own known-answer
tests (test/runtests.jl:51-127 of ExtendableASGFEM.jl): Hermite ONBasis
integrals, norms, orthonormality, triple products (tolerance 1e-12 as there),
the tensorised triple products, and the coupling tensor G built from them.
Closed forms are in tests/golden/basis_closed_forms.json (make_golden.py)."""
import json
import math
import os

import numpy as np
import pytest

from oracle import basis as ob
from oracle import mopcontrol as om

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "basis_closed_forms.json")))
TOL = 1e-12  # test/runtests.jl:35


@pytest.fixture(scope="module")
def onb():
    order = GOLD["hermite_1d_order"]
    return ob.ONBasis(ob.HERMITE, order, 3 * order)


def test_hermite_integrals(onb):
    for j in range(onb.maxorder + 1):
        assert abs(onb.integral(j) - (1.0 if j == 0 else 0.0)) < TOL


def test_hermite_norms(onb):
    for j, v in GOLD["hermite_norms"]:
        assert abs(onb.norm4poly(j) - v) < TOL * max(1.0, v)


def test_hermite_orthonormality(onb):
    for j in range(onb.maxorder + 1):
        for k in range(j, onb.maxorder + 1):
            assert abs(onb.scalar_product(j, k) - (1.0 if j == k else 0.0)) < TOL


def test_hermite_triple_products(onb):
    for j, k, l, v in GOLD["hermite_1d_triple"]:
        assert abs(onb.triple_product(j, k, l) - v) < TOL


def test_tensorized_hermite_triple_products():
    TB = ob.TensorizedBasis(ob.HERMITE, 3, 3, 6)
    assert TB.nmodes == 64
    for j, k, l, v in GOLD["hermite_tensor_M3_order3_triple_sample"]:
        assert abs(TB.triple_product(j, k, l) - v) < TOL


def test_hermite_G_is_triple_product_with_ym():
    """G[m, j, k] = <y_m H_j H_k> = triple_product(j, k, e_m) since H_1(y) = y."""
    TB = ob.TensorizedBasis(ob.HERMITE, 3, 3, 6)
    P = TB.nmodes
    for m in range(3):
        em = TB.multi_indices.index([1 if d == m else 0 for d in range(3)])
        for j in range(P):
            for k in range(P):
                assert abs(TB.G[m * P + j, k] - TB.triple_product(j, k, em)) < TOL


@pytest.mark.parametrize("obt,key", [(ob.LEGENDRE, "legendre_beta"), (ob.HERMITE, "hermite_beta")])
def test_coupling_closed_forms(obt, key):
    """G[j, j+e_m] = beta_{mu_j[m]+1}, G[j, j-e_m] = beta_{mu_j[m]}."""
    beta = dict((int(n), v) for n, v in GOLD[key])
    mis = om.generate_multiindices(2, 5)
    G = ob.get_tensor_multiplication_with_ym(obt, mis)
    P = len(mis)
    for j, mi in enumerate(mis):
        for m in range(2):
            up = list(mi)
            up[m] += 1
            if up in mis:
                assert abs(G[m * P + j, mis.index(up)] - beta[mi[m] + 1]) < 1e-15
            if mi[m] > 0:
                dn = list(mi)
                dn[m] -= 1
                assert abs(G[m * P + j, mis.index(dn)] - beta[mi[m]]) < 1e-15


def test_legendre_onbasis_orthonormal():
    onb = ob.ONBasis(ob.LEGENDRE, 8, 16)
    for j in range(9):
        assert abs(onb.norm4poly(j) - 1.0 / math.sqrt(2 * j + 1)) < TOL
        for k in range(9):
            assert abs(onb.scalar_product(j, k) - (1.0 if j == k else 0.0)) < TOL
    # G for Legendre is the triple product with y = H_1 / ||H_1||^{-1}: <y H_j H_k>
    TB = ob.TensorizedBasis(ob.LEGENDRE, 2, 3, 6)
    P = TB.nmodes
    e1 = TB.multi_indices.index([1, 0])
    h1 = 1.0 / math.sqrt(3.0)  # y = H_1 * ||P_1||, ||P_1|| = 1/sqrt(3) in the probability measure
    for j in range(P):
        for k in range(P):
            assert abs(TB.G[j, k] - h1 * TB.triple_product(j, k, e1)) < TOL
