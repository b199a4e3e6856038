"""Basis and quadrature tables (dg_tables_data.h, generated by
dgcuda_gb300/csrc/gen_tables.py): exactness of the rules, orthonormality of
the basis, and the distance to the reference's tabulation."""
from math import factorial

import numpy as np
import pytest

from conftest import ref_tables, split_tables


def oracle_tables(O, p):
    import dgcuda_gb300 as dg
    m = dg.Mesh.square(3, 3)
    V, es, sxy, se = m.arrays()
    o = O.Oracle(0, p, V, es, sxy, se, O.prm_vec())
    return split_tables(o.tables(), p)


@pytest.mark.parametrize("p", range(6))
def test_triangle_rule_exact_to_degree_2p(dglib, oracle_mod, p):
    B, GX, GY, SIDE, VERT, w, r, s, t1, w1 = oracle_tables(oracle_mod, p)
    for deg in range(2 * p + 1):
        for b in range(deg + 1):
            a = deg - b
            exact = factorial(a) * factorial(b) / factorial(a + b + 2)
            assert abs(np.sum(w * r ** a * s ** b) - exact) <= 2e-15


@pytest.mark.parametrize("p", range(6))
def test_gauss_legendre_exact_to_degree_2p_plus_1(dglib, oracle_mod, p):
    *_, t1, w1 = oracle_tables(oracle_mod, p)
    for k in range(2 * p + 2):
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs(np.sum(w1 * t1 ** k) - exact) <= 1e-15
    assert np.all(np.diff(t1) > 0)


@pytest.mark.parametrize("p", range(6))
def test_basis_orthonormal(dglib, oracle_mod, p):
    B, GX, GY, SIDE, VERT, w, *_ = oracle_tables(oracle_mod, p)
    npm, nq = (p + 1) * (p + 2) // 2, len(w)
    Bq = B.reshape(npm, nq)
    M = (Bq * w) @ Bq.T
    assert np.abs(M - np.eye(npm)).max() <= 5e-14


# bound on |exact - reference| per order, relative to the table's largest entry
REF_TABLE_GAP = {0: 1e-15, 1: 1e-14, 2: 1e-13, 3: 1e-11, 4: 2e-9, 5: 5e-7}


@pytest.mark.parametrize("p", range(6))
def test_reference_tabulation_differs_only_by_its_rounding(dglib, oracle_mod, p):
    mine = oracle_tables(oracle_mod, p)
    ref = split_tables(ref_tables(p), p)
    for a, b in zip(mine, ref):
        assert np.abs(a - b).max() <= REF_TABLE_GAP[p] * max(1.0, np.abs(b).max())
