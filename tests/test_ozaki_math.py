"""The exact-slice arithmetic of the tensor-core element stage, checked on
the CPU with Python integers: the host-built digit tables reproduce the basis
tables, and a contraction done the kernel's way (row exponent, 53-bit fixed
point, 7 balanced base-256 digits, the digit pairs with i + j >= 5, integer
class sums, one rounding) stays within the stated error bound of the exact
dot product, with every class sum inside the exact range of the f32
accumulator."""
from fractions import Fraction

import numpy as np
import pytest

from conftest import split_tables

BIAS = 0x80808080808080
KB = {"eval": 1, "proj": 3, "trace": 1}
OFF = {"eval": 0, "proj": 448, "trace": 1792}
COL = {"eval": 0, "proj": 1, "trace": 2}


def slot(item):
    pos, t = divmod(item, 4)
    return 2 * t + pos if pos < 2 else 2 * t + 8 + (pos - 2)


def bexp(x):
    return int((np.float64(x).view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF))


def to_fixed(x, m):
    """Signed 53-bit fixed point of x on a row with largest biased exponent m."""
    b = int(np.float64(x).view(np.uint64))
    eb = (b >> 52) & 0x7FF
    mant = (b & ((1 << 52) - 1)) | ((1 << 52) if eb else 0)
    sh = m - (eb if eb else 1)
    X = mant >> sh if sh < 64 else 0
    return -X if b >> 63 else X


def digits(X):
    """7 balanced base-256 digits of a signed integer |X| < 2^53."""
    Y = X + BIAS
    d = [((Y >> (8 * j)) & 255) - 128 for j in range(7)]
    assert sum(dj * 256 ** j for j, dj in enumerate(d)) == X
    return d


def table_digits(words, name):
    """d[i][kb][k][n] from the lanes' B-fragment words."""
    kbs = KB[name]
    h = words.view(np.uint16).reshape(2240, 4).view(np.float16).astype(np.float64)
    d = np.zeros((7, kbs, 16, 16))
    for i in range(7):
        for kb in range(kbs):
            for cg in range(2):
                for lane in range(32):
                    g, t = divmod(lane, 4)
                    n = cg * 8 + g
                    w = h[OFF[name] + ((i * kbs + kb) * 2 + cg) * 32 + lane]
                    d[i, kb, 2 * t, n], d[i, kb, 2 * t + 1, n] = w[0], w[1]
                    d[i, kb, 2 * t + 8, n], d[i, kb, 2 * t + 9, n] = w[2], w[3]
    return d.astype(np.int64)


def basis_tables(oracle_mod, p):
    import dgcuda_gb300 as dg
    m = dg.Mesh.square(3, 3)
    V, es, sxy, se = m.arrays()
    o = oracle_mod.Oracle(0, p, V, es, sxy, se, oracle_mod.prm_vec())
    B, GX, GY, SIDE = split_tables(o.tables(), p)[:4]
    npm, nq, n1 = (p + 1) * (p + 2) // 2, [1, 3, 6, 12, 16][p], p + 1
    B, GX, GY = (a.reshape(npm, nq) for a in (B, GX, GY))
    E = SIDE.reshape(3, npm, n1)                      # [f][i][j]
    return npm, nq, n1, B, GX, GY, E


def dense(dg, p):
    """The three tables the library split, as T[name][kb][kslot][nslot]."""
    D = dg.oz_table_image(p)[2]
    return {"eval": D[0:1], "proj": D[1:4], "trace": D[4:5]}


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_split_tables_are_the_basis_tables(dglib, oracle_mod, p):
    """The dense tables hold the basis values at the right slots (against
    the oracle's own evaluation of the same basis, which rounds
    differently: a few ulp)."""
    dg = dglib
    npm, nq, n1, B, GX, GY, E = basis_tables(oracle_mod, p)
    T = dense(dg, p)
    for q in range(nq):
        for i in range(npm):
            assert abs(T["eval"][0, slot(i), slot(q)] - B[i, q]) <= 1e-13
            assert abs(T["proj"][0, slot(q), slot(i)] - GX[i, q]) <= 1e-13
            assert abs(T["proj"][1, slot(q), slot(i)] - GY[i, q]) <= 1e-13
    for f in range(3):
        for j in range(n1):
            for i in range(npm):
                assert T["proj"][2, slot(f * n1 + j), slot(i)] == T["trace"][0, slot(i), slot(f * n1 + j)]
                assert abs(T["trace"][0, slot(i), slot(f * n1 + j)] - E[f, i, j]) <= 1e-13
    used = np.zeros((16, 16), bool)
    used[[slot(i) for i in range(npm)], :] = True
    assert np.all(T["eval"][0][~used] == 0)


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_digit_tables_reproduce_the_basis_tables(dglib, oracle_mod, p):
    dg = dglib
    words, colexp, _ = dg.oz_table_image(p)
    T = dense(dg, p)
    for name in KB:
        d = table_digits(words, name)
        assert np.abs(d).max() <= 128
        for kb in range(KB[name]):
            for k in range(16):
                for n in range(16):
                    M = int(colexp[COL[name], n])
                    Tint = sum(int(d[i, kb, k, n]) * 256 ** i for i in range(7))
                    exact = Fraction(float(T[name][kb, k, n]))
                    got = Fraction(Tint) * Fraction(2) ** (M - 1075)
                    # truncation to the column's fixed point: below one unit
                    assert abs(got - exact) < Fraction(2) ** (M - 1075)
                    if exact != 0 and bexp(T[name][kb, k, n]) == M:
                        assert got == exact


def emulate(x, col_digits, M):
    """One output of the contraction the kernel's way: x are the row's inputs
    at the K slots, col_digits[i][k] the table column's digits."""
    m = max(bexp(v) for v in x)
    if m == 0:
        return 0.0, [0] * 8
    X = [to_fixed(v, max(m, 1)) for v in x]
    dx = [digits(v) for v in X]
    cls = [0] * 8
    for i in range(7):
        for j in range(7):
            if i + j < 5:
                continue
            cls[12 - i - j] += sum(int(col_digits[i][k]) * dx[k][j] for k in range(len(x)))
    S = sum(c * 256 ** (7 - w) for w, c in enumerate(cls))
    return float(Fraction(S) * Fraction(2) ** (m + M - 2110)), cls


@pytest.mark.parametrize("p", [2, 3, 4])
def test_contraction_error_bound_and_exact_range(dglib, oracle_mod, p):
    dg = dglib
    words, colexp, _ = dg.oz_table_image(p)
    T = dense(dg, p)
    rng = np.random.default_rng(p)
    for name, kb_in in (("eval", [0]), ("proj", [0, 1, 2]), ("trace", [0])):
        d = table_digits(words, name)
        for trial in range(40):
            # rows of mixed scales, signs and zeros, as the solver sees them
            xs = [rng.standard_normal(16) * 10.0 ** rng.uniform(-3, 3, 16) for _ in kb_in]
            for x in xs:
                x[rng.random(16) < 0.2] = 0.0
            n = int(rng.integers(0, 16))
            M = int(colexp[COL[name], n])
            x_all = np.concatenate(xs)
            col = [[d[i, kb, k, n] for kb in kb_in for k in range(16)] for i in range(7)]
            got, cls = emulate(x_all, col, M)
            t_all = np.concatenate([T[name][kb, :, n] for kb in kb_in])
            exact = sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(x_all, t_all))
            scale = Fraction(float(np.abs(x_all).max())) * Fraction(float(np.abs(t_all).max()))
            K = int(np.count_nonzero(t_all))
            assert abs(Fraction(got) - exact) <= K * scale * Fraction(2) ** -52 + abs(exact) * Fraction(2) ** -53
            assert all(abs(c) < 2 ** 22 for c in cls)


def test_class_sums_cannot_leave_the_exact_f32_window():
    """Worst case over all inputs: 7 pairs per class, 36 real K slots, digit
    products at most 128 * 128."""
    pairs = max(sum(1 for i in range(7) for j in range(7) if i + j == s) for s in range(5, 13))
    assert pairs == 7
    assert pairs * 36 * 128 * 128 < 2 ** 22
