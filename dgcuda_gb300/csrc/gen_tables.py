#!/usr/bin/env python3
"""Generate dg_tables_data.h: quadrature rules and the orthonormal modal basis.

What is generated (for every order p = 0..5):

* the triangle rule used for the volume integral.  Order p uses the
  symmetric Dunavant rule of degree 2p (degree 1 for p = 0), exactly the
  rule selection of the reference (src/2d/conservation/main.cu:148-187,
  ``quad_2d[2p-1]``), with the weights halved so they sum to the area 1/2 of
  the reference triangle (main.cu:181).  The point order inside each rule
  follows the reference's tables (src/2d/conservation/quadrature.cu:7-122)
  because one piece of the reference depends on a point index (the advection
  CFL speed is sampled at point n_q/2, advection/advection.cu:177).  The
  orbit values are Dunavant's published 15-digit parameters;
* the (p+1)-point Gauss-Legendre rule on [-1, 1] for edges
  (main.cu:190-193), computed here to 40 digits;
* the orthonormal basis: Gram-Schmidt over the monomials 1, r, s, r^2, rs,
  s^2, r^3, ... (graded, decreasing power of r inside a degree, the order of
  src/2d/conservation/basis.cu:68-89) with the exact inner product
  int_T r^a s^b = a! b! / (a+b+2)! on the reference triangle
  {r, s >= 0, r + s <= 1}.  The orthogonalisation runs in exact rational
  arithmetic; only the final normalisation takes a 40-digit square root, so
  every table entry below is the correctly rounded double of the exact value
  at the (decimal) quadrature nodes;
* tabulations: phi at volume points, w * dphi/dr and w * dphi/ds at volume
  points (basis.cu:203-207), phi at the n_1 edge points of the three faces
  with face 2 traversed in reverse (basis.cu:210-214), phi at the three
  vertices (basis.cu:198-200), and the monomial coefficients.

Run:  python gen_tables.py > dg_tables_data.h
"""
from fractions import Fraction
from math import factorial
import mpmath

mpmath.mp.dps = 50
PMAX = 5
NPMAX = (PMAX + 1) * (PMAX + 2) // 2


def monomials(nmodes):
    out = []
    d = 0
    while len(out) < nmodes:
        for j in range(d + 1):
            out.append((d - j, j))
        d += 1
    return out[:nmodes]


def moment(a, b):
    return Fraction(factorial(a) * factorial(b), factorial(a + b + 2))


def inner(p, q):
    s = Fraction(0)
    for (a1, b1), c1 in p.items():
        for (a2, b2), c2 in q.items():
            s += c1 * c2 * moment(a1 + a2, b1 + b2)
    return s


def gram_schmidt(nmodes):
    mons = monomials(nmodes)
    qs, norms = [], []
    for m in mons:
        q = {m: Fraction(1)}
        for ql, nl in zip(qs, norms):
            c = inner({m: Fraction(1)}, ql) / nl
            for k, v in ql.items():
                q[k] = q.get(k, Fraction(0)) - c * v
        qs.append(q)
        norms.append(inner(q, q))
    # orthonormal: phi_k = q_k / sqrt(|q_k|^2), coefficients in monomial order
    phis = []
    for q, n in zip(qs, norms):
        inv = 1 / mpmath.sqrt(mpmath.mpf(n.numerator) / n.denominator)
        phis.append([mpmath.mpf(q.get(m, Fraction(0)).numerator) /
                     q.get(m, Fraction(0)).denominator * inv for m in mons])
    return mons, phis


def ev(coef, mons, r, s):
    return sum(c * r ** a * s ** b for c, (a, b) in zip(coef, mons))


def ev_dr(coef, mons, r, s):
    return sum(c * a * r ** (a - 1) * s ** b for c, (a, b) in zip(coef, mons) if a > 0)


def ev_ds(coef, mons, r, s):
    return sum(c * b * r ** a * s ** (b - 1) for c, (a, b) in zip(coef, mons) if b > 0)


M = mpmath.mpf


def orbit3(a, w):
    """(1-2a, a), (a, 1-2a), (a, a): reference point order for a 3-orbit."""
    b = 1 - 2 * a
    return [(b, a, w), (a, b, w), (a, a, w)]


def perm6(p, order, w):
    return [(p[i], p[j], w) for (i, j) in order]


def dunavant(degree):
    """Dunavant symmetric rules (degree 1, 2, 4, 6, 8, 10); weights sum to 1."""
    third = M(1) / 3
    if degree == 1:
        return [(third, third, M(1))]
    if degree == 2:
        a, b = M(1) / 6, M(2) / 3
        return [(a, a, third), (b, a, third), (a, b, third)]
    if degree == 4:
        return (orbit3(M('0.091576213509771'), M('0.109951743655322')) +
                orbit3(M('0.445948490915965'), M('0.223381589678011')))
    if degree == 6:
        c = (M('0.636502499121399'), M('0.310352451033784'), M('0.053145049844817'))
        return (orbit3(M('0.063089014491502'), M('0.050844906370207')) +
                orbit3(M('0.249286745170910'), M('0.116786275726379')) +
                perm6(c, [(0, 1), (1, 0), (0, 2), (1, 2), (2, 1), (2, 0)],
                      M('0.082851075618374')))
    if degree == 8:
        d = (M('0.008394777409958'), M('0.728492392955404'), M('0.263112829634638'))
        return ([(third, third, M('0.144315607677787'))] +
                orbit3(M('0.459292588292723'), M('0.095091634267285')) +
                orbit3(M('0.170569307751760'), M('0.103217370534718')) +
                orbit3(M('0.050547228317031'), M('0.032458497623198')) +
                perm6(d, [(0, 1), (1, 0), (2, 0), (0, 2), (2, 1), (1, 2)],
                      M('0.027230314174435')))
    if degree == 10:
        c = (M('0.141707219414880'), M('0.307939838764121'), M('0.550352941820999'))
        d = (M('0.025003534762686'), M('0.246672560639903'), M('0.728323904597411'))
        e = (M('0.009540815400299'), M('0.066803251012200'), M('0.923655933587500'))
        return ([(third, third, M('0.090817990382754'))] +
                orbit3(M('0.485577633383657'), M('0.036725957756467')) +
                orbit3(M('0.109481575485037'), M('0.045321059435528')) +
                perm6(c, [(0, 1), (1, 0), (1, 2), (2, 1), (2, 0), (0, 2)],
                      M('0.072757916845420')) +
                perm6(d, [(0, 1), (1, 0), (0, 2), (2, 0), (2, 1), (1, 2)],
                      M('0.028327242531057')) +
                perm6(e, [(0, 1), (1, 0), (1, 2), (2, 1), (2, 0), (0, 2)],
                      M('0.009421666963733')))
    raise ValueError(degree)


def gauss_legendre(n):
    """n-point Gauss-Legendre nodes (ascending) and weights on [-1, 1]."""
    xs, ws = [], []
    for k in range(1, n + 1):
        x = mpmath.cos(mpmath.pi * (k - M(1) / 4) / (n + M(1) / 2))
        for _ in range(100):
            p0, p1 = M(1), x
            for m in range(2, n + 1):
                p0, p1 = p1, ((2 * m - 1) * x * p1 - (m - 1) * p0) / m
            dp = n * (x * p1 - p0) / (x * x - 1) if n > 1 else M(1)
            if n == 1:
                p1, dp = x, M(1)
            dx = p1 / dp
            x -= dx
            if abs(dx) < M(10) ** -45:
                break
        if n == 1:
            x = M(0)
            dp = M(1)
        if abs(x) < M(10) ** -40:  # the middle node of an odd rule is exactly 0
            x = M(0)
        xs.append(x)
        ws.append(2 / ((1 - x * x) * dp * dp))
    order = sorted(range(n), key=lambda i: xs[i])
    return [xs[i] for i in order], [ws[i] for i in order]


def fmt(x):
    return repr(float(x))


def main():
    mons, phis = gram_schmidt(NPMAX)
    out = []
    out.append("/* Generated by gen_tables.py -- do not edit.  Quadrature rules and the")
    out.append(" * orthonormal modal basis on the reference triangle for p = 0..5. */")
    out.append("#pragma once")
    out.append("#define DG_PMAX %d" % PMAX)
    out.append("#define DG_NP_MAX %d" % NPMAX)
    out.append("#define DG_NQ_MAX 25")
    out.append("#define DG_N1_MAX 6")
    nq_list, n1_list = [], []
    blocks = []
    for p in range(PMAX + 1):
        npm = (p + 1) * (p + 2) // 2
        rule = dunavant(1 if p == 0 else 2 * p)
        nq = len(rule)
        t1, w1 = gauss_legendre(p + 1)
        n1 = p + 1
        nq_list.append(nq)
        n1_list.append(n1)
        r = [x[0] for x in rule]
        s = [x[1] for x in rule]
        w = [x[2] / 2 for x in rule]
        B = [[ev(phis[i], mons, r[q], s[q]) for i in range(npm)] for q in range(nq)]
        GR = [[w[q] * ev_dr(phis[i], mons, r[q], s[q]) for i in range(npm)] for q in range(nq)]
        GS = [[w[q] * ev_ds(phis[i], mons, r[q], s[q]) for i in range(npm)] for q in range(nq)]
        E = []
        for f in range(3):
            rows = []
            for j in range(n1):
                if f == 0:
                    rr, ss = M(1) / 2 + t1[j] / 2, M(0)
                elif f == 1:
                    rr, ss = (1 - t1[j]) / 2, (1 + t1[j]) / 2
                else:
                    rr, ss = M(0), M(1) / 2 + t1[n1 - 1 - j] / 2
                rows.append([ev(phis[i], mons, rr, ss) for i in range(npm)])
            E.append(rows)
        V = [[ev(phis[i], mons, vr, vs) for i in range(npm)]
             for (vr, vs) in [(M(0), M(0)), (M(1), M(0)), (M(0), M(1))]]

        def arr1(name, vals, n):
            vals = list(vals) + [0] * (n - len(vals))
            return "  /* %s */ {%s}" % (name, ", ".join(fmt(v) for v in vals))

        def arr2(name, rows, n0, n1_):
            rr = []
            for k in range(n0):
                row = rows[k] if k < len(rows) else []
                row = list(row) + [0] * (n1_ - len(row))
                rr.append("{%s}" % ", ".join(fmt(v) for v in row))
            return "  /* %s */ {%s}" % (name, ",\n    ".join(rr))

        def arr3(name, blk, n0, n1_, n2):
            parts = []
            for k in range(n0):
                rows = blk[k]
                rr = []
                for j in range(n1_):
                    row = rows[j] if j < len(rows) else []
                    row = list(row) + [0] * (n2 - len(row))
                    rr.append("{%s}" % ", ".join(fmt(v) for v in row))
                parts.append("{%s}" % ",\n     ".join(rr))
            return "  /* %s */ {%s}" % (name, ",\n    ".join(parts))

        blk = ["  /* p = %d */ {" % p, "  %d, %d, %d," % (npm, nq, n1)]
        blk.append(arr1("r", r, 25) + ",")
        blk.append(arr1("s", s, 25) + ",")
        blk.append(arr1("w", w, 25) + ",")
        blk.append(arr1("t1", t1, 6) + ",")
        blk.append(arr1("w1", w1, 6) + ",")
        blk.append(arr2("B[q][i]", B, 25, NPMAX) + ",")
        blk.append(arr2("GR[q][i]", GR, 25, NPMAX) + ",")
        blk.append(arr2("GS[q][i]", GS, 25, NPMAX) + ",")
        blk.append(arr3("E[f][j][i]", E, 3, 6, NPMAX) + ",")
        blk.append(arr2("V[v][i]", V, 3, NPMAX))
        blk.append("  }")
        blocks.append("\n".join(blk))
    out.append("typedef struct {")
    out.append("  int n_p, n_q, n_1;")
    out.append("  double r[25], s[25], w[25];      /* volume rule, weights sum to 1/2 */")
    out.append("  double t1[6], w1[6];             /* edge rule on [-1,1], weights sum to 2 */")
    out.append("  double B[25][%d];                /* phi_i(r_q, s_q) */" % NPMAX)
    out.append("  double GR[25][%d];               /* w_q dphi_i/dr (r_q, s_q) */" % NPMAX)
    out.append("  double GS[25][%d];               /* w_q dphi_i/ds (r_q, s_q) */" % NPMAX)
    out.append("  double E[3][6][%d];              /* phi_i at edge point j of face f */" % NPMAX)
    out.append("  double V[3][%d];                 /* phi_i at the three vertices */" % NPMAX)
    out.append("} dg_order_tables;")
    out.append("static const dg_order_tables DG_TABLES[DG_PMAX + 1] = {")
    out.append(",\n".join(blocks))
    out.append("};")
    out.append("/* monomial exponents (a, b) of r^a s^b in basis order */")
    out.append("static const int DG_MONO[%d][2] = {%s};" % (
        NPMAX, ", ".join("{%d, %d}" % m for m in mons)))
    out.append("/* phi_i = sum_k DG_COEF[i][k] r^a_k s^b_k */")
    out.append("static const double DG_COEF[%d][%d] = {" % (NPMAX, NPMAX))
    out.append(",\n".join("  {%s}" % ", ".join(fmt(c) for c in row) for row in phis))
    out.append("};")
    print("\n".join(out))


if __name__ == "__main__":
    main()
