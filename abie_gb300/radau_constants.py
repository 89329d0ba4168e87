"""Derive the Gauss-Radau (order 15) spacing and change-of-basis constants.

The Radau15 predictor-corrector (Everhart 1985) samples the force at
h_0 = 0 and at the seven roots of (P_7(x) + P_8(x)) / (1 + x) mapped from
[-1, 1] to [0, 1] (Radau quadrature with the left end point fixed).  From
the spacings follow

* ``rs[i][j] = 1 / (h_i - h_j)`` for j < i, the divided-difference factors
  that turn sampled forces into the Newton-form coefficients g;
* ``cs[j][k]``, the coefficient of t**k in prod_{i=1..j} (t - h_i), which
  turns the Newton-form coefficients g into power-form coefficients b
  (b_k = sum_j cs[j][k] g_j).

The reference hard-codes these tables in src/integrator_gauss_radau15.h:24-54.
They are re-derived here with 60-digit arithmetic and rounded once to binary64,
and ``tests/test_oracle.py`` checks that every value equals, bit for bit, the
value the reference library was compiled with.

Run as a script to regenerate ``csrc/radau_constants.h``.
"""
import os

import mpmath

mpmath.mp.dps = 60

NH = 8


def spacings():
    """The eight Radau spacings on [0, 1], h_0 = 0 first, ascending."""
    x = mpmath.mpf
    # (P_7 + P_8)/(1+x) has 7 simple roots in (-1, 1); find them by bracketing
    # sign changes on a fine grid and polishing with the secant-free bisection
    # of mpmath.findroot (anderson) from a bracket.
    def f(v):
        return (mpmath.legendre(7, v) + mpmath.legendre(8, v)) / (1 + v)

    grid = [x(-1) + x(2) * k / 4000 for k in range(1, 4000)]
    roots = []
    for a, b in zip(grid[:-1], grid[1:]):
        fa, fb = f(a), f(b)
        if fa == 0:
            roots.append(a)
        elif fa * fb < 0:
            roots.append(mpmath.findroot(f, (a, b), solver="anderson"))
    assert len(roots) == NH - 1, roots
    return [x(0)] + [(r + 1) / 2 for r in sorted(roots)]


def tables():
    h = spacings()
    rs = [[mpmath.mpf(0)] * NH for _ in range(NH)]
    for i in range(NH):
        for j in range(i):
            rs[i][j] = 1 / (h[i] - h[j])
    # cs[j] = coefficients of prod_{i=1..j} (t - h_i), low order first.
    cs = [[mpmath.mpf(0)] * NH for _ in range(NH)]
    cs[0][0] = mpmath.mpf(1)
    for j in range(1, NH):
        for k in range(NH):
            prev_lower = cs[j - 1][k - 1] if k > 0 else mpmath.mpf(0)
            cs[j][k] = prev_lower - h[j] * cs[j - 1][k]
    return h, rs, cs


def fast_tables():
    """Tables of the reassociated (fast) sweep, each entry rounded once.

    * ``rsp[i][j] = prod_{l=j..i-1} rs[i][l]``: the divided-difference chain
      g_{i-1} = (((F_i - F_0) rs[i][0] - g_0) rs[i][1] - ...) rs[i][i-1]
      expanded into (F_i - F_0) rsp[i][0] - sum_{j<i-1} g_j rsp[i][j+1].
    * ``wpos[i][k] = s_i**(k+1) / ((k+2)(k+3)/2)``, s_i = h_i for i < 8 and
      s_8 = 1: the weights of b_k in the predicted position at spacing s_i.
    * ``wg[i][j] = sum_{k<=j} cs[j][k] wpos[i][k]``: the same weights on the
      Newton-form coefficients g_j, and ``vg[j] = sum_{k<=j} cs[j][k]/(k+2)``
      those of the predicted velocity at spacing 1; ``vgs[i][j]`` the
      velocity weights at every spacing s_i (row 8: s = 1).
    """
    h, rs, cs = tables()
    rsp = [[mpmath.mpf(0)] * NH for _ in range(NH)]
    for i in range(1, NH):
        for j in range(i):
            p = mpmath.mpf(1)
            for l in range(j, i):
                p *= rs[i][l]
            rsp[i][j] = p
    wpos = []
    for s in list(h) + [mpmath.mpf(1)]:
        wpos.append([s ** (k + 1) / ((k + 2) * (k + 3) / 2) for k in range(7)])
    # the same polynomials on the Newton-form coefficients g (b = C g):
    # sum_k b_k w_k = sum_j g_j sum_{k<=j} cs[j][k] w_k
    wg = [[sum(cs[j][k] * row[k] for k in range(j + 1)) for j in range(7)] for row in wpos]
    vg = [sum(cs[j][k] / (k + 2) for k in range(j + 1)) for j in range(7)]
    # velocity weights at every spacing: sum_k b_k s^(k+1) / (k+2) on g
    vgs = [[sum(cs[j][k] * s ** (k + 1) / (k + 2) for k in range(j + 1)) for j in range(7)]
           for s in list(h) + [mpmath.mpf(1)]]
    return ([[to_double(v) for v in row] for row in rsp],
            [[to_double(v) for v in row] for row in wpos],
            [[to_double(v) for v in row] for row in wg],
            [to_double(v) for v in vg],
            [[to_double(v) for v in row] for row in vgs])


def to_double(v):
    return float(mpmath.mpf(v))


def double_tables():
    h, rs, cs = tables()
    return ([to_double(v) for v in h],
            [[to_double(v) for v in row] for row in rs],
            [[to_double(v) for v in row] for row in cs])


def emit_header(path):
    h, rs, cs = double_tables()
    rsp, wpos, wg, vg, vgs = fast_tables()

    def row(vals):
        return "{" + ", ".join(float.hex(v) for v in vals) + "}"

    lines = [
        "/* Generated by abie_gb300/radau_constants.py -- do not edit. */",
        "/* Gauss-Radau spacings and Radau15 change-of-basis tables (binary64). */",
        "#ifndef ABIE_RADAU_CONSTANTS_H",
        "#define ABIE_RADAU_CONSTANTS_H",
        "#define ABIE_RADAU_HS_INIT " + row(h),
        "#define ABIE_RADAU_RS_INIT {" + ", ".join(row(r) for r in rs) + "}",
        "#define ABIE_RADAU_CS_INIT {" + ", ".join(row(c) for c in cs) + "}",
        "#define ABIE_RADAU_RSP_INIT {" + ", ".join(row(r) for r in rsp) + "}",
        "#define ABIE_RADAU_WPOS_INIT {" + ", ".join(row(w) for w in wpos) + "}",
        "#define ABIE_RADAU_WG_INIT {" + ", ".join(row(w) for w in wg) + "}",
        "#define ABIE_RADAU_VG_INIT " + row(vg),
        "#define ABIE_RADAU_VGS_INIT {" + ", ".join(row(w) for w in vgs) + "}",
        "#endif",
        "",
    ]
    with open(path, "w") as fh:
        fh.write("\n".join(lines))


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    emit_header(os.path.join(here, "csrc", "radau_constants.h"))
