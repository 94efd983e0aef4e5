"""Pixel quadrature rules, computed from their published mathematics.

Lensed integrates the surface brightness over each pixel with a 2-D rule on
the unit pixel [-0.5, 0.5]^2 (src/quadrature.c:21-43).  A rule has abscissae,
value weights and error weights; the render kernel sums
``(ww.x, ww.y) * compute(x + qq[n])`` over the rule's points in table order
(kernel/lensed.cl:28-32).  The rules named by the reference are

=======  ======  ==========================================================
name     points  construction
=======  ======  ==========================================================
point    1       centre of the pixel
sub2     4       2x2 sub-pixel centres, equal weights
sub4     16      4x4 sub-pixel centres, equal weights
gm75     17      Genz & Malik (1980) degree-7 fully symmetric rule with its
                 embedded degree-5 rule as the error estimate
g3k7     49      Cartesian product of the 7-point Gauss-Kronrod rule; the
                 error weights are the products of (Kronrod - Gauss) weights
g5k11    121     same with the 11-point Gauss-Kronrod rule
g7k15    225     same with the 15-point Gauss-Kronrod rule
=======  ======  ==========================================================

and two rules added here for the 9- and 25-point workloads (the reference has
no 3x3 or 5x5 rule):

=======  ======  ==========================================================
sub3     9       3x3 sub-pixel centres, equal weights, no error estimate
sub5     25      5x5 sub-pixel centres, equal weights, no error estimate
=======  ======  ==========================================================

Point order follows the reference's tables: Cartesian rules run over the
first coordinate in the outer loop, the second in the inner loop, both
ascending; the Genz-Malik rule lists the centre and then each symmetric
orbit in lexicographic order.

The Kronrod nodes are the roots of the Stieltjes polynomial E_{n+1}, the monic
polynomial orthogonal to x^0..x^n under the weight P_n(x) on [-1, 1]; weights
follow from exact integration of the monomials.  Both are solved with mpmath
at 60 digits and rounded to double.

``write_c_table`` emits ``lensed_gb300/csrc/lg_quad_rules.inc`` (committed;
``python -m lensed_gb300.quadrature`` regenerates it).
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from fractions import Fraction
from typing import Dict, List, Tuple

__all__ = ["QuadRule", "generate", "rule", "rule_names", "write_c_table"]


@dataclass(frozen=True)
class QuadRule:
    name: str
    info: str
    points: Tuple[Tuple[float, float], ...]
    weights: Tuple[float, ...]
    errors: Tuple[float, ...]

    @property
    def size(self) -> int:
        return len(self.points)


def _subsample(n: int) -> Tuple[List[Tuple[float, float]], List[float], List[float]]:
    nodes = [Fraction(2 * i + 1, 2 * n) - Fraction(1, 2) for i in range(n)]
    pts = [(float(a), float(b)) for a in nodes for b in nodes]
    w = float(Fraction(1, n * n))
    return pts, [w] * len(pts), [0.0] * len(pts)


def _legendre_coeffs(n: int) -> List[Fraction]:
    """Coefficients c[k] of x^k in the Legendre polynomial P_n (exact)."""
    p0, p1 = [Fraction(1)], [Fraction(0), Fraction(1)]
    if n == 0:
        return p0
    for k in range(1, n):
        # (k+1) P_{k+1} = (2k+1) x P_k - k P_{k-1}
        nxt = [Fraction(0)] * (k + 2)
        for i, c in enumerate(p1):
            nxt[i + 1] += Fraction(2 * k + 1, k + 1) * c
        for i, c in enumerate(p0):
            nxt[i] -= Fraction(k, k + 1) * c
        p0, p1 = p1, nxt
    return p1


def _moment(j: int) -> Fraction:
    """Integral of x^j over [-1, 1]."""
    return Fraction(0) if j % 2 else Fraction(2, j + 1)


def _gauss_kronrod(n: int):
    """Nodes (ascending), Kronrod weights and Gauss weights (0 at the
    Kronrod-only nodes) of the (2n+1)-point Gauss-Kronrod rule on [-1, 1]."""
    import mpmath as mp

    mp.mp.dps = 60
    pn = _legendre_coeffs(n)
    # Stieltjes polynomial E(x) = x^{n+1} + sum_{m<=n} e_m x^m with
    # int P_n(x) E(x) x^k dx = 0 for k = 0..n.
    def pmom(j):  # int P_n(x) x^j dx
        return sum(c * _moment(i + j) for i, c in enumerate(pn))

    a = [[pmom(m + k) for m in range(n + 1)] for k in range(n + 1)]
    rhs = [-pmom(n + 1 + k) for k in range(n + 1)]
    e = _solve_fraction(a, rhs)
    stieltjes = [mp.mpf(c.numerator) / c.denominator for c in e] + [mp.mpf(1)]
    kr_roots = mp.polyroots(list(reversed(stieltjes)), maxsteps=500, extraprec=400)
    legendre = [mp.mpf(c.numerator) / c.denominator for c in pn]
    g_roots = mp.polyroots(list(reversed(legendre)), maxsteps=500, extraprec=400)
    kr = sorted(mp.re(r) for r in kr_roots)
    gs = sorted(mp.re(r) for r in g_roots)
    nodes = sorted(kr + gs)
    m = len(nodes)
    # Kronrod weights: exact for x^0 .. x^(2n)
    vand = mp.matrix(m, m)
    mom = mp.matrix(m, 1)
    for j in range(m):
        for i, x in enumerate(nodes):
            vand[j, i] = x ** j
        mom[j] = mp.mpf(_moment(j).numerator) / _moment(j).denominator
    wk = mp.lu_solve(vand, mom)
    # Gauss weights: w_i = 2 / ((1 - x_i^2) P_n'(x_i)^2)
    dpn = [i * c for i, c in enumerate(pn)][1:]
    wg = {}
    for x in gs:
        d = sum(mp.mpf(c.numerator) / c.denominator * x ** i for i, c in enumerate(dpn))
        wg[x] = 2 / ((1 - x * x) * d * d)
    out_g = []
    for x in nodes:
        match = [g for g in gs if abs(g - x) < mp.mpf(10) ** -40]
        out_g.append(wg[match[0]] if match else mp.mpf(0))
    return nodes, [wk[i] for i in range(m)], out_g


def _solve_fraction(a, b):
    n = len(b)
    m = [row[:] + [b[i]] for i, row in enumerate(a)]
    for c in range(n):
        p = next(r for r in range(c, n) if m[r][c] != 0)
        m[c], m[p] = m[p], m[c]
        for r in range(n):
            if r != c and m[r][c] != 0:
                f = m[r][c] / m[c][c]
                m[r] = [x - f * y for x, y in zip(m[r], m[c])]
    return [m[i][n] / m[i][i] for i in range(n)]


def _cartesian_gk(n: int):
    nodes, wk, wg = _gauss_kronrod(n)
    # map [-1, 1] -> [-0.5, 0.5]: abscissa / 2, 1-D weight / 2
    xs = [x / 2 for x in nodes]
    k1 = [w / 2 for w in wk]
    e1 = [(k - g) / 2 for k, g in zip(wk, wg)]
    pts, w, e = [], [], []
    for i in range(len(xs)):
        for j in range(len(xs)):
            pts.append((float(xs[i]), float(xs[j])))
            w.append(float(k1[i] * k1[j]))
            e.append(float(e1[i] * e1[j]))
    return pts, w, e


def _genz_malik_2d():
    """Genz & Malik (1980) degree-7 rule in 2 dimensions with the embedded
    degree-5 rule; error weights are the differences of the two."""
    import mpmath as mp

    mp.mp.dps = 60
    nd = 2
    l2 = mp.sqrt(mp.mpf(9) / 70)
    l3 = mp.sqrt(mp.mpf(9) / 10)
    l4 = mp.sqrt(mp.mpf(9) / 10)
    l5 = mp.sqrt(mp.mpf(9) / 19)
    w7 = [
        mp.mpf(12824 - 9120 * nd + 400 * nd * nd) / 19683,
        mp.mpf(980) / 6561,
        mp.mpf(1820 - 400 * nd) / 19683,
        mp.mpf(200) / 19683,
        mp.mpf(6859) / 19683 / 2 ** nd,
    ]
    w5 = [
        mp.mpf(729 - 950 * nd + 50 * nd * nd) / 729,
        mp.mpf(245) / 486,
        mp.mpf(265 - 100 * nd) / 1458,
        mp.mpf(25) / 729,
        mp.mpf(0),
    ]
    orbits = [
        [(0, 0)],
        sorted([(-l2, 0), (0, -l2), (0, l2), (l2, 0)]),
        sorted([(-l3, 0), (0, -l3), (0, l3), (l3, 0)]),
        sorted([(-l4, -l4), (-l4, l4), (l4, -l4), (l4, l4)]),
        sorted([(-l5, -l5), (-l5, l5), (l5, -l5), (l5, l5)]),
    ]
    pts, w, e = [], [], []
    for k, orb in enumerate(orbits):
        for (a, b) in orb:
            # the unit cube [-1,1]^2 has volume 4; the pixel has volume 1
            pts.append((float(mp.mpf(a) / 2), float(mp.mpf(b) / 2)))
            w.append(float(w7[k]))
            e.append(float(w7[k] - w5[k]))
    return pts, w, e


def _build() -> Dict[str, QuadRule]:
    rules: Dict[str, QuadRule] = {}

    def add(name, info, data):
        pts, w, e = data
        rules[name] = QuadRule(name, info, tuple(pts), tuple(w), tuple(e))

    add("point", "single point sampling without error estimate", ([(0.0, 0.0)], [1.0], [0.0]))
    add("sub2", "2x2 subsampling without error estimate", _subsample(2))
    add("sub3", "3x3 subsampling without error estimate", _subsample(3))
    add("sub4", "4x4 subsampling without error estimate", _subsample(4))
    add("sub5", "5x5 subsampling without error estimate", _subsample(5))
    add("gm75", "Genz-Malik (7, 5) fully symmetric rule", _genz_malik_2d())
    add("g3k7", "Gauss-Kronrod (7, 3) Cartesian rule", _cartesian_gk(3))
    add("g5k11", "Gauss-Kronrod (11, 5) Cartesian rule", _cartesian_gk(5))
    add("g7k15", "Gauss-Kronrod (15, 7) Cartesian rule", _cartesian_gk(7))
    return rules


_RULES: Dict[str, QuadRule] | None = None
_TABLE = os.path.join(os.path.dirname(__file__), "csrc", "lg_quad_rules.inc")


def generate() -> Dict[str, QuadRule]:
    """Compute every rule from its mathematics (needs mpmath)."""
    return _build()


def _parse_table(path: str = _TABLE) -> Dict[str, QuadRule]:
    """Read the committed C table back (no mpmath needed at run time)."""
    import re

    text = open(path).read()
    arrays = {}
    for m in re.finditer(r"LG_QUAD_(\w+)_(PTS|WHT|ERR)\[\](?:\[2\])? = \{(.*?)\};", text, re.S):
        nums = [float(v) for v in re.findall(r"[-+0-9.eE]+(?:e[-+]?\d+)?", m.group(3))]
        arrays[(m.group(1), m.group(2))] = nums
    rules: Dict[str, QuadRule] = {}
    for m in re.finditer(r'\{"(\w+)", "([^"]*)", (\d+), LG_QUAD_', text):
        nm, info, size = m.group(1), m.group(2), int(m.group(3))
        u = nm.upper()
        pts = arrays[(u, "PTS")]
        rules[nm] = QuadRule(
            nm,
            info,
            tuple((pts[2 * i], pts[2 * i + 1]) for i in range(size)),
            tuple(arrays[(u, "WHT")]),
            tuple(arrays[(u, "ERR")]),
        )
    return rules


def _rules() -> Dict[str, QuadRule]:
    global _RULES
    if _RULES is None:
        _RULES = _parse_table() if os.path.exists(_TABLE) else _build()
    return _RULES


def rule(name: str) -> QuadRule:
    r = _rules()
    if name not in r:
        raise ValueError(f"invalid quadrature rule: {name} (known: {', '.join(r)})")
    return r[name]


def rule_names() -> List[str]:
    return list(_rules())


def write_c_table(path: str | None = None) -> str:
    """Write the C table used by the library (name, info, size, abscissae,
    value weights, error weights per rule)."""
    if path is None:
        path = _TABLE
    lines = [
        "/* Pixel quadrature rules on [-0.5, 0.5]^2, generated by",
        " * lensed_gb300/quadrature.py from the rules' mathematics",
        " * (subsampling grids, Genz-Malik 1980, Gauss-Kronrod).  Do not edit. */",
        "",
    ]
    rules = generate()
    names = list(rules)
    for nm in names:
        r = rules[nm]
        lines.append(f"static const double LG_QUAD_{nm.upper()}_PTS[][2] = {{")
        lines += [f"    {{{a!r}, {b!r}}}," for a, b in r.points]
        lines.append("};")
        lines.append(f"static const double LG_QUAD_{nm.upper()}_WHT[] = {{")
        lines += [f"    {w!r}," for w in r.weights]
        lines.append("};")
        lines.append(f"static const double LG_QUAD_{nm.upper()}_ERR[] = {{")
        lines += [f"    {w!r}," for w in r.errors]
        lines.append("};")
        lines.append("")
    lines.append("static const lg_quad_rule_data LG_QUAD_RULES[] = {")
    for nm in names:
        r = rules[nm]
        u = nm.upper()
        lines.append(
            f'    {{"{nm}", "{r.info}", {r.size}, LG_QUAD_{u}_PTS, LG_QUAD_{u}_WHT, LG_QUAD_{u}_ERR}},'
        )
    lines.append("    {0, 0, 0, 0, 0, 0}")
    lines.append("};")
    text = "\n".join(lines) + "\n"
    with open(path, "w") as f:
        f.write(text)
    return text


if __name__ == "__main__":
    print(write_c_table())
