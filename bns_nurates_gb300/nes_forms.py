"""Generator of the polynomial forms of the mixed path's NES/NPS integral
(bns_nurates_gb300/csrc/bnsn_nes32.cuh; run by hand, needs sympy).

The reference's out-kernel integral (MezzacappaIntOut, kernel_nes.hpp:50-78)
is a combination of Fermi integrals F_1..F_5 at eta - w', eta - w, eta and
eta - |w - w'| with polynomial coefficients, times 1/(w^2 w'^2), linear in
the couplings b1, b2.  Substituting
    F_k(eta + c) = int_{-c}^inf (u + c)^k f(u - eta) du,   f(t) = 1/(1 + e^t),
turns the numerator into  int_0^inf [b1 K_1(u) + b2 K_2(u)] f(u - eta) du
with K_1, K_2 piecewise polynomial in u.  With x = max(w, w'), y = min(w, w'),
d = x - y the pieces meet at 0, min(y, d), max(y, d), x; on [x, inf) they are
linear.  Written for w > w' (the other orientation is the same with the sign
of the reference's `sign`), each finite piece is a quintic whose Bernstein
coefficients on the piece are polynomials in m = min(y, d) and e = |d - y|
with non-negative coefficients: evaluated in that basis the kernel has no
cancellation at all.  This script derives the pieces from the reference
formula, checks that, and prints the coefficients as C expressions.

    python bns_nurates_gb300/nes_forms.py
"""

import sympy as sp

w, wp, u, t = sp.symbols('w wp u t', positive=True)
m, e, tau = sp.symbols('m e tau', positive=True)
b1, b2 = sp.symbols('b1 b2')


def numerator_pieces(ycase):
    """{c: poly} with N = sum_c [u > -c] poly(u) for w > w' (x = w, y = w')."""
    y, d = sp.symbols('y d', positive=True)
    W, WP = y + d, y
    fs = {}

    def F(k, c):
        key = (k, sp.simplify(c))
        if key not in fs:
            fs[key] = sp.Symbol(f"F{k}_{len(fs)}")
        return fs[key]

    x, yy, sign, adw = W, WP, 1, d
    dw = [F(k, -WP) - F(k, -W) for k in range(1, 6)]           # G_k(eta - w') - G_k(eta - w)
    dab = [F(k, sp.Integer(0)) - F(k, -adw) for k in range(3, 6)]
    S, P = W + WP, W * WP
    # MezzacappaIntOut (kernel_nes.hpp:50-78) times w^2 w'^2
    N = ((b1 + b2) * (sign * dab[2] - dw[4]) / 5
         - b1 * S * (dw[3] + 2 * (S * dw[2] + 3 * P * dw[1]))
         + sign * ((b1 * x - b2 * yy) * dab[1] + 2 * (b1 * x * x + b2 * yy * yy) * dab[0])) \
        - 6 * b1 * dw[0] * (W * W * WP * WP)
    N = sp.expand(N)
    pieces = {}
    for (k, c), sym in fs.items():
        co = N.coeff(sym)
        if co != 0:
            pieces[c] = pieces.get(c, 0) + co * (u + c) ** k
    # ycase: 'dgy' (d > y) -> y = m, d = m + e; 'dly' -> d = m, y = m + e
    sub = {y: m, d: m + e} if ycase == 'dgy' else {d: m, y: m + e}
    return pieces, sub, (y, d)


def bernstein(poly_t, L):
    """Bernstein coefficients (degree 5, times C(5, j)) of poly(t) on [0, L]."""
    P = sp.Poly(sp.expand(poly_t.subs(t, L * tau)), tau)
    a = [P.coeff_monomial(tau ** k) for k in range(6)]
    c = [sum(sp.binomial(k, j) / sp.binomial(5, j) * a[j] for j in range(k + 1))
         for k in range(6)]
    return [sp.factor(sp.expand(c[j] * sp.binomial(5, j))) for j in range(6)]


def nonneg(expr):
    ex = sp.expand(expr)
    if ex == 0:
        return True
    return all(cf >= 0 for cf in sp.Poly(ex, m, e).coeffs())


def main():
    for ycase in ('dgy', 'dly'):
        pieces, sub, (y, d) = numerator_pieces(ycase)
        order = sorted(pieces, key=lambda c: float((-c).subs(sub).subs({m: 1.0, e: 0.5})))
        ends = [(-c) for c in order] + [sp.oo]
        total = 0
        for i, c in enumerate(order):
            total += pieces[c]
            p, q = ends[i], ends[i + 1]
            for name, bb in (("K1", {b1: 1, b2: 0}), ("K2", {b1: 0, b2: 1})):
                K = sp.expand(total.subs(bb).subs(u, p + t).subs(sub))
                if q == sp.oo:
                    A, B = sp.factor(K.subs(t, 0)), sp.factor(sp.diff(K, t))
                    assert nonneg(A) and nonneg(B) and sp.expand(K - A - B * t) == 0
                    print(f"// {ycase} tail {name}: A + B t,  A = {A},  B = {B}")
                    continue
                L = sp.expand((q - p).subs(sub))
                g = bernstein(K, L)
                assert all(nonneg(gj) for gj in g), (ycase, i, name)
                print(f"// {ycase} piece {i} (length {L}) {name}:")
                for j, gj in enumerate(g):
                    print(f"//   g{j} = {gj}")


def f1_ratio_chebyshev(deg=12):
    """Chebyshev coefficients c_0 .. c_deg (c_0 halved) of R(2 s) = F_1/F_0 on
    [-1, 1], F_0(t) = ln(1 + e^t), F_1(t) = -Li_2(-e^t): the tail of the NES
    integral needs F_1 on [-2, 2], where a direct expansion cancels; R is
    smooth, positive and O(1), so F_1 = F_0 R keeps FP32 relative accuracy.
    Truncation error < 4e-9 relative."""
    import mpmath as mp
    mp.mp.dps = 40
    n = 40
    nodes = [mp.cos(mp.pi * (k + mp.mpf(1) / 2) / n) for k in range(n)]
    vals = [-mp.polylog(2, -mp.e ** (2 * v)) / mp.log(1 + mp.e ** (2 * v)) for v in nodes]
    out = []
    for j in range(deg + 1):
        cj = 2 * sum(v * mp.cos(j * mp.acos(x)) for v, x in zip(vals, nodes)) / n
        out.append(float(cj / 2 if j == 0 else cj))
    print("// R = F_1 / F_0 Chebyshev coefficients:", ", ".join(repr(c) for c in out))
    return out


if __name__ == "__main__":
    main()
    f1_ratio_chebyshev()
