"""Fixture nes_m.npz: exact values of the reference's NES/NPS out-kernel
integral MezzacappaIntOut(w, w', b1, b2) (kernel_nes.hpp:31-78, the general
branch) for (b1, b2) = (1, 0) and (0, 1), on (w, w') pairs of the NES
quadrature grid (m1_opacities.hpp:880-905) and their reverses, for the unit
test of the mixed path's FP32 integral (tests/test_gpu_nes_mixed.py).

The formula is evaluated with mpmath at enough digits to carry its
catastrophic cancellation; F_k(x) = -Gamma(k+1) Li_{k+1}(-e^x).  Stored as
ln|M| and sign(M), with the inputs.

    python tests/golden/make_nes_golden.py
"""

import os

import mpmath as mp
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def F(k, x):
    return -mp.gamma(k + 1) * mp.polylog(k + 1, -mp.e ** x)


def mezzacappa_out(w, wp, eta, b1, b2):
    """kernel_nes.hpp:31-78 (ComputeFDIForInelastic and MezzacappaIntOut)."""
    x, y = max(w, wp), min(w, wp)
    sign = 1 if wp < w else -1
    adw = abs(w - wp)
    dw = [F(k, eta - wp) - F(k, eta - w) for k in range(1, 6)]
    dab = [F(k, eta) - F(k, eta - adw) for k in range(3, 6)]
    return ((((b1 + b2) * (sign * dab[2] - dw[4]) / 5
              - b1 * (w + wp) * (dw[3] + 2 * ((w + wp) * dw[2] + 3 * w * wp * dw[1]))
              + sign * ((b1 * x - b2 * y) * dab[1] + 2 * (b1 * x * x + b2 * y * y) * dab[0]))
             / (w * w * wp * wp)) - 6 * b1 * dw[0])


def main():
    rng = np.random.default_rng(20261205)
    pairs = []
    for n in (10, 20):
        xs, _ = np.polynomial.legendre.leggauss(n)
        xs = 0.5 * (xs + 1.)
        for _ in range(110):
            i, j, r = rng.integers(0, n), rng.integers(0, n), rng.integers(0, 2)
            a, b = (xs[i] * (1 - xs[j]), xs[i] * (1 + xs[j])) if r == 0 else \
                ((1 - xs[j]) / xs[i], (1 + xs[j]) / xs[i])
            w, wp = 4.364 * a, 4.364 * b
            pairs.append((w, wp) if rng.integers(0, 2) else (wp, w))
    etas = [-40., -5., -1., 0., 2.5, 8., 20., 45., 120., 300.]
    cols = {k: [] for k in ("w", "wp", "eta", "ln_m1", "s_m1", "ln_m2", "s_m2")}
    for k, (w, wp) in enumerate(pairs):
        ev = etas[k % len(etas)]
        mp.mp.dps = 60 + int(0.6 * abs(ev)) + 6 * int(abs(np.log10(min(w, wp))))
        W, WP, E = mp.mpf(w), mp.mpf(wp), mp.mpf(ev)
        m1 = mezzacappa_out(W, WP, E, 1, 0)
        m2 = mezzacappa_out(W, WP, E, 0, 1)
        cols["w"].append(w), cols["wp"].append(wp), cols["eta"].append(ev)
        cols["ln_m1"].append(float(mp.log(abs(m1)))), cols["s_m1"].append(float(mp.sign(m1)))
        cols["ln_m2"].append(float(mp.log(abs(m2)))), cols["s_m2"].append(float(mp.sign(m2)))
    np.savez(os.path.join(HERE, "nes_m.npz"), **{k: np.array(v) for k, v in cols.items()})
    print(len(pairs), "pairs")


if __name__ == "__main__":
    main()
