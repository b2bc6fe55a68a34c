"""Fixture pair_j.npz: exact values of the pair-annihilation integrals
J_0 = PairPsi(y, z) / (1 - e^{y+z}) and J_1 = PairPsi(z, y) / (1 - e^{y+z})
(kernel_pair.hpp:16-120, l = 0) on quadrature-grid cells, for the unit test
of the mixed path's FP32 integral (tests/test_gpu_pair_mixed.py).

The reference's own formula is evaluated with mpmath at 60 + eta/2 + ...
digits, enough to carry its catastrophic cancellation; F_k(x) =
-Gamma(k+1) Li_{k+1}(-e^x) are its unnormalised Fermi integrals.  Stored as
ln J (float64), with the inputs.

    python tests/golden/make_pair_golden.py
"""

import os

import mpmath as mp
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def F(k, x):
    return -mp.gamma(k + 1) * mp.polylog(k + 1, -mp.e ** x)


def psi(y, z, eta):
    """PairPsi(l = 0) of kernel_pair.hpp:16-120: (Psi(y, z), Psi(z, y))."""
    f = lambda k, a: F(k, eta + a)
    a1my, a1mz, a1py, a1pz = f(1, -y), f(1, -z), f(1, y), f(1, z)
    a2my, a2mz, a2py, a2pz = f(2, -y), f(2, -z), f(2, y), f(2, z)
    a3e, a3my, a3mz, a3py, a3pz = f(3, 0), f(3, -y), f(3, -z), f(3, y), f(3, z)
    a3myz, a3pyz = f(3, -y - z), f(3, y + z)
    a4e, a4my, a4mz, a4py, a4pz = f(4, 0), f(4, -y), f(4, -z), f(4, y), f(4, z)
    a4myz, a4pyz = f(4, -y - z), f(4, y + z)
    a5my, a5mz, a5py, a5pz, a5myz, a5pyz = (f(5, -y), f(5, -z), f(5, y), f(5, z),
                                            f(5, -y - z), f(5, y + z))
    c0, c1 = 20 * a4my, 20 * a4pz
    c2 = 120 * a2my - 120 * a2pz
    c3 = -40 * a3my + 40 * a3pz
    c4 = 40 * a3e
    c5 = 40 * a3myz - c4
    c6 = -20 * a4e
    c7 = 20 * a4myz + c6
    c8 = -40 * a3pyz + c4
    c9 = 20 * a4pyz + c6
    c10 = -4 * a5my + 4 * a5myz - 4 * a5mz + 4 * a5py - 4 * a5pyz + 4 * a5pz
    c11, c12 = 20 * a4py, 20 * a4mz
    c13 = -40 * a3mz + 40 * a3py
    c14 = 120 * a2mz - 120 * a2py
    den = 15 * (y * z) ** 2
    p0 = (c10 + y * (-c0 + c1 + c7 + y * (c3 + c5 + z * (c2 + z * (-120 * a1my + 120 * a1pz)))
                     + z * (80 * a3my - 80 * a3pz - c2 * z)) + z * (c0 - c1 + c9 + z * (c3 + c8)))
    p1 = (c10 + y * (-c11 + c12 + c9 + y * (c13 + c8))
          + z * (c11 - c12 + c7 + y * (80 * a3mz - 80 * a3py - c14 * y)
                 + z * (c13 + c5 + y * (c14 + y * (-120 * a1mz + 120 * a1py)))))
    return p0 / den, p1 / den


def main():
    rng = np.random.default_rng(20261204)
    cells = []
    for n in (8, 20):
        x, _ = np.polynomial.legendre.leggauss(n)
        x = 0.5 * (x + 1.)
        nodes = np.concatenate([2.182 * x, 2.182 / x])   # y = omega / T of the grey grid
        for _ in range(160):
            a, b = rng.integers(0, 2 * n, 2)
            cells.append((nodes[a], nodes[b]))
    etas = [-60., -25., -3., 0., 1.5, 8., 22.24, 45., 120., 190.]
    y, z, eta, l0, l1 = [], [], [], [], []
    for k, (yv, zv) in enumerate(cells):
        ev = etas[k % len(etas)]
        if ev - yv - zv > 200.:
            continue
        mp.mp.dps = 60 + int(0.5 * max(ev, 0.) + 2. * abs(np.log10(yv * zv)))
        p0, p1 = psi(mp.mpf(yv), mp.mpf(zv), mp.mpf(ev))
        d = 1 - mp.e ** (mp.mpf(yv) + mp.mpf(zv))
        y.append(yv), z.append(zv), eta.append(ev)
        l0.append(float(mp.log(p0 / d)))
        l1.append(float(mp.log(p1 / d)))
    np.savez(os.path.join(HERE, "pair_j.npz"), y=np.array(y), z=np.array(z), eta=np.array(eta),
             ln_j0=np.array(l0), ln_j1=np.array(l1))
    print(len(y), "cells")


if __name__ == "__main__":
    main()
