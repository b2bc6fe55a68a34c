"""Synthetic stand-in for the Guo & Martinez-Pinedo (2019) bremsstrahlung table.

The published GP19 response table is not distributed with bns_nurates (its
``GP19Table.hpp`` is a missing large blob), so its physics values cannot be
reproduced here.  This module builds a clearly synthetic, strictly positive
table with the same 4-D layout the GP19 kernel expects
(``kernel_brem_GP19.hpp:75-139``): axes in baryon density ``nb`` [fm^-3],
electron fraction ``Ye``, temperature ``T`` [MeV] and pair energy ``w`` [MeV],
data flattened as ``[nb][Ye][T][w]`` with ``w`` fastest, in MeV^-1.

The axis ranges follow the ranges stated in the kernel's comments
(``kernel_brem_GP19.hpp:377-383``): nb in [1e-4, 1] fm^-3, Ye <= 0.5,
T in [2, 50] MeV on a 2 MeV grid (so the extrapolation anchors T = 2, 4, 48
and 50 MeV are grid points) and w in [0.05, 398] MeV.  The values are a
smooth Lorentzian in ``w`` whose width grows with ``nb`` and ``T``; they are
only used to exercise the interpolation, clipping and extrapolation code of the
GP19 path with identical bits on the CPU oracle and on the GPU.

A real table is loaded through the same ``load`` entry point of the library
(``bnsn_gp19_set_table``) from user-supplied arrays.
"""

import math

import numpy as np

NB_DIMS = 13
YE_DIMS = 11
T_DIMS = 25
W_DIMS = 32


def axes():
    """Return (nb, ye, t, w) axes as float64 numpy arrays."""
    nb = np.array([10.0 ** (-4.0 + 4.0 * i / (NB_DIMS - 1)) for i in range(NB_DIMS)])
    ye = np.array([0.05 * i for i in range(YE_DIMS)])
    t = np.array([2.0 * (i + 1) for i in range(T_DIMS)])
    wmin, wmax = 0.05, 398.0
    lw0, lw1 = math.log(wmin), math.log(wmax)
    w = np.array([math.exp(lw0 + (lw1 - lw0) * i / (W_DIMS - 1)) for i in range(W_DIMS)])
    # pin the end points exactly
    nb[0], nb[-1] = 1e-4, 1.0
    w[0], w[-1] = wmin, wmax
    return nb, ye, t, w


def table():
    """Return a dict with the axes, their logarithms and the flattened data."""
    nb, ye, t, w = axes()
    lognb = np.array([math.log(v) for v in nb])
    logw = np.array([math.log(v) for v in w])
    NB, YE, TT, WW = np.meshgrid(nb, ye, t, w, indexing="ij")
    gamma = 4.0 * (NB / 0.16) ** 0.6 * (TT / 10.0) ** 0.5 + 0.05
    data = (1.0 + 0.3 * YE) * gamma / (WW * WW + gamma * gamma) / np.sqrt(TT)
    data = np.ascontiguousarray(data.reshape(-1), dtype=np.float64)
    return {
        "dims": (NB_DIMS, YE_DIMS, T_DIMS, W_DIMS),
        "nb": nb, "ye": ye, "t": t, "w": w,
        "lognb": lognb, "logw": logw,
        "data": data,
    }
