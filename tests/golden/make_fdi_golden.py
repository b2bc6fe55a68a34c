"""Generate tests/golden/fdi_family.npz: the reference's Fermi-Dirac integral
family (functions.hpp:442-4375, FDI_m92 .. FDI_p212) on a fixed set of
arguments, with high-precision values to pin it.

Run where the reference checkout is available (mpmath needed):
    python tests/golden/make_fdi_golden.py

Arguments: a few per Chebyshev interval of the library's tables (seeded), the
interval boundaries and their floating-point neighbours, the series region
below -4, the asymptotic region above 100, and the special values (+-0,
+-inf, NaN, huge).  Stored per twice-order k2 (-9, -7, ..., -1, 0, ..., 21):

  x            the arguments (shared by every order)
  ref_<k2>     the reference's FDI_* of x (oracle/_ref, compiled from the
               reference headers)
  mp_<k2>      F_{k2/2}(x) = -Gamma(k2/2 + 1) Li_{k2/2+1}(-e^x) from mpmath at
               34 digits, rounded to double (NaN where x is not finite or
               below -1e4)
  scale_<k2>   max |F| over [x - 1, x + 1] (mpmath): the size the error of an
               approximation is measured against near the zeros of the
               negative orders
"""

import ctypes
import multiprocessing as mproc
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from bns_nurates_gb300 import fdi_tables as ft  # noqa: E402
from oracle import build_ref  # noqa: E402

SEED = 20261204


def arguments():
    rng = np.random.default_rng(SEED)
    xs = [rng.uniform(-60.0, ft.X_LO, 24), rng.uniform(-745.0, -60.0, 4)]
    for i in range(ft.PIECES):
        c, h = ft.piece(i)
        xs.append(rng.uniform(c - h, c + h, 4))
    edges = [ft.X_LO + ft.WIDTH * i for i in range(ft.NARROW + 1)]
    edges += [ft.X_MID + ft.WIDE * i for i in range(1, ft.PIECES - ft.NARROW + 1)]
    edges = np.array(edges)
    xs += [edges, np.nextafter(edges, -np.inf), np.array([-2.0, np.nextafter(-2.0, 0.0)])]
    xs.append(np.exp(rng.uniform(np.log(100.0), np.log(1e4), 16)))
    xs.append(np.array([0.0, -0.0, 1e-300, -1e-300, 1e5, 1e6, 1e30, 1e300, -1e300,
                        np.inf, -np.inf, np.nan]))
    return np.concatenate(xs)


def _truth(args):
    k2, x = args
    if not np.isfinite(x) or x < -1e4:
        return np.nan, np.nan
    v = float(ft.f_mp(k2 / 2, float(x)))
    win = [abs(float(ft.f_mp(k2 / 2, float(x) + d))) for d in np.linspace(-1.0, 1.0, 9)]
    return v, max(win + [abs(v)])


def main():
    if not build_ref.build(verbose=True):
        raise SystemExit("reference checkout not found")
    lib = ctypes.CDLL(os.path.join(build_ref.OUT, "libbnsn_ref.so"))
    lib.ref_fdi_family.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_void_p,
                                   ctypes.c_void_p]
    x = arguments()
    data = {"x": x}
    jobs = [(k2, float(v)) for k2 in ft.FAMILY2 for v in x]
    with mproc.get_context("spawn").Pool(os.cpu_count()) as pool:
        res = pool.map(_truth, jobs, chunksize=16)
    for n, k2 in enumerate(ft.FAMILY2):
        out = np.empty_like(x)
        if lib.ref_fdi_family(k2, x.size, x.ctypes.data, out.ctypes.data) != 0:
            raise RuntimeError(f"order {k2} missing from the reference")
        r = res[n * x.size:(n + 1) * x.size]
        data[f"ref_{k2}"] = out
        data[f"mp_{k2}"] = np.array([v for v, _ in r])
        data[f"scale_{k2}"] = np.array([s for _, s in r])
    np.savez_compressed(os.path.join(HERE, "fdi_family.npz"), **data)
    print("wrote fdi_family.npz:", x.size, "arguments x", len(ft.FAMILY2), "orders")


if __name__ == "__main__":
    main()
