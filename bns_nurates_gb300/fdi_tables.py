"""Coefficient tables of the Fermi-Dirac integral family F_j, j = -9/2 ... 21/2.

F_j(x) = integral_0^inf t^j / (exp(t - x) + 1) dt for j > -1, without the
1 / Gamma(j + 1) normalisation (the convention of functions.hpp:442-4375),
continued to j < -1 by dF_{j+1}/dx = (j + 1) F_j; for every j,
F_j(x) = -Gamma(j + 1) Li_{j+1}(-e^x).

The integer orders 0..5 are evaluated by the library's restatement of the
reference's rational approximations (bnsn_fp64.cuh).  Every other member of
the family the reference defines (FDI_m92 .. FDI_m12, FDI_p12 .. FDI_p212 and
FDI_p6 .. FDI_p10) is evaluated in three regimes with tables made here:

  x < -4        : the alternating series
                  sum_{n=1}^{16} (-1)^{n+1} Gamma(j+1) n^{-(j+1)} e^{n x},
                  in Horner form in -e^x
  -4 <= x < 100 : 28 Chebyshev expansions of degree 24, one per interval:
                  [-4 + 2i, -2 + 2i] below 40, [40 + 10i, 50 + 10i] above (the
                  only singularities of F_j are at x = +-i pi, +-3i pi, ..., so
                  on the narrow intervals the coefficients fall by >= 6.7 per
                  degree and on the wide ones by >= 18)
  x >= 100      : the Sommerfeld expansion
                  x^{j+1} / (j+1) (1 + sum_k 2 eta(2k) (j+1)(j)...(j+2-2k) x^{-2k}),
                  12 terms; the truncation and the exponentially small
                  remainder are below 1e-20 of the leading term; x^{j+1}
                  by repeated squaring times sqrt(x) for half-integer j

``generate()`` computes the coefficients with mpmath at 34 digits and writes
csrc/bnsn_fdi_tab.h (checked in; mpmath is only needed to regenerate it).
``load_header()`` and ``evaluate()`` are the same evaluation in numpy (FP64),
used by the CPU tests to check the tables without a GPU.

Regenerate with:  python bns_nurates_gb300/fdi_tables.py
"""

import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(HERE, "csrc", "bnsn_fdi_tab.h")

# Twice the order of each table slot: the half-integers -9/2 .. 21/2 and the
# integers 6 .. 10 (0 .. 5 have their own rational approximations).
ORDERS2 = (-9, -7, -5, -3, -1, 1, 3, 5, 7, 9, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21)
# Every twice-order of the family (functions.hpp:442-4375).
FAMILY2 = (-9, -7, -5, -3, -1) + tuple(range(0, 22))

SERIES_TERMS = 16
X_LO, X_MID, X_HI = -4.0, 40.0, 100.0
WIDTH, WIDE = 2.0, 10.0
NARROW = int((X_MID - X_LO) / WIDTH)
PIECES = NARROW + int((X_HI - X_MID) / WIDE)
CHEB_TERMS = 25
CHEB_NODES = 40
ASYM_TERMS = 12
DPS = 34


def _mp():
    import mpmath

    mpmath.mp.dps = DPS
    return mpmath


def f_mp(j, x):
    """F_j(x) in mpmath (the unnormalised convention): the alternating series
    in e^x for x < -1 (mpmath's polylog loses the tiny values of order 1 to
    its log(1 - z) form), the Sommerfeld series for x > 200 (its remainder is
    of order e^-x) and -Gamma(j+1) Li_{j+1}(-e^x) in between."""
    mp = _mp()
    j = mp.mpf(j)
    x = mp.mpf(x)
    if x < -1:
        e, s, n = mp.exp(x), mp.mpf(0), 1
        while True:
            t = mp.power(e, n) * mp.power(n, -(j + 1))
            s += t if n % 2 else -t
            if abs(t) < abs(s) * mp.mpf(10) ** (-DPS - 2):
                break
            n += 1
        return mp.gamma(j + 1) * s
    if x > 200:
        u, s, fall = 1 / (x * x), mp.mpf(1), mp.mpf(1)
        for k in range(1, 60):
            fall *= (j + 1 - (2 * k - 2)) * (j + 1 - (2 * k - 1))
            t = 2 * mp.altzeta(2 * k) * fall * mp.power(u, k)
            s += t
            if abs(t) < mp.mpf(10) ** (-DPS - 2):
                break
        return mp.power(x, j + 1) / (j + 1) * s
    return mp.re(-mp.gamma(j + 1) * mp.polylog(j + 1, -mp.exp(x)))


def _series(j):
    mp = _mp()
    g = mp.gamma(mp.mpf(j) + 1)
    return [float(g * mp.power(n, -(mp.mpf(j) + 1))) for n in range(1, SERIES_TERMS + 1)]


def _cheb_piece(args):
    j, i = args
    mp = _mp()
    centre, half = (mp.mpf(c) for c in piece(i))
    th = [mp.pi * (k + mp.mpf(0.5)) / CHEB_NODES for k in range(CHEB_NODES)]
    fv = [f_mp(j, centre + half * mp.cos(t)) for t in th]
    out = []
    for m in range(CHEB_TERMS):
        c = 2 * mp.fsum(fv[k] * mp.cos(m * th[k]) for k in range(CHEB_NODES)) / CHEB_NODES
        out.append(float(c / 2 if m == 0 else c))
    return j, i, out


def piece(i):
    """Centre and half-width of Chebyshev interval i."""
    if i < NARROW:
        return X_LO + WIDTH * i + WIDTH / 2, WIDTH / 2
    return X_MID + WIDE * (i - NARROW) + WIDE / 2, WIDE / 2


def _asym(j):
    """2 eta(2k) (j+1) j ... (j+2-2k), k = 1..ASYM_TERMS (eta: Dirichlet eta)."""
    mp = _mp()
    j1 = mp.mpf(j) + 1
    out, fall = [], mp.mpf(1)
    for k in range(1, ASYM_TERMS + 1):
        fall *= (j1 - (2 * k - 2)) * (j1 - (2 * k - 1))
        out.append(float(2 * mp.altzeta(2 * k) * fall))
    return out


def _hex_rows(rows, indent):
    return (",\n" + indent).join("{" + ", ".join(float(v).hex() for v in r) + "}" for r in rows)


def generate(path=HEADER, workers=None):
    import multiprocessing as mproc

    mp = _mp()
    jobs = [(k2 / 2, i) for k2 in ORDERS2 for i in range(PIECES)]
    ctx = mproc.get_context("spawn")
    with ctx.Pool(workers or os.cpu_count()) as pool:
        res = pool.map(_cheb_piece, jobs, chunksize=4)
    cheb = {(j, i): c for j, i, c in res}
    lines = [
        "// Generated by bns_nurates_gb300/fdi_tables.py (mpmath %s, %d digits); do not edit."
        % (mp.__version__, DPS),
        "// Tables of the Fermi-Dirac integral family evaluated by fdi.cu:",
        "// alternating-series coefficients (x < -4), Chebyshev coefficients of",
        "// the intervals of [-4, 100) and Sommerfeld coefficients (x >= 100).",
        "#pragma once",
        "",
        "namespace bnsn {",
        "namespace fdit {",
        "",
        "constexpr int kNumOrders   = %d;" % len(ORDERS2),
        "constexpr int kSeriesTerms = %d;" % SERIES_TERMS,
        "constexpr int kPieces      = %d;" % PIECES,
        "constexpr int kChebTerms   = %d;" % CHEB_TERMS,
        "constexpr int kAsymTerms   = %d;" % ASYM_TERMS,
        "constexpr int kNarrow      = %d;" % NARROW,
        "constexpr double kXlo = %r, kXmid = %r, kXhi = %r;" % (X_LO, X_MID, X_HI),
        "constexpr double kWidth = %r, kWide = %r;" % (WIDTH, WIDE),
        "",
        "// twice the order of each slot",
        "constexpr int kTwice[kNumOrders] = {%s};" % ", ".join(str(k) for k in ORDERS2),
        "",
        "// Gamma(j + 1) n^-(j + 1), n = 1..kSeriesTerms",
        "__device__ const double kSeries[kNumOrders][kSeriesTerms] = {",
        "    " + _hex_rows([_series(k2 / 2) for k2 in ORDERS2], "    ") + "};",
        "",
        "// Chebyshev coefficients c_0 .. c_24 of F_j on interval i, c_0 halved:",
        "// [-4 + 2i, -2 + 2i] for i < kNarrow, else [40 + 10k, 50 + 10k], k = i - kNarrow",
        "__device__ const double kCheb[kNumOrders][kPieces][kChebTerms] = {",
    ]
    for n, k2 in enumerate(ORDERS2):
        rows = [cheb[(k2 / 2, i)] for i in range(PIECES)]
        lines.append("    {" + _hex_rows(rows, "     ") + "}" + ("," if n + 1 < len(ORDERS2) else ""))
    lines += [
        "};",
        "",
        "// 2 eta(2k) (j+1) j ... (j+2-2k), k = 1..kAsymTerms",
        "__device__ const double kAsym[kNumOrders][kAsymTerms] = {",
        "    " + _hex_rows([_asym(k2 / 2) for k2 in ORDERS2], "    ") + "};",
        "",
        "} // namespace fdit",
        "} // namespace bnsn",
        "",
    ]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def load_header(path=HEADER):
    """The tables of csrc/bnsn_fdi_tab.h as numpy arrays (exact, hex literals)."""
    with open(path) as f:
        text = f.read()

    def block(name):
        m = re.search(r"%s\[[^=]*=\s*\{(.*?)\};" % name, text, re.S)
        vals = re.findall(r"-?0x[0-9a-fA-Fp.+-]+|-?inf|nan", m.group(1))
        return np.array([float.fromhex(v) for v in vals])

    n = len(ORDERS2)
    return {
        "series": block("kSeries").reshape(n, SERIES_TERMS),
        "cheb": block("kCheb").reshape(n, PIECES, CHEB_TERMS),
        "asym": block("kAsym").reshape(n, ASYM_TERMS),
    }


def pow_half(x, h):
    """x^(h/2) as the kernel forms it: an integer power by repeated squaring,
    times sqrt(x) for odd h, inverted for negative h."""
    a = abs(h)
    q = a >> 1
    v = np.ones_like(x)
    b = x.copy()
    while q:
        if q & 1:
            v = v * b
        q >>= 1
        if q:
            b = b * b
    if a & 1:
        v = v * np.sqrt(x)
    return 1.0 / v if h < 0 else v


def evaluate(k2, x, tabs):
    """F_{k2/2}(x) for a table order, in FP64 with the kernel's operation order."""
    slot = ORDERS2.index(k2)
    x = np.asarray(x, dtype=np.float64)
    out = np.empty_like(x)
    j1 = 0.5 * k2 + 1.0
    lo = x < X_LO
    hi = x >= X_HI
    mid = ~(lo | hi | np.isnan(x))
    with np.errstate(over="ignore", invalid="ignore", divide="ignore", under="ignore"):
        e = np.exp(x[lo])
        z = -e
        c = tabs["series"][slot]
        p = np.full_like(z, c[-1])
        for n in range(SERIES_TERMS - 2, -1, -1):
            p = p * z + c[n]
        out[lo] = e * p
        xm = x[mid]
        i = np.where(xm < X_MID, np.floor((xm - X_LO) * (1.0 / WIDTH)),
                     NARROW + np.floor((xm - X_MID) * (1.0 / WIDE)))
        i = np.clip(i.astype(np.int64), 0, PIECES - 1)
        narrow = i < NARROW
        cen = np.where(narrow, X_LO + WIDTH * i + WIDTH / 2,
                       X_MID + WIDE * (i - NARROW) + WIDE / 2)
        t = (xm - cen) * np.where(narrow, 2.0 / WIDTH, 2.0 / WIDE)
        cc = tabs["cheb"][slot][i]
        b1 = np.zeros_like(t)
        b2 = np.zeros_like(t)
        t2 = 2.0 * t
        for m in range(CHEB_TERMS - 1, 0, -1):
            b0 = t2 * b1 + (cc[:, m] - b2)
            b2, b1 = b1, b0
        out[mid] = t * b1 + (cc[:, 0] - b2)
        xh = x[hi]
        u = 1.0 / (xh * xh)
        a = tabs["asym"][slot]
        s = np.full_like(u, a[-1])
        for k in range(ASYM_TERMS - 2, -1, -1):
            s = s * u + a[k]
        s = s * u + 1.0
        out[hi] = pow_half(xh, k2 + 2) / j1 * s
    nan = np.isnan(x)
    out[nan] = 0.0 if k2 % 2 == 0 else np.nan
    return out


if __name__ == "__main__":
    generate()
    print("wrote", HEADER)
