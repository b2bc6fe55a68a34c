"""The Fermi-Dirac integral family (functions.hpp:442-4375, FDI_m92 .. FDI_p212).

Fixture: tests/golden/fdi_family.npz (tests/golden/make_fdi_golden.py) holds
the reference's own FDI_* values (compiled reference) and mpmath values at
34 digits on 228 arguments covering every regime.  Errors are measured
against max(|F|, scale) where scale (negative orders only) is max |F| over
[x - 1, x + 1]: F_{-5/2}, F_{-7/2} and F_{-9/2} cross zero, and there an
approximation's error is set by the size of the function around the zero.

CPU: the fixture pins the reference to mpmath; the library's tables
(bns_nurates_gb300/csrc/bnsn_fdi_tab.h), evaluated in numpy with the kernel's
operation order, are checked against both.  GPU: bnsn_fdi / bnsn_fdi_host of
every order against the reference's values, including the non-finite
arguments.
"""

import ctypes

import numpy as np
import pytest

from conftest import golden

from bns_nurates_gb300 import fdi_tables as ft

# Reference vs mpmath: a few 1e-16 (Fukushima's approximations are good to
# about 1e-15); the library's tables are built to the same level.
TOL_PIN = 2e-15
TOL_TAB = 1.5e-15
TOL_GPU = 3e-15


def _fixture():
    return golden("fdi_family.npz")


def _norm_err(a, b, k2, scale):
    den = np.abs(b)
    if k2 < 0:
        den = np.maximum(den, scale)
    with np.errstate(invalid="ignore", divide="ignore"):
        e = np.abs(a - b) / den
    e[(a == b)] = 0.0
    return e


def _same_nonfinite(a, b):
    """NaN where the other is NaN; infinities and zeros equal (sign included)."""
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    m = ~na & (~np.isfinite(b) | (b == 0))
    return np.array_equal(a[m], b[m]) and np.array_equal(np.signbit(a[m]), np.signbit(b[m]))


def test_reference_pinned_to_mpmath():
    d = _fixture()
    x = d["x"]
    for k2 in ft.FAMILY2:
        ref, mp, sc = d[f"ref_{k2}"], d[f"mp_{k2}"], d[f"scale_{k2}"]
        m = np.isfinite(mp) & np.isfinite(ref)
        e = _norm_err(ref[m], mp[m], k2, sc[m])
        assert e.max() <= TOL_PIN, (k2, float(e.max()), float(x[m][e.argmax()]))


def test_tables_match_mpmath_and_reference():
    d = _fixture()
    x = d["x"]
    tabs = ft.load_header()
    for k2 in ft.ORDERS2:
        mine = ft.evaluate(k2, x, tabs)
        ref, mp, sc = d[f"ref_{k2}"], d[f"mp_{k2}"], d[f"scale_{k2}"]
        m = np.isfinite(mp) & np.isfinite(mine)
        e = _norm_err(mine[m], mp[m], k2, sc[m])
        assert e.max() <= TOL_TAB, (k2, float(e.max()), float(x[m][e.argmax()]))
        f = np.isfinite(ref) & (ref != 0)
        e2 = _norm_err(mine[f], ref[f], k2, np.nan_to_num(sc[f], nan=0.0))
        assert e2.max() <= TOL_PIN + TOL_TAB, (k2, float(e2.max()))
        assert _same_nonfinite(mine[~f], ref[~f]), k2


def test_table_regime_edges_are_continuous():
    """Both sides of every regime and interval boundary agree to the table
    accuracy (no jump between Chebyshev intervals)."""
    tabs = ft.load_header()
    edges = [ft.X_LO + ft.WIDTH * i for i in range(ft.NARROW + 1)]
    edges += [ft.X_MID + ft.WIDE * i for i in range(1, ft.PIECES - ft.NARROW + 1)]
    edges = np.array(edges)
    below = np.nextafter(edges, -np.inf)
    for k2 in ft.ORDERS2:
        a = ft.evaluate(k2, below, tabs)
        b = ft.evaluate(k2, edges, tabs)
        scale = np.abs(b) if k2 >= 0 else np.maximum(np.abs(a), np.abs(b)) + 1e-3 * np.abs(
            ft.evaluate(k2, edges + 1.0, tabs))
        assert np.all(np.abs(a - b) <= 3e-15 * scale + 1e-300), k2


def test_fdi_rejects_bad_order(lib):
    lib.bnsn_fdi.restype = ctypes.c_int
    lib.bnsn_fdi.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                             ctypes.c_void_p]
    for k2 in (-11, -8, -2, 22, 100):
        assert lib.bnsn_fdi(k2, None, None, 0, None) != 0
    import bns_nurates_gb300 as bn
    with pytest.raises(ValueError):
        bn.api._twice_order(0.25)
    with pytest.raises(ValueError):
        bn.api._twice_order(-1.0)
    assert bn.api._twice_order(10.5) == 21


@pytest.mark.gpu
def test_gpu_fdi_family_matches_reference(cuda):
    import bns_nurates_gb300 as bn
    torch = cuda
    d = _fixture()
    x = d["x"]
    xd = torch.from_numpy(x).cuda()
    launches0 = bn.kernel_launches()
    for k2 in ft.FAMILY2:
        got = bn.fdi(k2 / 2, xd).cpu().numpy()
        ref, sc = d[f"ref_{k2}"], np.nan_to_num(d[f"scale_{k2}"], nan=0.0)
        f = np.isfinite(ref) & (ref != 0)
        e = _norm_err(got[f], ref[f], k2, sc[f])
        assert e.max() <= TOL_GPU, (k2, float(e.max()), float(x[f][e.argmax()]))
        assert _same_nonfinite(got[~f], ref[~f]), (k2, got[~f], ref[~f])
        if k2 in ft.ORDERS2:
            # the device evaluation is the numpy one up to fma rounding
            emu = ft.evaluate(k2, x, ft.load_header())
            m = np.isfinite(emu) & (emu != 0)
            e3 = _norm_err(got[m], emu[m], k2, sc[m])
            assert e3.max() <= 1e-15, (k2, float(e3.max()))
    assert bn.kernel_launches() - launches0 == len(ft.FAMILY2)


@pytest.mark.gpu
def test_gpu_fdi_host_and_large_batch(cuda):
    import bns_nurates_gb300 as bn
    torch = cuda
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-50.0, 120.0, 1 << 20), [np.nan, np.inf, -np.inf]])
    for order in (-4.5, 0.5, 3, 10.5):
        h = bn.fdi_host(order, x)
        dv = bn.fdi(order, torch.from_numpy(x).cuda()).cpu().numpy()
        assert np.array_equal(np.isnan(h), np.isnan(dv))
        m = ~np.isnan(h)
        assert np.array_equal(h[m], dv[m]), order
    # empty batch is a no-op
    assert bn.fdi_host(1.5, np.empty(0)).size == 0


def test_pow_half_accuracy():
    """x^(h/2) by repeated squaring (times sqrt(x) for odd h), the form of the
    Sommerfeld regime, stays within a few ulp of the correctly rounded power."""
    x = np.exp(np.linspace(np.log(100.0), np.log(1e25), 4001))
    for h in range(-7, 24):
        got = ft.pow_half(x, h)
        want = np.power(x, 0.5 * h)
        ok = np.isfinite(want) & (want > 0)
        r = np.abs(got[ok] - want[ok]) / want[ok]
        assert r.max() <= 8 * np.finfo(float).eps, (h, float(r.max()))


def test_aux_workload_has_no_reference_arm():
    import json
    import subprocess
    import sys
    from conftest import REPO
    out = subprocess.run([sys.executable, "bench.py", "--workload", "aux", "--impl", "reference"],
                         cwd=REPO, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line
