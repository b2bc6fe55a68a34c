"""The C ABI without a GPU: library loads, exports every declared entry point,
keeps the reference's struct layouts, validates arguments, and its host
utilities (quadrature, workload generator) behave."""

import ctypes
import json
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO

HEADER = os.path.join(REPO, "include", "bns_nurates_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    # declarations only: comments may name types or functions in prose
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    return sorted(set(re.findall(r"\b(bnsn_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 12
    for name in names:
        assert hasattr(lib, name), name


def test_ctypes_layout_matches_reference(lib):
    import bns_nurates_gb300._capi as C
    with open(os.path.join(GOLDEN, "layout.json")) as f:
        lay = json.load(f)
    for sname, fields in lay.items():
        cls = getattr(C, sname)
        assert ctypes.sizeof(cls) == fields["__size__"], sname
        for fname, off in fields.items():
            if fname.startswith("__"):
                continue
            assert getattr(cls, fname).offset == off, (sname, fname)


def test_c_header_layout_matches_reference(tmp_path):
    """Compile a probe against include/bns_nurates_gb300.h with the C compiler
    and compare sizeof/offsetof with the reference's (golden/layout.json)."""
    with open(os.path.join(GOLDEN, "layout.json")) as f:
        lay = json.load(f)
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "bns_nurates_gb300.h"',
             'int main(void) {']
    for sname, fields in lay.items():
        lines.append(f'printf("{sname} __size__ %zu\\n", sizeof({sname}));')
        for fname in fields:
            if not fname.startswith("__"):
                lines.append(f'printf("{sname} {fname} %zu\\n", offsetof({sname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o",
                           str(exe)])
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        sname, fname, val = line.split()
        assert int(val) == lay[sname][fname], line


def test_gauss_legendre_matches_oracle_bitwise(lib, port):
    import bns_nurates_gb300 as bn
    for n in (1, 2, 3, 6, 10, 16, 20):
        q = bn.gauss_legendre(n)
        x, w = bn.quad_arrays(q)
        xo, wo = port.gauss_legendre(n)
        assert np.array_equal(x, xo) and np.array_equal(w, wo)
    with pytest.raises(bn.BnsnError):
        bn.gauss_legendre(0)
    with pytest.raises(bn.BnsnError):
        bn.gauss_legendre(21)


def test_synthetic_points_deterministic_and_plausible(lib):
    import bns_nurates_gb300 as bn
    eos, m1 = bn.synthetic_points(11, 3000)
    eos2, m12 = bn.synthetic_points(11, 3000, nthreads=3)
    assert np.array_equal(eos, eos2) and np.array_equal(m1, m12)
    e3, m3 = bn.synthetic_points(11, 1000, first=2000)      # point k depends on (seed, k)
    assert np.array_equal(e3, eos[:, 2000:]) and np.array_equal(m3, m1[:, 2000:])
    assert np.isfinite(eos).all() and np.isfinite(m1).all()
    rho = eos[0] * 1e21 * 1.66053906892e-24
    assert rho.min() >= 1e6 * (1 - 1e-12) and rho.max() <= 1e15 * (1 + 1e-12)
    assert eos[1].min() >= 0.5 and eos[1].max() <= 100.
    assert eos[2].min() >= 0.01 and eos[2].max() <= 0.6
    assert np.all(eos[7] > 0.)                       # net electron density > 0
    assert np.all(np.abs(eos[9]) <= 20.)
    assert np.all(m1[8:] >= 1. / 3.) and np.all(m1[8:] <= 1.)
    assert np.array_equal(m1[3], m1[2]) and np.array_equal(m1[7], m1[6])


def test_argument_errors_without_device(lib):
    """Bad arguments are rejected before any device is touched."""
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import _capi as C
    q = bn.gauss_legendre(10)
    fl, pa = bn.opacity_flags(), bn.opacity_params()
    eos, m1 = C.EosSoA(), C.M1SoA()
    out = C.M1OpacitiesSoA()
    f = lib.bnsn_m1_opacities
    # NULL output struct
    assert f(ctypes.byref(q), ctypes.byref(q), ctypes.byref(fl), ctypes.byref(pa),
             ctypes.byref(eos), ctypes.byref(m1), None, 1, 0, None, 10, None) == C.ERR_ARG
    # NULL field pointers with npts > 0
    assert f(ctypes.byref(q), ctypes.byref(q), ctypes.byref(fl), ctypes.byref(pa),
             ctypes.byref(eos), ctypes.byref(m1), None, 1, 0, ctypes.byref(out), 10,
             None) == C.ERR_ARG
    # quadrature order out of range
    bad = bn.gauss_legendre(10)
    bad.nx = 21
    assert f(ctypes.byref(bad), ctypes.byref(q), ctypes.byref(fl), ctypes.byref(pa),
             ctypes.byref(eos), ctypes.byref(m1), None, 1, 0, ctypes.byref(out), 10,
             None) == C.ERR_NQUAD
    # unknown precision / stim flag / brem implementation
    assert f(ctypes.byref(q), ctypes.byref(q), ctypes.byref(fl), ctypes.byref(pa),
             ctypes.byref(eos), ctypes.byref(m1), None, 1, 7, ctypes.byref(out), 10,
             None) == C.ERR_ARG
    assert f(ctypes.byref(q), ctypes.byref(q), ctypes.byref(fl), ctypes.byref(pa),
             ctypes.byref(eos), ctypes.byref(m1), None, 3, 0, ctypes.byref(out), 10,
             None) == C.ERR_ARG
    pb = bn.opacity_params(brem_implementation=5)
    assert f(ctypes.byref(q), ctypes.byref(q), ctypes.byref(fl), ctypes.byref(pb),
             ctypes.byref(eos), ctypes.byref(m1), None, 1, 0, ctypes.byref(out), 10,
             None) == C.ERR_ARG
    assert b"brem" in lib.bnsn_last_error()
    assert lib.bnsn_status_string(C.ERR_NQUAD) == b"quadrature order out of range"
    # negative energies for the spectral call
    e = (ctypes.c_double * 2)(1.0, -2.0)
    so = C.SpectralSoA()
    assert lib.bnsn_spectral_opacities(ctypes.byref(q), ctypes.byref(fl), ctypes.byref(pa),
                                       ctypes.byref(eos), ctypes.byref(m1), None, e, 2, 1, 0,
                                       ctypes.byref(so), 10, None) == C.ERR_ARG
    # GP19 table validation (non-increasing axis)
    dims = (ctypes.c_int * 4)(2, 2, 2, 2)
    ax = (ctypes.c_double * 2)(1.0, 0.5)
    data = (ctypes.c_double * 16)()
    assert lib.bnsn_gp19_set_table(dims, ax, ax, ax, ax, None, None, data) == C.ERR_ARG


def test_oracle_header_states_role():
    """The oracle sources say they are test infrastructure."""
    for name in ("bnsn_oracle.c", "ref_driver.cpp", "__init__.py"):
        text = open(os.path.join(REPO, "oracle", name)).read()
        assert re.search(r"test infrastructure", text, re.I), name


def test_product_does_not_import_oracle():
    pkg = os.path.join(REPO, "bns_nurates_gb300")
    for root, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(root, fn)).read()
                assert "import oracle" not in text and "from oracle" not in text, fn
                assert "libbnsn_oracle" not in text and "libbnsn_ref" not in text, fn
