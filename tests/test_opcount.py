"""The op-counting build of the reference (oracle/opcount.py), whose counts
are the benchmark's algorithmic work per point (profiles/op_counts.json).

The counting real type must not change what the reference computes: its
outputs are compared bit for bit with the plain build of the same headers.
"""

import json
import os

import numpy as np
import pytest

from conftest import REPO


def test_committed_table_covers_the_bench_phases():
    with open(os.path.join(REPO, "profiles", "op_counts.json")) as f:
        t = json.load(f)
    for wl, phases in (("c5", ("prelude", "pair", "brem", "neps")),
                       ("c3", ("prelude", "pair", "brem"))):
        for ph in phases:
            assert t[wl]["phases"][ph]["work"] > 0, (wl, ph)
        assert t[wl]["outputs_equal_plain_build"] == 1.0


def test_counting_build_computes_what_the_reference_computes(port, ref):
    import ctypes
    from oracle import opcount
    lib = ctypes.CDLL(opcount.build())
    eos, m1 = port.synthetic_points(4242, 24, first=500)
    for flags, pars, nq in (((1, 1, 1, 1, 1), (1, 0, 1, 1, 1, 2, 1, 0), 8),
                            ((1, 1, 1, 0, 1), (1, 0, 1, 1, 1, 0, 1, 0), 10),
                            ((0, 1, 1, 0, 0), (0, 1, 0, 0, 0, 1, 0, 1), 6)):
        x, w = port.gauss_legendre(nq)
        calls, counts, nuf, out = opcount.count(lib, eos, m1, flags, pars, x, w)
        want = ref.m1_opacities(eos, m1, flags, pars, (x, w))
        assert np.array_equal(out, want)
        assert calls[opcount.COUNTED.index("distr")] == 1.0
        if flags[1]:
            # the reference evaluates each unordered cell pair once: M(M+1)/2
            m = 2 * nq
            assert calls[opcount.COUNTED.index("PairKernels")] == m * (m + 1) / 2
        assert 0 < nuf <= calls[opcount.COUNTED.index("TotalNuF")]
