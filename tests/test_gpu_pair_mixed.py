"""The mixed path's pair-annihilation integrals (bnsn_pair_j_mixed) against
exact values of the reference's PairPsi / (1 - e^{y+z}) (kernel_pair.hpp:
16-120), evaluated with mpmath at up to ~200 digits on quadrature-grid cells
(tests/golden/pair_j.npz, tests/golden/make_pair_golden.py).  The reference's
FP64 formula cancels catastrophically on many of these cells; the FP32
integral must be within 6e-7 relative of the exact value on every one (its
polynomial coefficients carry y and z rounded to FP32)."""

import numpy as np
import pytest

import bns_nurates_gb300 as bn
from conftest import golden

pytestmark = pytest.mark.gpu

TOL = 6e-7


def test_pair_integral_vs_exact(cuda):
    g = golden("pair_j.npz")
    t = lambda a: cuda.from_numpy(np.ascontiguousarray(a)).cuda()
    j0, j1, ls = bn.pair_j_mixed(t(g["y"]), t(g["z"]), t(g["eta"]))
    cuda.cuda.synchronize()
    ls = ls.cpu().numpy()
    for j, ln_true, name in ((j0, g["ln_j0"], "J0"), (j1, g["ln_j1"], "J1")):
        got = np.log(j.cpu().numpy()) + ls
        err = np.abs(np.expm1(got - ln_true))
        k = int(np.argmax(err))
        assert err.max() <= TOL, (f"{name}: rel err {err[k]:.3e} at y={g['y'][k]:.6g} "
                                  f"z={g['z'][k]:.6g} eta={g['eta'][k]:.6g}")


def test_pair_integral_zero_beyond_reference_cut(cuda):
    """eta - y - z > 200: the reference sets PairPsi to zero."""
    y = cuda.tensor([0.5, 1.0], dtype=cuda.float64, device="cuda")
    j0, j1, _ = bn.pair_j_mixed(y, y, cuda.tensor([250., 202.5], dtype=cuda.float64,
                                                  device="cuda"))
    assert j0.cpu().numpy().tolist() == [0., 0.] and j1.cpu().numpy().tolist() == [0., 0.]
