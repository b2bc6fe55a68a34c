"""The mixed path's NES/NPS out-kernel integrals (bnsn_nes_m_mixed) against
exact values of the reference's MezzacappaIntOut (kernel_nes.hpp:31-78),
evaluated with mpmath at up to ~250 digits on pairs of the NES quadrature grid
and their reverses at eta from -40 to 300 (tests/golden/nes_m.npz,
tests/golden/make_nes_golden.py).  The reference's FP64 formula cancels
catastrophically on many of these; the FP32 integral must be within 6e-7
relative of the exact value on every one, with the right sign."""

import numpy as np
import pytest

import bns_nurates_gb300 as bn
from conftest import golden

pytestmark = pytest.mark.gpu

TOL = 6e-7


def test_nes_integral_vs_exact(cuda):
    g = golden("nes_m.npz")
    t = lambda a: cuda.from_numpy(np.ascontiguousarray(a)).cuda()
    m1, m2, ls = bn.nes_m_mixed(t(g["w"]), t(g["wp"]), t(g["eta"]))
    cuda.cuda.synchronize()
    ls = ls.cpu().numpy()
    for m, ln_true, s_true, name in ((m1, g["ln_m1"], g["s_m1"], "b1 part"),
                                     (m2, g["ln_m2"], g["s_m2"], "b2 part")):
        m = m.cpu().numpy()
        assert (np.sign(m) == s_true).all(), name
        err = np.abs(np.expm1(np.log(np.abs(m)) + ls - ln_true))
        k = int(np.argmax(err))
        assert err.max() <= TOL, (f"{name}: rel err {err[k]:.3e} at w={g['w'][k]:.6g} "
                                  f"w'={g['wp'][k]:.6g} eta={g['eta'][k]:.6g}")


def test_nes_integral_reverse_is_negative(cuda):
    """MezzacappaIntOut(w', w) = -MezzacappaIntOut(w, w')."""
    w = cuda.tensor([0.3, 2.0, 7.5], dtype=cuda.float64, device="cuda")
    wp = cuda.tensor([1.1, 0.4, 9.0], dtype=cuda.float64, device="cuda")
    eta = cuda.tensor([3.0, -2.0, 40.0], dtype=cuda.float64, device="cuda")
    a1, a2, la = bn.nes_m_mixed(w, wp, eta)
    b1, b2, lb = bn.nes_m_mixed(wp, w, eta)
    assert cuda.equal(la, lb)
    assert cuda.allclose(a1, -b1, rtol=1e-6) and cuda.allclose(a2, -b2, rtol=1e-6)
