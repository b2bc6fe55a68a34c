"""Diagnostic counters: non-finite outputs (points the reference would also
fill with NaN) and the mixed spectral path's FP64 recomputations."""

import numpy as np
import pytest

import bns_nurates_gb300 as bn

pytestmark = pytest.mark.gpu


def _params(brem):
    return bn.opacity_params(True, False, True, True, True, brem_implementation=brem,
                             use_NN_medium_corr=True, neglect_blocking=False)


def test_nonfinite_counters_match_the_oracle(cuda, port):
    """Ye below the GP19 table's first Ye node makes the GP19 bracket search
    fail, which the reference turns into NaN brem kernels (and so NaN
    outputs); the counters report exactly those points and energies."""
    eos, m1 = bn.synthetic_points(4242, 64)
    bad = [3, 10, 41]
    eos[2, bad] = -0.05
    flags, pars = (1, 1, 1, 1, 1), (1, 0, 1, 1, 1, 2, 1, 0)
    energies = np.logspace(0., np.log10(300.), 12)
    e, m = cuda.from_numpy(eos).cuda(), cuda.from_numpy(m1).cuda()
    q = bn.gauss_legendre(10)
    for precision in ("fp64", "mixed"):
        bn.nonfinite_outputs(reset=True)
        grey = bn.m1_opacities(e, m, bn.opacity_flags(*flags), _params(2), q,
                               precision=precision).cpu().numpy()
        spec = bn.spectral_opacities(e, m, bn.opacity_flags(*flags), _params(2), q, energies,
                                     precision=precision).cpu().numpy()
        got = bn.nonfinite_outputs(reset=True)
        grey_bad = np.flatnonzero(~np.isfinite(grey).all(axis=0))
        spec_bad = (~np.isfinite(spec).all(axis=0)).sum()
        assert list(grey_bad) == bad, precision
        assert got == {"grey_points": len(bad), "spectral_pairs": int(spec_bad)}, precision
        assert spec_bad == len(bad) * energies.size
        assert bn.nonfinite_outputs() == {"grey_points": 0, "spectral_pairs": 0}
    # the oracle agrees on which outputs are non-finite
    want = port.m1_opacities(eos, m1, flags, pars, port.gauss_legendre(10))
    assert (np.isfinite(want) == np.isfinite(grey)).all()


def test_spectral_mixed_stats_count_every_pair(cuda):
    eos, m1 = bn.synthetic_points(17, 300)
    energies = np.logspace(0., np.log10(300.), 24)
    e, m = cuda.from_numpy(eos).cuda(), cuda.from_numpy(m1).cuda()
    bn.spectral_mixed_stats(reset=True)
    bn.spectral_opacities(e, m, bn.opacity_flags(), _params(0), bn.gauss_legendre(10), energies,
                          precision="fp64")
    assert bn.spectral_mixed_stats()["evaluated"] == 0  # the plain path does not count
    bn.spectral_opacities(e, m, bn.opacity_flags(), _params(0), bn.gauss_legendre(10), energies,
                          precision="mixed")
    st = bn.spectral_mixed_stats(reset=True)
    assert st["evaluated"] == 300 * 24
    assert st["fp64"] < st["evaluated"] // 2
    assert st["fp64"] <= st["pb_fp64"] + st["nes_fp64"]


def test_grey_mixed_stats_count_every_point(cuda):
    """The mixed grey path counts its points and the ones it hands to the
    double-float and FP64 passes; the plain path counts nothing."""
    eos, m1 = bn.synthetic_points(23, 500)
    e, m = cuda.from_numpy(eos).cuda(), cuda.from_numpy(m1).cuda()
    flags = bn.opacity_flags(use_abs_em=1, use_pair=1, use_brem=1, use_inelastic_scatt=1,
                             use_iso=1)
    bn.grey_mixed_stats(reset=True)
    bn.m1_opacities(e, m, flags, _params(0), bn.gauss_legendre(10), precision="fp64")
    assert bn.grey_mixed_stats()["evaluated"] == 0
    bn.m1_opacities(e, m, flags, _params(0), bn.gauss_legendre(10), precision="mixed")
    st = bn.grey_mixed_stats(reset=True)
    assert st["evaluated"] == 500
    for k in ("nes_df", "nes_fp64", "pair_fp64", "brem_fp64"):
        assert 0 <= st[k] < 250, (k, st)
    assert bn.grey_mixed_stats() == {"evaluated": 0, "nes_df": 0, "nes_fp64": 0,
                                     "pair_fp64": 0, "brem_fp64": 0}
