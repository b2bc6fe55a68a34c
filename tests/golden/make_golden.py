"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run where the reference checkout is available:  python tests/golden/make_golden.py
It builds oracle/_ref (the reference headers compiled in place, see
oracle/build_ref.py) and writes, for seeded synthetic inputs, the inputs and
the reference's outputs:

  grey_hr98_n10.npz      beta + iso + pair + HR98, n = 10, stimulated
  grey_all_hr98_n10.npz  all reactions (NES on), HR98, n = 10, stimulated
  grey_all_gp19_n20.npz  all reactions, GP19 (synthetic table), n = 20
  grey_brt06_nostim.npz  all reactions, BRT06, not stimulated, no blocking
  grey_given_distr.npz   equilibrium distribution passed in (not rebuilt)
  spectral_n10.npz       24 log-spaced energies 1-300 MeV, both forms
  point_a.npz            the reference example point (mwe.cpp:19-55)
  layout.json            sizeof/offsetof of the public structs

The synthetic inputs come from the library's seeded generator
(bnsn_synthetic_points); the fixtures store them, so the tests never need
the generator to reproduce them.
"""

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

import oracle  # noqa: E402
from oracle import build_ref  # noqa: E402

SEED = 20261203
ENERGIES = np.logspace(0.0, np.log10(300.0), 24)


def params(use_dU=1, use_dm_eff=0, use_WM_ab=1, use_WM_sc=1, use_decay=1, brem=0,
           medium=1, neglect_blocking=0):
    return [use_dU, use_dm_eff, use_WM_ab, use_WM_sc, use_decay, brem, medium,
            neglect_blocking]


def main():
    assert build_ref.build(verbose=True), "the reference checkout is required"
    oracle.build()
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import build as libbuild
    libbuild.build()
    ref = oracle.ref()
    q10 = ref.gauss_legendre(10)
    q20 = ref.gauss_legendre(20)

    def grey(name, npts, first, flags, pars, quad, stim=1, distr=False):
        eos, m1 = bn.synthetic_points(SEED, npts, first=first)
        d = None
        if distr:
            d, m1eq = ref.nu_equilibrium(eos)
            m1 = m1eq
        out = ref.m1_opacities(eos, m1, flags, pars, quad, distr=d, stim_abs=stim)
        np.savez_compressed(os.path.join(HERE, name), eos=eos, m1=m1,
                            distr=np.zeros((0,)) if d is None else d, out=out,
                            flags=np.array(flags), pars=np.array(pars), stim=stim,
                            x=quad[0], w=quad[1])
        print(name, out.shape)

    grey("grey_hr98_n10.npz", 64, 0, [1, 1, 1, 0, 1], params(), q10)
    grey("grey_all_hr98_n10.npz", 32, 1000, [1, 1, 1, 1, 1], params(), q10)
    grey("grey_all_gp19_n20.npz", 12, 2000, [1, 1, 1, 1, 1], params(brem=2), q20)
    grey("grey_brt06_nostim.npz", 16, 3000, [1, 1, 1, 1, 1],
         params(brem=1, neglect_blocking=1, use_dU=0, use_decay=0), q10, stim=0)
    grey("grey_given_distr.npz", 16, 4000, [1, 1, 1, 1, 1], params(), q10, distr=True)

    eos, m1 = bn.synthetic_points(SEED, 6, first=5000)
    flags, pars = [1, 1, 1, 1, 1], params()
    sp1 = ref.spectral(eos, m1, flags, pars, q10, ENERGIES, stimulated=1)
    sp0 = ref.spectral(eos, m1, flags, pars, q10, ENERGIES, stimulated=0)
    np.savez_compressed(os.path.join(HERE, "spectral_n10.npz"), eos=eos, m1=m1,
                        energies=ENERGIES, stim1=sp1, stim0=sp0, flags=np.array(flags),
                        pars=np.array(pars), x=q10[0], w=q10[1])
    print("spectral_n10.npz", sp1.shape)

    # mwe.cpp point A (nb in cm^-3, M1 densities in cm^-3, MeV cm^-3)
    nb, T, ye = 4.208366627847035e+38, 12.406403541564941, 0.07158458232879639
    eosA = np.array([[nb * 1e-21], [T], [ye], [ye], [1. - ye], [1.011017977368873e+03],
                     [1.221590136808168e+03], [1.871814489040245e+02], [0.],
                     [18.92714728], [280.16495513 - 278.87162217]])
    n = [3.776741015683965e+33, 1.205553071624256e+35, 2.271245089833032e+34,
         2.271245089833032e+34]
    J = [1.404570452828258e+35, 5.320827032977899e+36, 8.885618224045794e+35,
         8.885618224045794e+35]
    m1A = np.array([[v * 1e-21] for v in n] + [[v * 1e-21] for v in J] + [[1. / 3.]] * 4)
    parsA = params(use_dU=1, use_dm_eff=0, use_decay=1, brem=2)
    q6 = ref.gauss_legendre(6)
    outA = ref.m1_opacities(eosA, m1A, [1, 1, 1, 1, 1], parsA, q6)
    spA = ref.spectral(eosA, m1A, [1, 1, 1, 1, 1], parsA, q6, np.array([10.]), stimulated=0)
    np.savez_compressed(os.path.join(HERE, "point_a.npz"), eos=eosA, m1=m1A, out=outA,
                        spec=spA, pars=np.array(parsA), x=q6[0], w=q6[1])
    print("point_a.npz")

    lay = subprocess.check_output([oracle.REF_LAYOUT], text=True)
    with open(os.path.join(HERE, "layout.json"), "w") as f:
        json.dump(json.loads(lay), f, indent=1, sort_keys=True)
    print("layout.json")


if __name__ == "__main__":
    main()
