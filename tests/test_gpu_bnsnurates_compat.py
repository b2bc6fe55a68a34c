"""The reference's bindings/test_bindings.py flow through
bns_nurates_gb300.bnsnurates on the GPU: equilibrium distribution and
densities, distribution parameters from M1 moments, grey and spectral rates,
against the oracle with the conditioning probes of test_gpu_parity.py."""

import numpy as np
import pytest

import bns_nurates_gb300.bnsnurates as bns
from conftest import golden
from test_gpu_parity import COND_SPEC, assert_close, probes

pytestmark = pytest.mark.gpu

NAMES = ("nb", "temp", "ye", "yp", "yn", "mu_p", "mu_n", "mu_e", "mu_mu", "dU", "dm_eff")
BREM = {0: "HR98", 1: "BRT06", 2: "GP19"}


def _eos(col):
    e = bns.MyEOSParams()
    for k, nme in enumerate(NAMES):
        setattr(e, nme, float(col[k]))
    return e


def _dicts(pars):
    flags = {'use_abs_em': True, 'use_pair': True, 'use_brem': True,
             'use_inelastic_scatt': True, 'use_iso': True}
    keys = ('use_dU', 'use_dm_eff', 'use_WM_ab', 'use_WM_sc', 'use_decay')
    opars = {k: bool(v) for k, v in zip(keys, pars[:5])}
    opars.update(brem_implementation=BREM[int(pars[5])], use_NN_medium_corr=bool(pars[6]),
                 neglect_blocking=bool(pars[7]))
    return flags, opars


def test_bindings_flow_part2_matches_golden(cuda, port):
    """PART 2 of test_bindings.py: distribution from M1 moments, then grey and
    spectral rates of point A with dict flags and parameters."""
    g = golden("point_a.npz")
    eos = _eos(g["eos"][:, 0])
    m1 = bns.M1Quantities()
    m1.n = g["m1"][0:4, 0]
    m1.J = g["m1"][4:8, 0]
    m1.chi = g["m1"][8:12, 0]
    gp = bns.GreyOpacityParams()
    gp.eos_pars = eos
    gp.opacity_flags, gp.opacity_pars = _dicts(g["pars"])
    gp.m1_pars = m1
    gp.distr_pars = bns.CalculateDistrParamsFromM1(m1, eos)
    quad = bns.cvar.quadrature_default
    quad.nx = len(g["x"])
    bns.GaussLegendre(quad)
    try:
        rates = bns.ComputeM1Opacities(quad, quad, gp)
        spec = bns.ComputeSpectralOpacitiesNotStimulatedAbs(10., quad, gp)
    finally:
        quad.nx = 20
    got = np.array([rates[k] for k in ("eta_0", "kappa_0_a", "eta", "kappa_a", "kappa_s")])
    pfma = __import__("oracle").port_fma()
    qo = (g["x"], g["w"])
    pr = [p[:, 0] for p in probes(port.m1_opacities, pfma.m1_opacities, g["eos"], g["m1"],
                                   (1, 1, 1, 1, 1), g["pars"], qo)]
    assert_close(got.ravel(), g["out"][:, 0], pr, what="point A grey (dict API)")
    got = np.array([spec[k] for k in ("j", "kappa", "j_s", "kappa_s")]).ravel()
    pr = [p[:, 0, 0] for p in probes(port.spectral, pfma.spectral, g["eos"], g["m1"],
                                      (1, 1, 1, 1, 1), g["pars"], qo, np.array([10.]),
                                      stimulated=0)]
    assert_close(got, g["spec"][:, 0, 0], pr, what="point A spectral (dict API)",
                 cond=COND_SPEC)


def test_bindings_flow_part1_equilibrium(cuda, port):
    """PART 1: NuEquilibriumParams + ComputeM1DensitiesEq, then grey rates."""
    eos_a, _ = port.synthetic_points(11, 4)
    want_d, want_m1 = port.nu_equilibrium(eos_a)
    pars = (1, 0, 1, 1, 1, 0, 1, 0)
    for p in range(eos_a.shape[1]):
        eos = _eos(eos_a[:, p])
        d = bns.NuEquilibriumParams(eos)
        m1 = bns.M1Quantities()
        bns.ComputeM1DensitiesEq(eos, d, m1)
        m1.chi = [1. / 3.] * 4
        np.testing.assert_allclose(m1.n, want_m1[0:4, p], rtol=1e-13)
        np.testing.assert_allclose(m1.J, want_m1[4:8, p], rtol=1e-13)
        gp = bns.GreyOpacityParams()
        gp.eos_pars = eos
        gp.opacity_flags, gp.opacity_pars = _dicts(pars)
        gp.distr_pars = d
        gp.m1_pars = m1
        quad = bns.MyQuadrature()
        quad.nx, quad.x1, quad.x2, quad.dim = 10, 0., 1., 1
        bns.GaussLegendre(quad)
        got = bns.ComputeM1Opacities(quad, quad, gp)
        qx = (np.array(quad.points[:10]), np.array(quad.w[:10]))
        m1c = np.concatenate([m1.n, m1.J, m1.chi])[:, None]
        want = port.m1_opacities(eos_a[:, p:p + 1], m1c, (1, 1, 1, 1, 1), pars, qx,
                                 distr=want_d[:, p:p + 1])[:, 0]
        pfma = __import__("oracle").port_fma()
        pr = [q[:, 0] for q in probes(port.m1_opacities, pfma.m1_opacities, eos_a[:, p:p + 1],
                                      m1c, (1, 1, 1, 1, 1), pars, qx,
                                      distr=want_d[:, p:p + 1])]
        out = np.array([got[k] for k in ("eta_0", "kappa_0_a", "eta", "kappa_a", "kappa_s")])
        assert_close(out.ravel(), want, pr, what=f"equilibrium point {p}")
