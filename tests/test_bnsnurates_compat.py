"""The SWIG-module conventions of bns_nurates_gb300.bnsnurates (the
reference's bindings/bnsnurates.i): dict flags and parameters with a string
brem implementation, list-valued arrays, the module's default quadrature and
the equilibrium distribution parameters.  Host-side parts only."""

import numpy as np
import pytest

import bns_nurates_gb300.bnsnurates as bns


def test_flags_and_params_dicts_round_trip():
    gp = bns.GreyOpacityParams()
    flags = {'use_abs_em': True, 'use_pair': False, 'use_brem': True,
             'use_inelastic_scatt': False, 'use_iso': True}
    gp.opacity_flags = flags
    assert gp.opacity_flags == {k: int(v) for k, v in flags.items()}
    pars = {'use_dU': True, 'use_dm_eff': False, 'use_WM_ab': True, 'use_WM_sc': False,
            'use_decay': True, 'brem_implementation': 'BRT06', 'neglect_blocking': False,
            'use_NN_medium_corr': True}
    gp.opacity_pars = pars
    got = gp.opacity_pars
    assert got['brem_implementation'] == 'BRT06'
    assert {k: v for k, v in got.items() if k != 'brem_implementation'} == \
        {k: int(v) for k, v in pars.items() if k != 'brem_implementation'}
    # the C struct underneath holds the enum value
    raw = super(bns.GreyOpacityParams, gp).__getattribute__('opacity_pars')
    assert raw.brem_implementation == 1 and raw.use_dU and not raw.use_WM_sc


@pytest.mark.parametrize("name, value", [("HR98", 0), ("BRT06", 1), ("GP19", 2),
                                         ("GP19_table", 2), ("other", 0)])
def test_brem_implementation_by_prefix(name, value):
    p = bns.opacity_params_from_dict({'use_dU': 1, 'use_dm_eff': 0, 'use_WM_ab': 1,
                                      'use_WM_sc': 1, 'use_decay': 1,
                                      'brem_implementation': name, 'neglect_blocking': 0,
                                      'use_NN_medium_corr': 1})
    assert p.brem_implementation == value


def test_struct_arrays_as_lists():
    m1 = bns.M1Quantities()
    m1.n = [1., 2., 3., 4.]
    m1.chi = (1. / 3.,) * 4
    m1.H = [[float(4 * i + j) for j in range(4)] for i in range(4)]
    assert m1.n == [1., 2., 3., 4.] and isinstance(m1.J, list)
    assert m1.H[2][3] == 11.
    with pytest.raises(ValueError):
        m1.J = [1., 2.]
    gp = bns.GreyOpacityParams()
    gp.m1_pars = m1
    assert list(gp.m1_pars.n) == [1., 2., 3., 4.]


def test_default_quadrature_and_gauss_legendre():
    q = bns.cvar.quadrature_default
    assert (q.type, q.dim, q.nx, q.ny, q.nz, q.x1, q.x2) == (0, 1, 20, 1, 1, 0., 1.)
    assert (q.y1, q.y2, q.z1, q.z2) == (-42.,) * 4
    assert bns.cvar.quadrature_default is q          # one module-level variable
    q.nx = 6
    bns.GaussLegendre(q)
    x, w = np.array(q.points[:6]), np.array(q.w[:6])
    xr, wr = np.polynomial.legendre.leggauss(6)
    # the reference's Newton iteration stops at ~1e-11 (integration.hpp:28-87)
    np.testing.assert_allclose(np.sort(x), np.sort(0.5 * (xr + 1.)), rtol=1e-10)
    np.testing.assert_allclose(w.sum(), 1., rtol=1e-10)
    q.nx = 20                                       # leave the default as found


def test_nu_equilibrium_params_match_oracle(port):
    """NuEquilibriumParams (distribution.hpp:253-290) on the oracle's points."""
    eos, _ = port.synthetic_points(3, 8)
    want, _ = port.nu_equilibrium(eos)
    names = ("nb", "temp", "ye", "yp", "yn", "mu_p", "mu_n", "mu_e", "mu_mu", "dU", "dm_eff")
    for p in range(eos.shape[1]):
        e = bns.MyEOSParams()
        for k, nme in enumerate(names):
            setattr(e, nme, float(eos[k, p]))
        d = bns.NuEquilibriumParams(e)
        got = np.concatenate([d.w_t, d.temp_t, d.eta_t, d.w_f, d.temp_f, d.c_f, d.beta_f])
        np.testing.assert_array_equal(got, want[:, p])
