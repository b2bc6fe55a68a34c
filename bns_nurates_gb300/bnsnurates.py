"""The reference's Python module ``bnsnurates`` (bindings/bnsnurates.i) on this
library: a user of the SWIG bindings switches with

    import bns_nurates_gb300.bnsnurates as bns

and keeps the rest of the script (bindings/test_bindings.py runs unchanged).
The conventions of the SWIG module are kept:

* the flags and parameters of ``GreyOpacityParams`` are set and read as
  dicts, with ``brem_implementation`` the string "HR98", "BRT06" or "GP19"
  (bnsnurates.i:64-90, 112-130; any other string selects HR98, as there);
* fixed-size arrays of the structs (``M1Quantities.n``, ``J``, ``chi``, ``H``,
  the distribution parameters, quadrature points) are set from and read as
  Python lists (bnsnurates.i:34-58, 96-106);
* ``ComputeM1Opacities`` and the spectral functions return dicts of lists
  (bnsnurates.i:132-220);
* ``cvar.quadrature_default`` is the module's one default quadrature, which
  ``GaussLegendre`` fills in place (bns_nurates.hpp:131-145);
* the ``print_*`` helpers print the same tables (bnsnurates.i:222-270).

The opacities run on the current CUDA device through the library's per-point
entry points; the distribution-function helpers follow distribution.hpp.
"""

import ctypes
import types

import numpy as np

from . import _capi as C
from . import api

# distribution.hpp:253-290 (CONST_C_F) and constants.hpp (4 pi / (h c)^3)
_CONST_C_F = 0.6
_PI = 3.14159265358979323846264338328
_H = 4.135667696e-21
_CLIGHT = 2.99792458e+17
_FOUR_PI_HC3 = (4. * _PI) / ((_H * _CLIGHT) * (_H * _CLIGHT) * (_H * _CLIGHT))
_BREM = {"HR98": C.BREM_HR98, "BRT06": C.BREM_BRT06, "GP19": C.BREM_GP19}
_BREM_NAME = {v: k for k, v in _BREM.items()}


def _is_array(t):
    return isinstance(t, type) and issubclass(t, ctypes.Array)


def _to_list(v):
    if isinstance(v, ctypes.Array):
        return [_to_list(x) for x in v]
    return v


def _fill(arr, value, name):
    if len(value) != len(arr):
        raise ValueError(f"Size mismatch. Expected {len(arr)} elements for {name}")
    for k, x in enumerate(value):
        if isinstance(arr[k], ctypes.Array):
            _fill(arr[k], x, name)
        else:
            arr[k] = float(x)


class _Lists:
    """Array fields read as lists and set from sequences (the SWIG typemaps)."""

    def __getattribute__(self, name):
        v = super().__getattribute__(name)
        return _to_list(v) if isinstance(v, ctypes.Array) else v

    def __setattr__(self, name, value):
        ftype = dict(type(self)._fields_).get(name)
        if ftype is not None and _is_array(ftype) and not isinstance(value, ctypes.Array):
            _fill(super().__getattribute__(name), list(value), name)
        else:
            super().__setattr__(name, value)


class MyEOSParams(_Lists, C.MyEOSParams):
    pass


class MyQuadrature(_Lists, C.MyQuadrature):
    pass


class M1Quantities(_Lists, C.M1Quantities):
    pass


class NuDistributionParams(_Lists, C.NuDistributionParams):
    pass


def opacity_flags_from_dict(d):
    """OpacityFlags from the SWIG dict (bnsnurates.i:64-72)."""
    return C.OpacityFlags(*(int(d[k]) for k in
                            ("use_abs_em", "use_pair", "use_brem", "use_inelastic_scatt",
                             "use_iso")))


def opacity_flags_to_dict(f):
    return {k: int(getattr(f, k)) for k, _ in C.OpacityFlags._fields_}


def opacity_params_from_dict(d):
    """OpacityParams from the SWIG dict (bnsnurates.i:75-90): the brem
    implementation by its name's prefix, HR98 otherwise."""
    name = str(d["brem_implementation"])
    brem = C.BREM_BRT06 if name.startswith("BRT06") else (
        C.BREM_GP19 if name.startswith("GP19") else C.BREM_HR98)
    return C.OpacityParams(bool(int(d["use_dU"])), bool(int(d["use_dm_eff"])),
                           bool(int(d["use_WM_ab"])), bool(int(d["use_WM_sc"])),
                           bool(int(d["use_decay"])), brem, bool(int(d["use_NN_medium_corr"])),
                           bool(int(d["neglect_blocking"])))


def opacity_params_to_dict(p):
    d = {k: int(getattr(p, k)) for k, _ in C.OpacityParams._fields_}
    d["brem_implementation"] = _BREM_NAME.get(p.brem_implementation, "HR98")
    return d


class GreyOpacityParams(C.GreyOpacityParams):
    """GreyOpacityParams whose opacity_flags / opacity_pars are dicts."""

    def __getattribute__(self, name):
        v = super().__getattribute__(name)
        if name == "opacity_flags":
            return opacity_flags_to_dict(v)
        if name == "opacity_pars":
            return opacity_params_to_dict(v)
        return v

    def __setattr__(self, name, value):
        if name == "opacity_flags" and isinstance(value, dict):
            value = opacity_flags_from_dict(value)
        elif name == "opacity_pars" and isinstance(value, dict):
            value = opacity_params_from_dict(value)
        super().__setattr__(name, value)


def _default_quadrature():
    q = MyQuadrature()
    q.type, q.alpha, q.dim, q.nx, q.ny, q.nz = 0, 0., 1, 20, 1, 1   # kGauleg on [0, 1]
    q.x1, q.x2 = 0., 1.
    q.y1 = q.y2 = q.z1 = q.z2 = -42.
    return q


# the module's global variables (SWIG's cvar)
cvar = types.SimpleNamespace(quadrature_default=_default_quadrature())


def GaussLegendre(quad):
    """Fill quad (nx nodes on [x1, x2] = [0, 1]) in place (integration.hpp:28-87)."""
    api._check(C.load().bnsn_gauss_legendre(ctypes.byref(quad)))


def NuEquilibriumParams(eos_pars):
    """Equilibrium distribution parameters (distribution.hpp:253-290)."""
    T = eos_pars.temp
    if not (0. < T < 1e3):
        raise ValueError(f"Given temperature is either negative or beyond 1 GeV (T={T:e}).")
    out = NuDistributionParams()
    out.w_t = [1.] * 4
    out.temp_t = [T] * 4
    out.w_f = [0.] * 4
    out.c_f = [_CONST_C_F] * 4
    out.temp_f = [T] * 4
    out.beta_f = [1.] * 4
    eta = (eos_pars.mu_e - eos_pars.mu_n + eos_pars.mu_p) / T
    out.eta_t = [eta, -eta, 0., 0.]
    return out


def ComputeM1DensitiesEq(eos_pars, distr_pars, m1_pars):
    """n and J of the equilibrium distribution (distribution.hpp:447-473):
    4 pi / (hc)^3 T^3 F_2(eta_t) and the same times T F_3(eta_t)."""
    T = eos_pars.temp
    eta = np.asarray(list(distr_pars.eta_t), dtype=np.float64)
    n_pre = _FOUR_PI_HC3 * (T * T * T)
    j_pre = n_pre * T
    f2, f3 = api.fdi_host(2, eta), api.fdi_host(3, eta)
    n = [n_pre * v for v in f2]
    J = [j_pre * v for v in f3]
    if not (np.isfinite(n).all() and np.isfinite(J).all()):
        raise ValueError("neutrino densities computed assuming equilibrium are not finite")
    m1_pars.n = n
    m1_pars.J = J


def CalculateDistrParamsFromM1(m1_pars, eos_pars):
    """Distribution parameters from the M1 moments (distribution.hpp:323-333)."""
    out = NuDistributionParams()
    api._check(C.load().bnsn_distr_from_m1_point(ctypes.byref(m1_pars), ctypes.byref(out)))
    return out


ComputeM1Opacities = api.ComputeM1Opacities
ComputeM1OpacitiesNotStimulated = api.ComputeM1OpacitiesNotStimulated
ComputeSpectralOpacitiesStimulatedAbs = api.ComputeSpectralOpacitiesStimulatedAbs
ComputeSpectralOpacitiesNotStimulatedAbs = api.ComputeSpectralOpacitiesNotStimulatedAbs


# ---------------------------------------------------------------------------
# printing helpers of the SWIG module (same tables)
# ---------------------------------------------------------------------------

def print_reactions(opacity_flags):
    print('# Included reactions:')
    print('# Neutrino abs on nucleons - e+/e- capture : %d' % opacity_flags["use_abs_em"])
    print('# Elastic scattering on nucleons           : %d' % opacity_flags["use_iso"])
    print('# Nucleon-nucleon bremmstrahlung           : %d' % opacity_flags["use_brem"])
    print('# e+ e- annihilation (and inverse)         : %d' % opacity_flags["use_pair"])
    print('# Inelastic scattering on e+/e-            : %d' % opacity_flags["use_inelastic_scatt"])
    print("")


def print_corrections(opacity_pars):
    print('# Included corrections:')
    print('# dU correction                        : %d' % opacity_pars["use_dU"])
    print('# Effective mass correction            : %d' % opacity_pars["use_dm_eff"])
    print('# Weak magnetism on charged reactions  : %d' % opacity_pars["use_WM_ab"])
    print('# Weak magnetism on neutral reactions  : %d' % opacity_pars["use_WM_sc"])
    print('# Include (inverse) nucleon decays     : %d' % opacity_pars["use_decay"])
    print('# Neglect blocking factors             : %d' % opacity_pars["neglect_blocking"])
    print('# Bremsstrahlung implementation        : %s' % opacity_pars["brem_implementation"])
    print('# Medium Fischer+16 correction to brem : %d' % opacity_pars["use_NN_medium_corr"])
    print("")


def print_neutrino_quantities(m1_pars):
    n, J, chi = m1_pars.n, m1_pars.J, m1_pars.chi
    print("    nue            anue            nux            anux")
    print("n  %13.6e  %13.6e   %13.6e  %13.6e     (cm^-3)" % tuple(n))
    print("J  %13.6e  %13.6e   %13.6e  %13.6e (MeV cm^-3)" % tuple(J))
    print("chi %12.10f   %12.10f    %12.10f   %12.10f" % tuple(chi))
    print("")


def print_spectral_rates(spec_rates):
    print("      j             j_s           kappa         kappa_s")
    for s, name in enumerate((" nue", "anue", " nux", "anux")):
        print("%s %13.6e %13.6e %13.6e %13.6e" % (name, spec_rates['j'][s], spec_rates['j_s'][s],
                                                 spec_rates['kappa'][s],
                                                 spec_rates['kappa_s'][s]))
    print("")


def print_integrated_rates(gray_rates):
    print("      eta0          eta1          kappa0        kappa1        scat1")
    for s, name in enumerate((" nue", "anue", " nux", "anux")):
        print("%s %13.6e %13.6e %13.6e %13.6e %13.6e" % (
            name, gray_rates['eta_0'][s], gray_rates['eta'][s], gray_rates['kappa_0_a'][s],
            gray_rates['kappa_a'][s], gray_rates['kappa_s'][s]))
    print("")
