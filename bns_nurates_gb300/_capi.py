"""ctypes view of include/bns_nurates_gb300.h.

The struct classes mirror the reference's public structs field for field
(bns_nurates include/bns_nurates.hpp:106-524), so their ctypes layout equals
the C layout; tests compare it against the reference build.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbnsn_gb300.so")

BS_N_MAX = 20
NQUAD_MAX = 20
c_double, c_int, c_bool = ctypes.c_double, ctypes.c_int, ctypes.c_bool

# status codes
OK, ERR_ARG, ERR_NQUAD, ERR_CUDA, ERR_NO_TABLE, ERR_NO_DEVICE = range(6)
FP64, MIXED = 0, 1
NOALLOC_MAX_POINTS = 4096
NUM_PHASES = 9
PHASES = ("prelude", "pair", "brem", "neps", "final", "spectral", "aux", "neps_accurate",
          "neps_fp64")
BREM_HR98, BREM_BRT06, BREM_GP19 = 0, 1, 2


class MyQuadrature(ctypes.Structure):
    _fields_ = [("type", c_int), ("alpha", c_double), ("dim", c_int), ("nx", c_int),
                ("ny", c_int), ("nz", c_int), ("x1", c_double), ("x2", c_double),
                ("y1", c_double), ("y2", c_double), ("z1", c_double), ("z2", c_double),
                ("points", c_double * BS_N_MAX), ("w", c_double * BS_N_MAX)]


class BremKernelParams(ctypes.Structure):
    _fields_ = [("omega", c_double), ("omega_prime", c_double), ("l", c_int),
                ("use_NN_medium_corr", c_bool)]


class PairKernelParams(ctypes.Structure):
    _fields_ = [(n, c_double) for n in
                ("omega", "omega_prime", "cos_theta", "mu", "mu_prime", "lmax", "filter")]


class InelasticScattKernelParams(ctypes.Structure):
    _fields_ = [("omega", c_double), ("omega_prime", c_double)]


class MyKernelParams(ctypes.Structure):
    _fields_ = [("pair_kernel_params", PairKernelParams),
                ("brem_kernel_params", BremKernelParams),
                ("inelastic_kernel_params", InelasticScattKernelParams)]


class MyKernelOutput(ctypes.Structure):
    _fields_ = [("em", c_double * 4), ("abs", c_double * 4)]


class MyEOSParams(ctypes.Structure):
    _fields_ = [(n, c_double) for n in
                ("nb", "temp", "ye", "yp", "yn", "mu_p", "mu_n", "mu_e", "mu_mu", "dU",
                 "dm_eff")]


class MyOpacity(ctypes.Structure):
    _fields_ = [("abs", c_double * 4), ("em", c_double * 4)]


class OpacityParams(ctypes.Structure):
    _fields_ = [("use_dU", c_bool), ("use_dm_eff", c_bool), ("use_WM_ab", c_bool),
                ("use_WM_sc", c_bool), ("use_decay", c_bool),
                ("brem_implementation", c_int), ("use_NN_medium_corr", c_bool),
                ("neglect_blocking", c_bool)]


class NuDistributionParams(ctypes.Structure):
    _fields_ = [(n, c_double * 4) for n in
                ("w_t", "temp_t", "eta_t", "w_f", "temp_f", "c_f", "beta_f")]


class M1Quantities(ctypes.Structure):
    _fields_ = [("n", c_double * 4), ("J", c_double * 4), ("H", (c_double * 4) * 4),
                ("chi", c_double * 4)]


class OpacityFlags(ctypes.Structure):
    _fields_ = [(n, c_int) for n in
                ("use_abs_em", "use_pair", "use_brem", "use_inelastic_scatt", "use_iso")]


class GreyOpacityParams(ctypes.Structure):
    _fields_ = [("opacity_pars", OpacityParams), ("kernel_pars", MyKernelParams),
                ("eos_pars", MyEOSParams), ("distr_pars", NuDistributionParams),
                ("m1_pars", M1Quantities), ("opacity_flags", OpacityFlags)]


class M1Opacities(ctypes.Structure):
    _fields_ = [(n, c_double * 4) for n in ("eta_0", "kappa_0_a", "eta", "kappa_a", "kappa_s")]


class SpectralOpacities(ctypes.Structure):
    _fields_ = [(n, c_double * 4) for n in ("j", "kappa", "j_s", "kappa_s")]


P = ctypes.c_void_p


class Block(ctypes.Structure):
    _fields_ = [("first", ctypes.c_int64), ("count", ctypes.c_int64), ("flags", OpacityFlags),
                ("brem_implementation", c_int), ("nquad", c_int)]


class EosSoA(ctypes.Structure):
    _fields_ = [(n, P) for n in ("nb", "temp", "ye", "yp", "yn", "mu_p", "mu_n", "mu_e",
                                  "mu_mu", "dU", "dm_eff")]


class M1SoA(ctypes.Structure):
    _fields_ = [("n", P * 4), ("J", P * 4), ("chi", P * 4)]


class DistrSoA(ctypes.Structure):
    _fields_ = [(n, P * 4) for n in ("w_t", "temp_t", "eta_t", "w_f", "temp_f", "c_f", "beta_f")]


class GridBox(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_int64 * 3), ("lo", ctypes.c_int64 * 3),
                ("hi", ctypes.c_int64 * 3), ("eos", P * 11), ("m1", P * 12), ("out", P * 20)]


class M1OpacitiesSoA(ctypes.Structure):
    _fields_ = [(n, P * 4) for n in ("eta_0", "kappa_0_a", "eta", "kappa_a", "kappa_s")]


class SpectralSoA(ctypes.Structure):
    _fields_ = [(n, P * 4) for n in ("j", "kappa", "j_s", "kappa_s")]


# every entry point of the header, with its ctypes signature
SIGNATURES = {
    "bnsn_m1_opacities": (c_int, [P, P, P, P, P, P, P, c_int, c_int, P, ctypes.c_int64, P]),
    "bnsn_m1_opacities_grid_boxes": (c_int, [P, P, P, P, P, c_int, P, P, c_int, c_int, P]),
    "bnsn_m1_opacities_noalloc": (c_int, [P, P, P, P, P, P, P, c_int, c_int, P, ctypes.c_int64,
                                          P]),
    "bnsn_spectral_opacities": (c_int, [P, P, P, P, P, P, P, c_int, c_int, c_int, P,
                                        ctypes.c_int64, P]),
    "bnsn_distr_from_m1": (c_int, [P, P, ctypes.c_int64, P]),
    "bnsn_nu_equilibrium": (c_int, [P, P, P, P, P, ctypes.c_int64, P]),
    "bnsn_gp19_set_table": (c_int, [P] * 8),
    "bnsn_compute_m1_opacities_point": (c_int, [P, P, P, c_int, P]),
    "bnsn_compute_spectral_opacities_point": (c_int, [c_double, P, P, c_int, P]),
    "bnsn_m1_opacities_host": (c_int, [P, P, P, P, P, P, c_int, c_int, P, ctypes.c_int64]),
    "bnsn_gauss_legendre": (c_int, [P]),
    "bnsn_synthetic_points": (c_int, [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64, P, P,
                                      c_int]),
    "bnsn_blocks_plan_create": (c_int, [P, c_int, P, c_int, c_int, c_int, P, P, P, P, P]),
    "bnsn_blocks_run": (c_int, [P, P, P, P, P]),
    "bnsn_blocks_plan_groups": (c_int, [P]),
    "bnsn_blocks_plan_info": (c_int, [P, c_int, P, P, P, P, P, P]),
    "bnsn_blocks_plan_layout": (c_int, [P, P, P, P]),
    "bnsn_blocks_set_options": (c_int, [ctypes.c_int64, ctypes.c_int64]),
    "bnsn_blocks_plan_destroy": (c_int, [P]),
    "bnsn_fp64_peak_probe": (c_int, [ctypes.c_int64, P]),
    "bnsn_fp32_peak_probe": (c_int, [ctypes.c_int64, P]),
    "bnsn_phase_timing": (c_int, [c_int]),
    "bnsn_phase_times": (c_int, [P, P]),
    "bnsn_kernel_launches": (ctypes.c_int64, []),
    "bnsn_spectral_mixed_stats": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64), ctypes.c_int]),
    "bnsn_distr_from_m1_point": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "bnsn_gp19_load_header": (ctypes.c_int, [ctypes.c_char_p]),
    "bnsn_grey_mixed_stats": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64), ctypes.c_int]),
    "bnsn_nonfinite_outputs": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64), ctypes.c_int]),
    "bnsn_fdi": (c_int, [c_int, P, P, ctypes.c_int64, P]),
    "bnsn_pair_j_mixed": (c_int, [P, P, P, P, P, P, ctypes.c_int64, P]),
    "bnsn_nes_m_mixed": (c_int, [P, P, P, P, P, P, ctypes.c_int64, P]),
    "bnsn_fdi_host": (c_int, [c_int, P, P, ctypes.c_int64]),
    "bnsn_status_string": (ctypes.c_char_p, [c_int]),
    "bnsn_last_error": (ctypes.c_char_p, []),
    "bnsn_version": (c_int, []),
}

_lib = None


def load():
    """Load the in-tree library; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m bns_nurates_gb300.build` "
                "(no CPU fallback exists)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib
