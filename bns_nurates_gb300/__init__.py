"""GB300-native grey and spectral neutrino opacities (bns_nurates hot path).

The computation lives in the CUDA library ``libbnsn_gb300.so`` built from
``csrc/`` for sm_103a (``python -m bns_nurates_gb300.build``).  This package
is the Python host mirror of its C ABI (``include/bns_nurates_gb300.h``).
"""

from ._capi import (BREM_BRT06, BREM_GP19, BREM_HR98, FP64, MIXED,  # noqa: F401
                    GreyOpacityParams, M1Opacities, MyEOSParams, MyQuadrature,
                    NuDistributionParams, OpacityFlags, OpacityParams, SpectralOpacities)
from .api import (BlocksPlan, BnsnError, ComputeM1Opacities, ComputeM1OpacitiesNotStimulated,  # noqa: F401
                  ComputeSpectralOpacitiesNotStimulatedAbs,
                  ComputeSpectralOpacitiesStimulatedAbs, FDI_NAMES, distr_from_m1, fdi,
                  fdi_host, flags_tuple,
                  fp32_peak_tflops, fp64_peak_tflops, gauss_legendre, gp19_table_from_header,
                  grey_mixed_stats,
                  kernel_launches, load_gp19_header, m1_opacities,
                  m1_opacities_grid_boxes, m1_opacities_host, nonfinite_outputs, nu_equilibrium, opacity_flags, opacity_params, params_tuple,
                  nes_m_mixed, pair_j_mixed, phase_times, phase_timing, quad_arrays, set_gp19_table, spectral_mixed_stats,
                  spectral_opacities, synthetic_points)


def lib():
    """The loaded C library (raises if it has not been built)."""
    from . import _capi
    return _capi.load()
