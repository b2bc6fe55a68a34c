/* C++ host drop-in for the per-point entry points of bns_nurates.
 *
 * Including this header instead of the reference's m1_opacities.hpp /
 * distribution.hpp / integration.hpp gives host code the reference's function
 * names and signatures over the GB300 library (each call is a batch of one
 * point on the current device, synchronous):
 *
 *   ComputeM1Opacities, ComputeM1OpacitiesNotStimulated
 *       (m1_opacities.hpp:1297-1313)
 *   ComputeSpectralOpacitiesNotStimulatedAbs, ComputeSpectralOpacitiesStimulatedAbs
 *       (m1_opacities.hpp:1506-1660)
 *   CalculateDistrParamsFromM1 (distribution.hpp:323-333)
 *   GaussLegendre (integration.hpp:28-87)
 *
 * The reference's functions return no status.  These return the same
 * structs; when the library reports an error (no sm_103 device, an argument
 * out of range, GP19 without a table) every field is NaN and
 * bnsn_last_error() holds the message.  Unlike the reference, grey_pars is
 * not written to (the reference uses its kernel_pars member as scratch).
 *
 * A grid code that calls these per point should move to the batched entry
 * points of bns_nurates_gb300.h: one call per patch instead of one per point.
 */
#ifndef BNS_NURATES_GB300_HPP
#define BNS_NURATES_GB300_HPP

#include <cmath>
#include <limits>

#include "bns_nurates_gb300.h"

namespace bnsn_dropin {

template <class T>
inline T all_nan()
{
    T v;
    double* d = reinterpret_cast<double*>(&v);
    for (unsigned k = 0; k < sizeof(T) / sizeof(double); ++k)
        d[k] = std::numeric_limits<double>::quiet_NaN();
    return v;
}

} // namespace bnsn_dropin

inline M1Opacities ComputeM1Opacities(const MyQuadrature* quad_1d, const MyQuadrature* quad_2d,
                                      GreyOpacityParams* my_grey_opacity_params)
{
    M1Opacities out;
    if (bnsn_compute_m1_opacities_point(quad_1d, quad_2d, my_grey_opacity_params, 1, &out) !=
        BNSN_OK)
        return bnsn_dropin::all_nan<M1Opacities>();
    return out;
}

inline M1Opacities ComputeM1OpacitiesNotStimulated(MyQuadrature* quad_1d, MyQuadrature* quad_2d,
                                                   GreyOpacityParams* my_grey_opacity_params)
{
    M1Opacities out;
    if (bnsn_compute_m1_opacities_point(quad_1d, quad_2d, my_grey_opacity_params, 0, &out) !=
        BNSN_OK)
        return bnsn_dropin::all_nan<M1Opacities>();
    return out;
}

inline SpectralOpacities ComputeSpectralOpacitiesNotStimulatedAbs(
    const double nu, MyQuadrature* quad_1d, GreyOpacityParams* my_grey_opacity_params)
{
    SpectralOpacities out;
    if (bnsn_compute_spectral_opacities_point(nu, quad_1d, my_grey_opacity_params, 0, &out) !=
        BNSN_OK)
        return bnsn_dropin::all_nan<SpectralOpacities>();
    return out;
}

inline SpectralOpacities ComputeSpectralOpacitiesStimulatedAbs(
    const double nu, MyQuadrature* quad_1d, GreyOpacityParams* my_grey_opacity_params)
{
    SpectralOpacities out;
    if (bnsn_compute_spectral_opacities_point(nu, quad_1d, my_grey_opacity_params, 1, &out) !=
        BNSN_OK)
        return bnsn_dropin::all_nan<SpectralOpacities>();
    return out;
}

inline NuDistributionParams CalculateDistrParamsFromM1(const M1Quantities* M1_pars,
                                                       const MyEOSParams* /*eos_pars*/)
{
    NuDistributionParams out;
    if (bnsn_distr_from_m1_point(M1_pars, &out) != BNSN_OK)
        return bnsn_dropin::all_nan<NuDistributionParams>();
    return out;
}

inline void GaussLegendre(MyQuadrature* quad)
{
    bnsn_gauss_legendre(quad);
}

#endif /* BNS_NURATES_GB300_HPP */
