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
 *   FDI_m92 .. FDI_m12, FDI_0, FDI_p12, FDI_p1, ..., FDI_p10, FDI_p212
 *       (functions.hpp:442-4375; one argument per call, NaN on error)
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

#define BNSN_DROPIN_FDI(NAME, K2)                                                        \
    inline double NAME(const double x)                                                   \
    {                                                                                    \
        double v;                                                                        \
        return bnsn_fdi_host(K2, &x, &v, 1) == BNSN_OK                                   \
                   ? v                                                                   \
                   : std::numeric_limits<double>::quiet_NaN();                           \
    }
BNSN_DROPIN_FDI(FDI_m92, -9)
BNSN_DROPIN_FDI(FDI_m72, -7)
BNSN_DROPIN_FDI(FDI_m52, -5)
BNSN_DROPIN_FDI(FDI_m32, -3)
BNSN_DROPIN_FDI(FDI_m12, -1)
BNSN_DROPIN_FDI(FDI_0, 0)
BNSN_DROPIN_FDI(FDI_p12, 1)
BNSN_DROPIN_FDI(FDI_p1, 2)
BNSN_DROPIN_FDI(FDI_p32, 3)
BNSN_DROPIN_FDI(FDI_p2, 4)
BNSN_DROPIN_FDI(FDI_p52, 5)
BNSN_DROPIN_FDI(FDI_p3, 6)
BNSN_DROPIN_FDI(FDI_p72, 7)
BNSN_DROPIN_FDI(FDI_p4, 8)
BNSN_DROPIN_FDI(FDI_p92, 9)
BNSN_DROPIN_FDI(FDI_p5, 10)
BNSN_DROPIN_FDI(FDI_p112, 11)
BNSN_DROPIN_FDI(FDI_p6, 12)
BNSN_DROPIN_FDI(FDI_p132, 13)
BNSN_DROPIN_FDI(FDI_p7, 14)
BNSN_DROPIN_FDI(FDI_p152, 15)
BNSN_DROPIN_FDI(FDI_p8, 16)
BNSN_DROPIN_FDI(FDI_p172, 17)
BNSN_DROPIN_FDI(FDI_p9, 18)
BNSN_DROPIN_FDI(FDI_p192, 19)
BNSN_DROPIN_FDI(FDI_p10, 20)
BNSN_DROPIN_FDI(FDI_p212, 21)
#undef BNSN_DROPIN_FDI

#endif /* BNS_NURATES_GB300_HPP */
