// Per-point host program written against the reference's function names
// (ComputeM1Opacities, ComputeSpectralOpacitiesStimulatedAbs,
// CalculateDistrParamsFromM1, GaussLegendre) through bns_nurates_gb300.hpp.
// Prints, for each synthetic point, the 28 distribution parameters, the 20
// grey outputs and the 16 spectral outputs at 10 MeV, one value per line.
// With a second argument "fdi": FDI_m92, FDI_m32, FDI_0, FDI_p12, FDI_p3,
// FDI_p10 and FDI_p212 at -3.5, 0.25, 7 and 60, one value per line.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "bns_nurates_gb300.hpp"

int main(int argc, char** argv)
{
    if (argc > 2 && argv[2][0] == 'f')
    {
        double (*fn[7])(double) = {FDI_m92, FDI_m32, FDI_0, FDI_p12, FDI_p3, FDI_p10, FDI_p212};
        const double xs[4]      = {-3.5, 0.25, 7., 60.};
        for (int f = 0; f < 7; ++f)
            for (int i = 0; i < 4; ++i)
                printf("%.17g\n", fn[f](xs[i]));
        return bnsn_last_error()[0] == 0 ? 0 : 1;
    }
    const int npts = argc > 1 ? atoi(argv[1]) : 4;
    std::vector<double> eos(11 * npts), m1(12 * npts);
    if (bnsn_synthetic_points(20261203, 0, npts, eos.data(), m1.data(), 1) != BNSN_OK)
        return 2;
    MyQuadrature quad = {};
    quad.nx           = 10;
    GaussLegendre(&quad);
    for (int p = 0; p < npts; ++p)
    {
        GreyOpacityParams gp = {};
        double* e = &gp.eos_pars.nb; // MyEOSParams: 11 doubles in field order
        for (int k = 0; k < 11; ++k)
            e[k] = eos[k * npts + p];
        for (int s = 0; s < total_num_species; ++s)
        {
            gp.m1_pars.n[s]   = m1[s * npts + p];
            gp.m1_pars.J[s]   = m1[(4 + s) * npts + p];
            gp.m1_pars.chi[s] = m1[(8 + s) * npts + p];
        }
        gp.opacity_flags = {1, 1, 1, 1, 1};
        gp.opacity_pars  = {true, false, true, true, true, BREM_HR98, true, false};
        gp.distr_pars    = CalculateDistrParamsFromM1(&gp.m1_pars, &gp.eos_pars);
        const M1Opacities grey = ComputeM1Opacities(&quad, &quad, &gp);
        const SpectralOpacities spec = ComputeSpectralOpacitiesStimulatedAbs(10., &quad, &gp);
        const double* d = &gp.distr_pars.w_t[0];
        for (int k = 0; k < 28; ++k)
            printf("%.17g\n", d[k]);
        const double* g = &grey.eta_0[0];
        for (int k = 0; k < 20; ++k)
            printf("%.17g\n", g[k]);
        const double* sp = &spec.j[0];
        for (int k = 0; k < 16; ++k)
            printf("%.17g\n", sp[k]);
    }
    return bnsn_last_error()[0] == 0 ? 0 : 1;
}
