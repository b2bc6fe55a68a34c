// Test infrastructure only: prints sizeof/offsetof of the reference's public
// structs (include/bns_nurates.hpp:106-524, unmodified BS_N_MAX = 20) as JSON,
// so tests can check that include/bns_nurates_gb300.h keeps the same layout.
#include <stddef.h>
#include <stdio.h>

#include "bns_nurates.hpp"

#define F(S, m) printf("    \"%s\": %zu,\n", #m, offsetof(S, m))
#define BEGIN(S) printf("  \"%s\": {\n    \"__size__\": %zu,\n", #S, sizeof(S))
#define END(last) printf("    \"__end__\": 0\n  }%s\n", last ? "" : ",")

int main()
{
    printf("{\n");
    BEGIN(MyQuadrature);
    F(MyQuadrature, type); F(MyQuadrature, alpha); F(MyQuadrature, dim);
    F(MyQuadrature, nx); F(MyQuadrature, ny); F(MyQuadrature, nz);
    F(MyQuadrature, x1); F(MyQuadrature, x2); F(MyQuadrature, y1);
    F(MyQuadrature, y2); F(MyQuadrature, z1); F(MyQuadrature, z2);
    F(MyQuadrature, points); F(MyQuadrature, w);
    END(0);
    BEGIN(MyEOSParams);
    F(MyEOSParams, nb); F(MyEOSParams, temp); F(MyEOSParams, ye);
    F(MyEOSParams, yp); F(MyEOSParams, yn); F(MyEOSParams, mu_p);
    F(MyEOSParams, mu_n); F(MyEOSParams, mu_e); F(MyEOSParams, mu_mu);
    F(MyEOSParams, dU); F(MyEOSParams, dm_eff);
    END(0);
    BEGIN(OpacityParams);
    F(OpacityParams, use_dU); F(OpacityParams, use_dm_eff);
    F(OpacityParams, use_WM_ab); F(OpacityParams, use_WM_sc);
    F(OpacityParams, use_decay); F(OpacityParams, brem_implementation);
    F(OpacityParams, use_NN_medium_corr); F(OpacityParams, neglect_blocking);
    END(0);
    BEGIN(OpacityFlags);
    F(OpacityFlags, use_abs_em); F(OpacityFlags, use_pair);
    F(OpacityFlags, use_brem); F(OpacityFlags, use_inelastic_scatt);
    F(OpacityFlags, use_iso);
    END(0);
    BEGIN(NuDistributionParams);
    F(NuDistributionParams, w_t); F(NuDistributionParams, temp_t);
    F(NuDistributionParams, eta_t); F(NuDistributionParams, w_f);
    F(NuDistributionParams, temp_f); F(NuDistributionParams, c_f);
    F(NuDistributionParams, beta_f);
    END(0);
    BEGIN(M1Quantities);
    F(M1Quantities, n); F(M1Quantities, J); F(M1Quantities, H);
    F(M1Quantities, chi);
    END(0);
    BEGIN(PairKernelParams);
    F(PairKernelParams, omega); F(PairKernelParams, omega_prime);
    F(PairKernelParams, cos_theta); F(PairKernelParams, mu);
    F(PairKernelParams, mu_prime); F(PairKernelParams, lmax);
    F(PairKernelParams, filter);
    END(0);
    BEGIN(BremKernelParams);
    F(BremKernelParams, omega); F(BremKernelParams, omega_prime);
    F(BremKernelParams, l); F(BremKernelParams, use_NN_medium_corr);
    END(0);
    BEGIN(InelasticScattKernelParams);
    F(InelasticScattKernelParams, omega);
    F(InelasticScattKernelParams, omega_prime);
    END(0);
    BEGIN(MyKernelParams);
    F(MyKernelParams, pair_kernel_params); F(MyKernelParams, brem_kernel_params);
    F(MyKernelParams, inelastic_kernel_params);
    END(0);
    BEGIN(GreyOpacityParams);
    F(GreyOpacityParams, opacity_pars); F(GreyOpacityParams, kernel_pars);
    F(GreyOpacityParams, eos_pars); F(GreyOpacityParams, distr_pars);
    F(GreyOpacityParams, m1_pars); F(GreyOpacityParams, opacity_flags);
    END(0);
    BEGIN(M1Opacities);
    F(M1Opacities, eta_0); F(M1Opacities, kappa_0_a); F(M1Opacities, eta);
    F(M1Opacities, kappa_a); F(M1Opacities, kappa_s);
    END(0);
    BEGIN(SpectralOpacities);
    F(SpectralOpacities, j); F(SpectralOpacities, kappa);
    F(SpectralOpacities, j_s); F(SpectralOpacities, kappa_s);
    END(0);
    BEGIN(MyOpacity);
    F(MyOpacity, abs); F(MyOpacity, em);
    END(0);
    BEGIN(MyKernelOutput);
    F(MyKernelOutput, em); F(MyKernelOutput, abs);
    END(1);
    printf("}\n");
    return 0;
}
