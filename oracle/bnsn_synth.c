/* bnsn_synth.c -- seeded synthetic thermodynamic points for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The benchmark's reference arm and the tests make
 * their inputs with this generator so that nothing on the CPU side loads the
 * product library.  It restates, operation for operation, the library's own
 * host generator (bnsn_synthetic_points, bns_nurates_gb300/csrc/host_utils.cpp);
 * both are compiled without floating-point contraction, so the two produce
 * bit-identical points on the same machine (tests/test_oracle_pins.py).
 *
 * The distribution it draws from is the workload description of the opacity
 * benchmarks: rho log-uniform in [1e6, 1e15] g/cm^3, T log-uniform in
 * [0.5, 100] MeV, Ye uniform in [0.01, 0.6]; mu_e of an ideal relativistic
 * e+- gas with net density nb*Ye (rest mass included); non-relativistic ideal
 * nucleons plus a mean-field shift dU uniform in [-20, 20] MeV; per neutrino
 * species (nue, anue, nux; anux := nux) T_nu = T*U(0.5, 1.5), eta_nu in
 * U(-5, 5), n and J the Fermi-Dirac moments (distribution.hpp:452-460 of the
 * reference uses the same normalisation) and chi in U[1/3, 1].
 */
#include <math.h>
#include <stdint.h>

#include "bnsn_oracle_consts.h"

void oracle_gauss_legendre(int n, double* x, double* w);

static double g_rx[16], g_rw[16];

static uint64_t mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

/* Uniform in [0, 1): stream k of point idx (53 random bits). */
static double uni(uint64_t seed, int64_t idx, int k)
{
    const uint64_t h =
        mix64(mix64(seed) ^ mix64((uint64_t)idx * 0xD1B54A32D192ED03ull + (uint64_t)k));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

/* 1/(e^a + 1) without overflow. */
static double fermi(double a)
{
    if (a > 0.)
    {
        const double e = exp(-a);
        return e / (1. + e);
    }
    return 1. / (1. + exp(a));
}

/* F_k(eta) = int_0^inf x^k / (e^{x - eta} + 1) dx: the bulk below eta - 30 in
 * closed form, then 16-point Gauss-Legendre panels (2 below the edge, 3
 * above it up to eta + 40). */
static double fermi_integral(double k, double eta)
{
    const double a  = eta > 0. ? eta : 0.;
    const double lo = a > 30. ? a - 30. : 0.;
    double s        = lo > 0. ? pow(lo, k + 1.) / (k + 1.) : 0.;
    const double seg_lo[2] = {lo, a};
    const double seg_hi[2] = {a, a + 40.};
    const int panels[2]    = {2, 3};
    for (int g = 0; g < 2; ++g)
    {
        double acc = 0.;
        if (!(seg_hi[g] > seg_lo[g]))
            continue;
        const double h = (seg_hi[g] - seg_lo[g]) / panels[g];
        for (int p = 0; p < panels[g]; ++p)
            for (int i = 0; i < 16; ++i)
            {
                const double x = seg_lo[g] + h * (p + g_rx[i]);
                acc += g_rw[i] * (pow(x, k) * fermi(x - eta));
            }
        s += acc * h;
    }
    return s;
}

/* F_{1/2}(eta) and dF/deta with x = u^2. */
static void fermi_half(double eta, double* F, double* dF)
{
    const double a   = eta > 0. ? eta : 0.;
    const double lo  = a > 30. ? a - 30. : 0.;
    const double ulo = sqrt(lo), uhi = sqrt(a + 40.);
    double f0        = lo > 0. ? pow(lo, 1.5) / 1.5 : 0.;
    double d0        = 0.;
    const int panels = 3;
    const double h   = (uhi - ulo) / panels;
    for (int p = 0; p < panels; ++p)
        for (int i = 0; i < 16; ++i)
        {
            const double u  = ulo + h * (p + g_rx[i]);
            const double fr = fermi(u * u - eta);
            f0 += g_rw[i] * h * 2. * u * u * fr;
            d0 += g_rw[i] * h * 2. * u * u * fr * (1. - fr);
        }
    *F  = f0;
    *dF = d0;
}

/* Net electron density [nm^-3] of an ideal relativistic e+- gas and its
 * derivative in mu. */
static void electron_net_density(double mu, double T, double* n, double* dn)
{
    const double m   = C_ME;
    const double hc  = C_HBAR * C_CLIGHT;
    const double pf2 = mu * mu - m * m;
    const double pf  = pf2 > 0. ? sqrt(pf2) : 0.;
    const double lo  = pf > 30. * T ? pf - 30. * T : 0.;
    double s         = lo > 0. ? lo * lo * lo / 3. : 0.;
    double ds        = 0.;
    const double edges[3] = {lo, pf, pf + 50. * T};
    const int panels[2]   = {2, 4};
    for (int seg = 0; seg < 2; ++seg)
    {
        if (!(edges[seg + 1] > edges[seg]))
            continue;
        const double h = (edges[seg + 1] - edges[seg]) / panels[seg];
        for (int p = 0; p < panels[seg]; ++p)
            for (int i = 0; i < 16; ++i)
            {
                const double pp = edges[seg] + h * (p + g_rx[i]);
                const double E  = sqrt(pp * pp + m * m);
                const double f1 = fermi((E - mu) / T), f2 = fermi((E + mu) / T);
                s += g_rw[i] * h * pp * pp * (f1 - f2);
                ds += g_rw[i] * h * pp * pp * (f1 * (1. - f1) + f2 * (1. - f2)) / T;
            }
    }
    const double c = 1. / (C_PI * C_PI * hc * hc * hc);
    *n  = s * c;
    *dn = ds * c;
}

/* mu_e from n_e: safeguarded Newton from the massless closed form. */
static double solve_mu_e(double ne, double T)
{
    const double hc = C_HBAR * C_CLIGHT;
    const double b  = 3. * C_PI * C_PI * hc * hc * hc * ne;
    const double pq = C_PI * C_PI * T * T / 3.;
    const double d  = sqrt(b * b / 4. + pq * pq * pq);
    double x        = cbrt(b / 2. + d) + cbrt(b / 2. - d);
    if (!(x > 0.))
        x = 1e-3 * T;
    double lo = 0., hi = 1e300;
    for (int it = 0; it < 60; ++it)
    {
        double n, dn;
        electron_net_density(x, T, &n, &dn);
        const double g = n - ne;
        if (g > 0.)
            hi = x;
        else
            lo = x;
        double xn = x - g / dn;
        if (!(xn > lo && xn < hi))
            xn = hi < 1e300 ? 0.5 * (lo + hi) : 2. * x + T;
        if (fabs(xn - x) < 1e-12 * (fabs(x) + T))
            return xn;
        x = xn;
    }
    return x;
}

/* Degeneracy of a non-relativistic ideal Fermi gas (g = 2) of mass m [MeV]
 * at density n [nm^-3]. */
static double solve_eta_nucleon(double n, double m, double T)
{
    const double hc     = C_HBAR * C_CLIGHT;
    const double pref   = 2. * sqrt(2.) * pow(m * T, 1.5) / (2. * C_PI * C_PI * hc * hc * hc);
    const double target = n / pref;
    double x  = target > 1. ? pow(1.5 * target, 2. / 3.) : log(target / (0.5 * sqrt(C_PI)));
    double lo = -1e300, hi = 1e300;
    for (int it = 0; it < 60; ++it)
    {
        double F, dF;
        fermi_half(x, &F, &dF);
        const double g = F - target;
        if (g > 0.)
            hi = x;
        else
            lo = x;
        double xn = x - g / dF;
        if (!(xn > lo && xn < hi))
            xn = (lo > -1e300 && hi < 1e300) ? 0.5 * (lo + hi) : (g > 0. ? x - 5. : x + 5.);
        if (fabs(xn - x) < 1e-12 * (1. + fabs(x)))
            return xn;
        x = xn;
    }
    return x;
}

/* Points first .. first+npts-1 of the seeded workload: eos[11][npts]
 * (nb temp ye yp yn mu_p mu_n mu_e mu_mu dU dm_eff) and m1[12][npts]
 * (n[4] J[4] chi[4]), field-major. */
int oracle_synthetic_points(uint64_t seed, int64_t first, int64_t npts, double* eos,
                            double* m1, int nthreads)
{
    if (npts < 0 || (npts > 0 && (!eos || !m1)))
        return 1;
    oracle_gauss_legendre(16, g_rx, g_rw);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t q = 0; q < npts; ++q)
    {
        const int64_t idx  = first + q;
        const double rho   = pow(10., 6. + 9. * uni(seed, idx, 0));
        const double T     = 0.5 * pow(200., uni(seed, idx, 1));
        const double ye    = 0.01 + 0.59 * uni(seed, idx, 2);
        const double nb    = rho / C_MU * 1e-21;
        const double dU    = -20. + 40. * uni(seed, idx, 3);
        const double mu_e  = solve_mu_e(nb * ye, T);
        const double eta_p = solve_eta_nucleon(nb * ye, C_MP, T);
        const double eta_n = solve_eta_nucleon(nb * (1. - ye), C_MN, T);
        const double v[11] = {nb,  T, ye, ye, 1. - ye, C_MP + T * eta_p,
                              C_MN + T * eta_n + dU, mu_e, 0., dU, C_Q};
        for (int f = 0; f < 11; ++f)
            eos[f * npts + q] = v[f];
        for (int s = 0; s < 3; ++s)
        {
            const double Tn  = T * (0.5 + uni(seed, idx, 4 + 3 * s));
            const double eta = -5. + 10. * uni(seed, idx, 5 + 3 * s);
            const double chi = 1. / 3. + (2. / 3.) * uni(seed, idx, 6 + 3 * s);
            const double n   = C_FOURPI_HC3 * Tn * Tn * Tn * fermi_integral(2., eta);
            const double J   = C_FOURPI_HC3 * Tn * Tn * Tn * Tn * fermi_integral(3., eta);
            m1[(0 + s) * npts + q] = n;
            m1[(4 + s) * npts + q] = J;
            m1[(8 + s) * npts + q] = chi;
        }
        m1[3 * npts + q]  = m1[2 * npts + q];
        m1[7 * npts + q]  = m1[6 * npts + q];
        m1[11 * npts + q] = m1[10 * npts + q];
    }
    return 0;
}
