// Host utilities of the C ABI: Gauss-Legendre quadrature and the seeded
// synthetic thermodynamic workload.

#include <math.h>
#include <stdint.h>

#include <vector>

#include "../../include/bns_nurates_gb300.h"
#include "bnsn_constants.h"

using namespace bnsn;

// ---------------------------------------------------------------------------
// Gauss-Legendre nodes/weights on [0, 1]: Newton iteration on the Legendre
// recurrence with the reference's starting guesses and tolerance
// (integration.hpp:28-87), so the nodes are the reference's own.
// ---------------------------------------------------------------------------
extern "C" int bnsn_gauss_legendre(MyQuadrature* q)
{
    if (!q || q->nx < 1 || q->nx > BS_N_MAX)
        return BNSN_ERR_ARG;
    const double eps = 1.0e-10;
    const int n      = q->nx;
    const int m      = (n + 1) / 2;
    const double xm = 0.5 * (1. + 0.), xl = 0.5 * (1. - 0.);
    for (int i = 0; i < m; ++i)
    {
        double z = cos(k::Pi * (i + 0.75) / (n + 0.5)), z1, pp, p1, p2, p3;
        do
        {
            p1 = 1.0;
            p2 = 0.0;
            for (int j = 0; j < n; ++j)
            {
                p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j + 1.0) * z * p2 - j * p3) / (j + 1);
            }
            pp = n * (z * p1 - p2) / ((z * z) - 1.0);
            z1 = z;
            z  = z1 - p1 / pp;
        } while (fabs(z - z1) > eps);
        q->points[i]         = xm - xl * z;
        q->points[n - 1 - i] = xm + xl * z;
        q->w[i]              = 2.0 * xl / ((1.0 - (z * z)) * (pp * pp));
        q->w[n - 1 - i]      = q->w[i];
    }
    q->type = kGauleg;
    q->dim  = 1;
    q->ny = q->nz = 1;
    q->x1 = 0.;
    q->x2 = 1.;
    q->y1 = q->y2 = q->z1 = q->z2 = -42.;
    return BNSN_OK;
}

// ---------------------------------------------------------------------------
// Synthetic workload
// ---------------------------------------------------------------------------
namespace {

inline uint64_t mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Uniform in [0, 1): stream k of point idx.
inline double uni(uint64_t seed, int64_t idx, int k)
{
    const uint64_t h =
        mix64(mix64(seed) ^ mix64((uint64_t)idx * 0xD1B54A32D192ED03ull + (uint64_t)k));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// Gauss-Legendre rule on [0, 1] for the generator's own integrals.
struct Rule
{
    double x[32], w[32];
    Rule()
    {
        MyQuadrature q;
        q.nx = 16;
        bnsn_gauss_legendre(&q);
        for (int i = 0; i < 16; ++i)
        {
            x[i] = q.points[i];
            w[i] = q.w[i];
        }
    }
};

const Rule& rule()
{
    static Rule r;
    return r;
}

inline double fermi(double a) // 1/(e^a + 1), stable
{
    if (a > 0.)
    {
        const double e = exp(-a);
        return e / (1. + e);
    }
    return 1. / (1. + exp(a));
}

// Integral of f over [lo, hi] with the 16-point rule on `panels` equal panels.
template <class F>
double integrate(F f, double lo, double hi, int panels)
{
    if (!(hi > lo))
        return 0.;
    const Rule& R = rule();
    const double h = (hi - lo) / panels;
    double s       = 0.;
    for (int p = 0; p < panels; ++p)
        for (int i = 0; i < 16; ++i)
            s += R.w[i] * f(lo + h * (p + R.x[i]));
    return s * h;
}

// Complete Fermi integral F_k(eta) = int_0^inf x^k/(e^{x-eta}+1) dx for
// k = 2, 3 (neutrino moments), integrand split at the edge.
double fermi_integral(double k, double eta)
{
    auto f = [&](double x) { return pow(x, k) * fermi(x - eta); };
    const double a  = eta > 0. ? eta : 0.;
    const double lo = a > 30. ? a - 30. : 0.;
    const double s  = lo > 0. ? pow(lo, k + 1.) / (k + 1.) : 0.;
    return s + integrate(f, lo, a, 2) + integrate(f, a, a + 40., 3);
}

// F_{1/2}(eta) and its eta-derivative, x = u^2 to remove the sqrt at 0.
void fermi_half(double eta, double* F, double* dF)
{
    const double a   = eta > 0. ? eta : 0.;
    const double lo  = a > 30. ? a - 30. : 0.;
    const double ulo = sqrt(lo), uhi = sqrt(a + 40.);
    double f0 = lo > 0. ? pow(lo, 1.5) / 1.5 : 0.;
    double d0 = 0.;
    const Rule& R = rule();
    const int panels = 3;
    const double h   = (uhi - ulo) / panels;
    for (int p = 0; p < panels; ++p)
        for (int i = 0; i < 16; ++i)
        {
            const double u  = ulo + h * (p + R.x[i]);
            const double fr = fermi(u * u - eta);
            f0 += R.w[i] * h * 2. * u * u * fr;
            d0 += R.w[i] * h * 2. * u * u * fr * (1. - fr);
        }
    *F  = f0;
    *dF = d0;
}

// Net e- density [nm^-3] of an ideal relativistic e+- gas at (mu, T), rest
// mass included, and d(density)/d(mu).
void electron_net_density(double mu, double T, double* n, double* dn)
{
    const double m   = k::Me;
    const double hc  = k::Hbar * k::Clight; // MeV nm
    const double pf2 = mu * mu - m * m;
    const double pf  = pf2 > 0. ? sqrt(pf2) : 0.;
    const double lo  = pf > 30. * T ? pf - 30. * T : 0.;
    double s  = lo > 0. ? lo * lo * lo / 3. : 0.;
    double ds = 0.;
    const Rule& R = rule();
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
                const double pp = edges[seg] + h * (p + R.x[i]);
                const double E  = sqrt(pp * pp + m * m);
                const double f1 = fermi((E - mu) / T), f2 = fermi((E + mu) / T);
                s += R.w[i] * h * pp * pp * (f1 - f2);
                ds += R.w[i] * h * pp * pp * (f1 * (1. - f1) + f2 * (1. - f2)) / T;
            }
    }
    const double c = 1. / (k::Pi * k::Pi * hc * hc * hc);
    *n  = s * c;
    *dn = ds * c;
}

// mu_e from n_e: Newton from the massless closed form
// (mu^3 + pi^2 T^2 mu = 3 pi^2 hc^3 n), bracketed, bisection fallback.
double solve_mu_e(double ne, double T)
{
    const double hc = k::Hbar * k::Clight;
    const double b  = 3. * k::Pi * k::Pi * hc * hc * hc * ne;
    const double pq = k::Pi * k::Pi * T * T / 3.;
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

// eta of a non-relativistic ideal Fermi gas (g = 2) of mass m [MeV] with
// density n [nm^-3]: n = 2 sqrt(2) (m T)^{3/2} F_{1/2}(eta) / (2 pi^2 hc^3).
double solve_eta_nucleon(double n, double m, double T)
{
    const double hc     = k::Hbar * k::Clight;
    const double pref   = 2. * sqrt(2.) * pow(m * T, 1.5) / (2. * k::Pi * k::Pi * hc * hc * hc);
    const double target = n / pref;
    double x = target > 1. ? pow(1.5 * target, 2. / 3.) : log(target / (0.5 * sqrt(k::Pi)));
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

} // namespace

extern "C" int bnsn_synthetic_points(uint64_t seed, int64_t first, int64_t npts,
                                     double* eos, double* m1, int nthreads)
{
    if (npts < 0 || (npts > 0 && (!eos || !m1)))
        return BNSN_ERR_ARG;
    (void)rule();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t q = 0; q < npts; ++q)
    {
        const int64_t idx = first + q;
        const double rho  = pow(10., 6. + 9. * uni(seed, idx, 0));          // g/cm^3
        const double T    = 0.5 * pow(200., uni(seed, idx, 1));             // MeV
        const double ye   = 0.01 + 0.59 * uni(seed, idx, 2);
        const double nb   = rho / k::Mu * 1e-21;                             // nm^-3
        const double dU   = -20. + 40. * uni(seed, idx, 3);                 // MeV
        const double mu_e = solve_mu_e(nb * ye, T);
        const double eta_p = solve_eta_nucleon(nb * ye, k::Mp, T);
        const double eta_n = solve_eta_nucleon(nb * (1. - ye), k::Mn, T);
        const double v[11] = {nb,  T, ye, ye, 1. - ye, k::Mp + T * eta_p,
                              k::Mn + T * eta_n + dU, mu_e, 0., dU, k::Q};
        for (int f = 0; f < 11; ++f)
            eos[f * npts + q] = v[f];
        for (int s = 0; s < 3; ++s)
        {
            const double Tn  = T * (0.5 + uni(seed, idx, 4 + 3 * s));
            const double eta = -5. + 10. * uni(seed, idx, 5 + 3 * s);
            const double chi = 1. / 3. + (2. / 3.) * uni(seed, idx, 6 + 3 * s);
            const double n   = k::FourPiHc3 * Tn * Tn * Tn * fermi_integral(2., eta);
            const double J   = k::FourPiHc3 * Tn * Tn * Tn * Tn * fermi_integral(3., eta);
            m1[(0 + s) * npts + q] = n;
            m1[(4 + s) * npts + q] = J;
            m1[(8 + s) * npts + q] = chi;
        }
        m1[3 * npts + q]  = m1[2 * npts + q];
        m1[7 * npts + q]  = m1[6 * npts + q];
        m1[11 * npts + q] = m1[10 * npts + q];
    }
    return BNSN_OK;
}
