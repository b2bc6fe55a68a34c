// Double-precision device physics of the opacity path.
//
// These are the per-value building blocks of the FP64 kernels.  The formulas
// are those of the reference (cited per function); the structure is the
// GPU's: Fermi-Dirac integrals of several orders share one exponential per
// argument, and everything that does not depend on the energy pair (HR98
// channel constants, NES Fermi integrals at eta, beta-process prefactors) is
// hoisted into per-point structs computed once per point by a few lanes.
#pragma once

#include <math.h>
#include <stdint.h>

#include "bnsn_constants.h"

namespace bnsn {
namespace fp64 {

#define BNSN_DI __device__ __forceinline__

// ---------------------------------------------------------------------------
// Elementary functions (functions.hpp)
// ---------------------------------------------------------------------------

// functions.hpp:66-75: exp of the argument clamped to [-700, 700]; NaN maps
// to the lower bound.
BNSN_DI double safe_exp(double x)
{
    const double lo = (x > k::ExpLow) ? x : k::ExpLow;
    return exp((lo < k::ExpUpp) ? lo : k::ExpUpp);
}

// functions.hpp:4376-4396
BNSN_DI double fermi_distr(double e, double temp, double mu)
{
    const double arg = (e - mu) / temp;
    if (arg > 0.)
    {
        const double t = safe_exp(-arg);
        return t / (t + 1.);
    }
    return 1. / (safe_exp(arg) + 1.);
}

// functions.hpp:4401-4413 for d1 = w' - w and d2 = w - w' at once (both
// share e^{-|d|}); d2 is passed explicitly so that w == w' gives +0 for both,
// as in the reference.
BNSN_DI void neps_exp_pair(double d1, double d2, double* f1, double* f2)
{
    const double e = safe_exp(-fabs(d1));
    const int n1   = signbit(d1) != 0;
    const int n2   = signbit(d2) != 0;
    *f1            = (n1 - (!n1) * e) / (1. - e + (d1 == 0.));
    *f2            = (n2 - (!n2) * e) / (1. - e + (d2 == 0.));
}

// functions.hpp:99-137, 140-180: modified Bessel I1 / K1 polynomial fits
BNSN_DI double bessi1(double x)
{
    double ax = fabs(x), ans, y;
    if (ax < 3.75)
    {
        y   = x / 3.75;
        y   = y * y;
        ans = ax * (0.5 + y * (0.87890594 + y * (0.51498869 + y * (0.15084934 +
              y * (0.2658733e-1 + y * (0.301532e-2 + y * 0.32411e-3))))));
    }
    else
    {
        y   = 3.75 / ax;
        ans = 0.2282967e-1 + y * (-0.2895312e-1 + y * (0.1787654e-1 - y * 0.420059e-2));
        ans = 0.39894228 + y * (-0.3988024e-1 + y * (-0.362018e-2 + y * (0.163801e-2 +
              y * (-0.1031555e-1 + y * ans))));
        ans *= (exp(ax) / sqrt(ax));
    }
    return x < 0. ? -ans : ans;
}

BNSN_DI double bessk1(double x)
{
    double y, ans;
    if (x <= 2.)
    {
        y   = x * x / 4.;
        ans = (log(x / 2.) * bessi1(x)) +
              (1.0 / x) * (1.0 + y * (0.15443144 + y * (-0.67278579 + y * (-0.18156897 +
              y * (-0.1919402e-1 + y * (-0.110404e-2 + y * (-0.4686e-4)))))));
    }
    else
    {
        y   = 2. / x;
        ans = (exp(-x) / sqrt(x)) *
              (1.25331414 + y * (0.23498619 + y * (-0.3655620e-1 + y * (0.1504268e-1 +
              y * (-0.780353e-2 + y * (0.325614e-2 + y * (-0.68245e-3)))))));
    }
    return ans;
}

// ---------------------------------------------------------------------------
// Complete Fermi-Dirac integrals F_k, k = 0..5 (functions.hpp:1550-2838):
// Fukushima's piecewise minimax rational approximations in x = -|y|
// (x < -2: series in e^x; -2 <= x <= 0: rational in s = -x/2) with the
// reflection polynomial for y > 0.  A NaN argument yields 0.
// ---------------------------------------------------------------------------

template <int N>
BNSN_DI double horner(const double (&c)[N], double t)
{
    double p = c[N - 1];
#pragma unroll
    for (int i = N - 2; i >= 0; --i)
        p = c[i] + t * p;
    return p;
}

// Coefficient tables (functions.hpp:1550-2838), numerator/denominator of
// the x < -2 (an, ad) and -2 <= x <= 0 (bn, bd) rational forms.
__device__ constexpr double kAN0[5] = {22696.2126132366633, 5222.0667923565138, 357.623326425354522, 6.9167792879948140, 0.00200096064827815813};
__device__ constexpr double kAD0[5] = {45392.4252264733267, 14539.5980679273792, 1611.36476693109675, 71.072178562726798, 1.0};
__device__ constexpr double kBN0[9] = {159.601717762460980, 23.7193942338278703, 0.377783268730614356, 10.5181677709577503, 3.78181326142271599, -0.441998676614933572, -0.450072959113928254, -0.0734798777056723512, 0.000915454570009894267};
__device__ constexpr double kBD0[8] = {284.26032127745967, 315.2592651624449, 310.2713981221035, 206.21640678892182, 96.77898293084927, 35.456591489081173, 8.1762315442738975, 1.0};
__device__ constexpr double kAN1[5] = {22189.1070807945062, 4915.92700908746777, 322.901386168881348, 5.9897442965804548, 0.00397641173774375092};
__device__ constexpr double kAD1[5] = {88756.428323178025, 25002.3197546553836, 2389.06277237306633, 88.376214553692756, 1.0};
__device__ constexpr double kBN1[9] = {145.488167182330098, 251.392824471576922, 56.6537141912783024, 17.9918985363509694, 20.1369115558099802, 7.09659390228556164, 0.199701180197912643, -0.403173132925886253, -0.0792966701498222697};
__device__ constexpr double kBD1[9] = {606.0757707716040, 374.1806357435014, 252.1367051536344, 27.2746245830016, -61.57766112137513, -53.72117554363975, -25.678454878692950, -7.1995819520154718, -1.0};
__device__ constexpr double kAN2[4] = {1914.06748184935743, 273.085756700981399, 8.5861610217850095, 0.0161890243763741414};
__device__ constexpr double kAD2[4] = {7656.2699273974454, 1399.35442210906621, 72.929152915475392, 1.0};
__device__ constexpr double kBN2[9] = {2711.49678259128843, 1299.85460914884154, 222.606134197895041, 172.881855215582924, 112.951038040682055, 24.0376482128898634, -2.68393549333878715, -2.14077421411719935, -0.326188299771397236};
__device__ constexpr double kBD2[9] = {2517.1726659917047, 3038.7689794575778, 2541.7823512372631, 1428.0589853413436, 531.62378035996132, 122.54595216479181, 8.395768655115050, -3.9142702096919080, -1.0};
__device__ constexpr double kAN3[4] = {5121.6401850302408, 664.28706260743472, 19.0856927562699544, 0.0410982603688952131};
__device__ constexpr double kAD3[4] = {13657.7071600806539, 2136.54222460571183, 92.376788603062645, 1.0};
__device__ constexpr double kBN3[8] = {7881.24597452900838, 4323.07526636309661, 1260.13125873282465, 653.359212389160499, 354.630774329461644, 113.373708671587772, 19.9559488532742796, 1.59407954898394322};
__device__ constexpr double kBD3[8] = {2570.7250703533430, 2972.7443644211129, 2393.9995533270879, 1259.0724833462608, 459.86413596901097, 112.60906419590854, 16.468882811659000, 1.0};
__device__ constexpr double kAN4[4] = {18247.2542465629199, 2120.56302902849207, 54.659507299984584, 0.121876197098273914};
__device__ constexpr double kAD4[4] = {24329.6723287505678, 3261.01909656925521, 117.071576489684022, 1.0};
__device__ constexpr double kBN4[8] = {33093.9102025608137, 19031.4783357798975, 5431.08357152245897, 2393.94262931609398, 1268.40017257978070, 418.662172475927160, 77.4108960876508190, 6.67374311450268357};
__device__ constexpr double kBD4[8] = {2645.4885670047153, 3236.2237702166948, 2500.5977847175497, 1278.0109577275445, 448.99020896813485, 105.86020755838874, 15.216887271751039, 1.0};
__device__ constexpr double kAN5[4] = {81190.938912603315, 8368.4990332049831, 190.753830813273698, 0.413800735538960261};
__device__ constexpr double kAD5[4] = {43301.8340867217726, 4977.68099709243407, 148.484432990224213, 1.0};
__device__ constexpr double kBN5[8] = {159651.547840031111, 96307.2005742063042, 26923.5693307648389, 9274.54751848368696, 4445.76333033698006, 1461.45267097859337, 272.164427980501432, 23.6526046298891619};
__device__ constexpr double kBD5[8] = {2522.7839609396783, 3244.5527999477567, 2403.0532924519756, 1176.7202478443275, 397.7596246691212, 91.84661231161838, 13.491911254479298, 1.0};

template <int K> struct FdiCoef;

template <> struct FdiCoef<0>
{
    static constexpr double a0 = 1.;
    BNSN_DI static const double (&an())[5] { return kAN0; }
    BNSN_DI static const double (&ad())[5] { return kAD0; }
    BNSN_DI static const double (&bn())[9] { return kBN0; }
    BNSN_DI static const double (&bd())[8] { return kBD0; }
    BNSN_DI static double reflect(double fd, double y) { return fd + y; }
};

template <> struct FdiCoef<1>
{
    static constexpr double a0 = 1.;
    BNSN_DI static const double (&an())[5] { return kAN1; }
    BNSN_DI static const double (&ad())[5] { return kAD1; }
    BNSN_DI static const double (&bn())[9] { return kBN1; }
    BNSN_DI static const double (&bd())[9] { return kBD1; }
    BNSN_DI static double reflect(double fd, double y)
    {
        return -fd + 1.64493406684822644 + 0.5 * y * y;
    }
};

template <> struct FdiCoef<2>
{
    static constexpr double a0 = 2.;
    BNSN_DI static const double (&an())[4] { return kAN2; }
    BNSN_DI static const double (&ad())[4] { return kAD2; }
    BNSN_DI static const double (&bn())[9] { return kBN2; }
    BNSN_DI static const double (&bd())[9] { return kBD2; }
    BNSN_DI static double reflect(double fd, double y)
    {
        return fd + y * (3.28986813369645287 + 0.333333333333333333 * y * y);
    }
};

template <> struct FdiCoef<3>
{
    static constexpr double a0 = 6.;
    BNSN_DI static const double (&an())[4] { return kAN3; }
    BNSN_DI static const double (&ad())[4] { return kAD3; }
    BNSN_DI static const double (&bn())[8] { return kBN3; }
    BNSN_DI static const double (&bd())[8] { return kBD3; }
    BNSN_DI static double reflect(double fd, double y)
    {
        const double y2 = y * y;
        return -fd + 11.3643939539669510 + y2 * (4.93480220054467931 + y2 * 0.25);
    }
};

template <> struct FdiCoef<4>
{
    static constexpr double a0 = 24.;
    BNSN_DI static const double (&an())[4] { return kAN4; }
    BNSN_DI static const double (&ad())[4] { return kAD4; }
    BNSN_DI static const double (&bn())[8] { return kBN4; }
    BNSN_DI static const double (&bd())[8] { return kBD4; }
    BNSN_DI static double reflect(double fd, double y)
    {
        const double y2 = y * y;
        return fd + y * (45.4575758158678040 + y2 * (6.57973626739290575 + y2 * 0.2));
    }
};

template <> struct FdiCoef<5>
{
    static constexpr double a0 = 120.;
    BNSN_DI static const double (&an())[4] { return kAN5; }
    BNSN_DI static const double (&ad())[4] { return kAD5; }
    BNSN_DI static const double (&bn())[8] { return kBN5; }
    BNSN_DI static const double (&bd())[8] { return kBD5; }
    BNSN_DI static double reflect(double fd, double y)
    {
        const double y2 = y * y;
        return -fd + 236.532261911384425 +
               y2 * (113.643939539669510 +
                     y2 * (8.22467033424113218 + y2 * 0.166666666666666667));
    }
};


// F_K(y) for K = KLO..KHI at one argument; out[K - KLO].  The regime test and
// the exponential are shared by all orders.
template <int KLO, int KHI>
BNSN_DI void fdi_orders(double y, double* out)
{
    const double x = -fabs(y);
    if (x < -2.)
    {
        const double ex = exp(x);
        const double t  = ex * k::FdiLit;
#define BNSN_FDI_LOW(K)                                                          \
    if (KLO <= K && K <= KHI)                                                    \
        out[K - KLO] = ex * (FdiCoef<K>::a0 -                                    \
                             ex * horner(FdiCoef<K>::an(), t) / horner(FdiCoef<K>::ad(), t));
        BNSN_FDI_LOW(0) BNSN_FDI_LOW(1) BNSN_FDI_LOW(2)
        BNSN_FDI_LOW(3) BNSN_FDI_LOW(4) BNSN_FDI_LOW(5)
#undef BNSN_FDI_LOW
    }
    else if (x <= 0.)
    {
        const double s = -0.5 * x;
        const double t = 1. - s;
#define BNSN_FDI_MID(K)                                                          \
    if (KLO <= K && K <= KHI)                                                    \
        out[K - KLO] = horner(FdiCoef<K>::bn(), t) / horner(FdiCoef<K>::bd(), s);
        BNSN_FDI_MID(0) BNSN_FDI_MID(1) BNSN_FDI_MID(2)
        BNSN_FDI_MID(3) BNSN_FDI_MID(4) BNSN_FDI_MID(5)
#undef BNSN_FDI_MID
    }
    else
    {
#pragma unroll
        for (int kk = 0; kk <= KHI - KLO; ++kk)
            out[kk] = 0.;
    }
    if (y > 0.)
    {
#define BNSN_FDI_REF(K)                                                          \
    if (KLO <= K && K <= KHI)                                                    \
        out[K - KLO] = FdiCoef<K>::reflect(out[K - KLO], y);
        BNSN_FDI_REF(0) BNSN_FDI_REF(1) BNSN_FDI_REF(2)
        BNSN_FDI_REF(3) BNSN_FDI_REF(4) BNSN_FDI_REF(5)
#undef BNSN_FDI_REF
    }
}

template <int K>
BNSN_DI double fdi(double y)
{
    double v;
    fdi_orders<K, K>(y, &v);
    return v;
}

// ---------------------------------------------------------------------------
// Distribution function (distribution.hpp)
// ---------------------------------------------------------------------------

struct Distr
{
    double w_t[4], temp_t[4], eta_t[4], w_f[4], temp_f[4], c_f[4], beta_f[4];
};

// distribution.hpp:51-175 and :206-243 for one species; gamma36 is
// GammaStirling(3.6) (functions.hpp:4460-4471), evaluated on the host.
BNSN_DI void distr_species(double n_in, double J_in, double chi, double gamma36,
                           double* w_t, double* temp_t, double* eta_t,
                           double* w_f, double* temp_f, double* c_f,
                           double* beta_f)
{
    const double n = (n_in > 1e-100) ? n_in : 1e-100;
    const double J = (J_in > 1e-100) ? J_in : 1e-100;
    *w_t           = 1.5 * (1. - chi);
    const double q = n / J;
    const double y = n * (q * q * q) / k::FourPiHc3;
    double eta;
    if (y < 0.005)
    {
        const double num =
            y * (y * (y * (y * (y * (y + 0.19926987701997) + 38865.0149220478) +
                           14364.6331099737) + 5750.1878570758) + 1120.71610972194) +
            1.60356108438235e-8;
        const double den =
            y * (y * (y * (y * (y * (y + 1.0) + 38840.0743174942) - 99.9009680656931) -
                      171.874844843596) + 75.7101579899442) + 83.0160130941424;
        eta = log(num / den);
    }
    else if (y <= 0.7)
    {
        const double num =
            y * (y * (y * (y * (y * (41.3836568203438 * y + 32.5515666786612) -
                                157.774993512235) + 66.5726772426253) +
                      14.4883415579211) + 0.315360380575709) + 0.000660414331285249;
        const double den =
            y * (y * (y * (y * (y * (y + 1.8888797407042) - 5.35488690539183) +
                           1.94673781342617) + 0.483128792035557) +
                 0.0113386564109086) + 2.64160073447322e-5;
        eta = num / den - 30.;
    }
    else if (y > 0.7 && y < 0.7901234567745267)
    {
        const double num =
            y * (y * (y * (y * (y * (3852.81416018959 * y - 5316.18895799799) +
                                1102.91561586553) + 1.54082262710661e-6) +
                      1732.89925128741) - 1769.59868329086) + 586.406885304906;
        const double den =
            y * (y * (y * (y * (y * (y + 255.936658313629) + 9.42360945627147e-5) -
                           81.2467063138386) - 180.100197053091) - 89.0343496217014) +
            143.849128123195;
        eta = exp(num / den);
    }
    else
    {
        eta = 20.;
    }
    eta = (eta < 20.) ? eta : 20.;
    double f23[2];
    fdi_orders<2, 3>(eta, f23);
    *eta_t  = eta;
    *temp_t = f23[0] * J / (f23[1] * n);

    *w_f             = 0.5 * (3. * chi - 1.);
    *c_f             = k::CF;
    const double Tnu = J / (n * (k::CF + 3.));
    *temp_f          = Tnu;
    *beta_f          = n / (k::FourPiHc3 * gamma36 * pow(Tnu, k::CF + 3.));
}

// distribution.hpp:298-315 (TotalNuF) for the 4 species at one energy;
// pow(omega, c_f) is evaluated once when the species share c_f.
BNSN_DI void total_nu_f4(double omega, const Distr& d, bool same_cf, double* g)
{
    double pw = same_cf ? pow(omega, d.c_f[0]) : 0.;
#pragma unroll
    for (int s = 0; s < 4; ++s)
    {
        const double T_t = d.temp_t[s];
        const double ft  = fermi_distr(omega, T_t, d.temp_t[s] * d.eta_t[s]);
        const double p   = same_cf ? pw : pow(omega, d.c_f[s]);
        const double fn  = d.beta_f[s] * p * exp(-omega / d.temp_f[s]);
        g[s]             = d.w_t[s] * ft + d.w_f[s] * fn;
    }
}

// ---------------------------------------------------------------------------
// Weak magnetism (weak_magnetism.hpp)
// ---------------------------------------------------------------------------

// weak_magnetism.hpp:45-104; reac 1: protons, 2: neutrons, 3: charged current.
// The four quotients by (1 + tau) share one reciprocal (FP64 division is a
// multi-instruction sequence on the FP64 pipe; the results move by an ulp).
BNSN_DI void nuc_form_factors(double E, int reac, double* cv, double* ca, double* F2)
{
    const double lamp = 1.793, lamn = -1.913;
    const double ehor = E * k::WmEScale;
    const double tau  = 0.5 * (ehor * ehor) / (1. + ehor);
    const double eta  = 1. / (1. + 5.6 * tau);
    const double gq   = 1. + 4.97 * tau;
    const double Gt   = 1. / ((gq * gq) * (1. + tau)); // G / (1 + tau)
    const double Fp1  = (1. + tau * (1. + lamp)) * Gt;
    const double Fp2  = lamp * Gt;
    const double Fn1  = tau * lamn * (1. - eta) * Gt;
    const double Fn2  = lamn * (1. + tau * eta) * Gt;
    const double d3   = 1. + 3.53 * tau;
    if (reac == 1)
    {
        *cv = (0.5 - 2. * k::SinThW2) * Fp1 - 0.5 * Fn1;
        *ca = 0.5 * (k::Ga - k::Gs) / (d3 * d3);
        *F2 = (0.5 - 2. * k::SinThW2) * Fp2 - 0.5 * Fn2;
    }
    else if (reac == 2)
    {
        *cv = (0.5 - 2. * k::SinThW2) * Fn1 - 0.5 * Fp1;
        *ca = -0.5 * (k::Ga + k::Gs) / (d3 * d3);
        *F2 = (0.5 - 2. * k::SinThW2) * Fn2 - 0.5 * Fp2;
    }
    else
    {
        *cv = Fp1 - Fn1;
        *ca = k::Ga / (d3 * d3);
        *F2 = Fp2 - Fn2;
    }
}

// weak_magnetism.hpp:123-160
BNSN_DI void wm_abs_em(double omega, double* R, double* Rbar)
{
    double cv, ca, F2;
    nuc_form_factors(omega, 3, &cv, &ca, &F2);
    const double e  = omega * k::WmEScale;
    const double e2 = e * e;
    const double a  = 1. + (4. / 3.) * e;
    const double b  = 1. + 2. * e;
    const double tmp1 = (cv * cv) * (1. + 4. * e + (16. / 3.) * e2) + 3. * ca * ca * (a * a) +
                        (8. / 3.) * cv * F2 * e2 +
                        (5. / 3.) * e2 * (1. + (2. / 5.) * e) * (F2 * F2);
    const double tmp2 = 4. * (cv + F2) * ca * e * (1. + (4. / 3.) * e);
    const double itmp3 = 1. / (((k::Gv * k::Gv) + 3. * (k::Ga * k::Ga)) * (b * b * b));
    *R    = (tmp1 + tmp2) * itmp3;
    *Rbar = (tmp1 - tmp2) * itmp3;
}

// weak_magnetism.hpp:165-210
BNSN_DI void wm_scatt(double omega, int reac, double* R0, double* R1)
{
    double cv, ca, F2;
    nuc_form_factors(omega, reac, &cv, &ca, &F2);
    constexpr double ih0p = 1. / k::IsoH0p, ih0n = 1. / k::IsoH0n;
    constexpr double ih1p = 1. / k::IsoH1p, ih1n = 1. / k::IsoH1n;
    const double ih0 = reac == 1 ? ih0p : ih0n;
    const double ih1 = reac == 1 ? ih1p : ih1n;
    const double e  = omega * k::WmEScale;
    const double ef = e * F2;
    *R0 = ((cv * cv) + 3. * (ca * ca) + 1.5 * (ef * ef) + 2. * (e * e) * cv * F2) * ih0;
    *R1 = ((cv * cv) - (ca * ca) - 2. * (ef * ef) - 4. * (e * e) * cv * F2) * ih1;
}

// ---------------------------------------------------------------------------
// Beta processes (formulas_beta_iso.hpp:64-341)
// ---------------------------------------------------------------------------

// formulas_beta_iso.hpp:64-97
BNSN_DI double eta_nn_abs(double n_in, double n_out, double mu_hat, double T)
{
    if (fabs(mu_hat) < 1.0e-02)
        return n_in;
    const double etanp = (n_out - n_in) / (safe_exp(-mu_hat / T) - 1.);
    return etanp < 0. ? n_in : etanp;
}

// Per-point constants of AbsOpacitySingleLep for electrons.
struct BetaPoint
{
    double T, Qprime, etanp, etapn, mu_e, mu_p, mu_n;
    int use_WM_ab, use_decay;
};

BNSN_DI BetaPoint beta_point(double nb, double T, double yp, double yn,
                             double mu_p, double mu_n, double mu_e, double dU_in,
                             double dm_eff, bool use_dU, bool use_dm_eff,
                             bool use_WM_ab, bool use_decay)
{
    BetaPoint b;
    const double dU  = use_dU ? dU_in : 0.;
    const double dQ  = use_dm_eff ? dm_eff : k::Q;
    const double nn  = nb * yn;
    const double np  = nb * yp;
    const double mu_hat = mu_n - mu_p - dQ;
    b.Qprime    = dQ + dU;
    const double mu_np = mu_hat - dU;
    b.etanp     = eta_nn_abs(nn, np, mu_np, T);
    b.etapn     = eta_nn_abs(np, nn, -mu_np, T);
    b.T         = T;
    b.mu_e      = mu_e;
    b.mu_p      = mu_p;
    b.mu_n      = mu_n;
    b.use_WM_ab = use_WM_ab;
    b.use_decay = use_decay;
    return b;
}

// formulas_beta_iso.hpp:138-279 for one species: anti = 0 gives
// (absorption, emission) of nu_e, anti = 1 of anti-nu_e, [s^-1].
BNSN_DI void beta_rates(const BetaPoint& b, double omega, int anti, double* ab,
                        double* em)
{
    const double m2 = k::Me * k::Me;
    double R = 1., Rbar = 1.;
    if (b.use_WM_ab)
        wm_abs_em(omega, &R, &Rbar);
    double cap = 0., dec = 0.;
    if (!anti)
    {
        const double Ee = omega + b.Qprime, Ep = -Ee;
        const double Ee2 = Ee * Ee, Ep2 = Ep * Ep;
        const double fe = fermi_distr(Ee, b.T, +b.mu_e);
        const double fp = fermi_distr(Ep, b.T, -b.mu_e);
        if (Ee - k::Me >= 0.)
            cap = Ee2 * sqrt(1. - m2 / Ee2) * R;
        if (b.use_decay && Ep - k::Me >= 0.)
            dec = Ep2 * sqrt(1. - m2 / Ep2);
        *em = k::BetaConst * b.etapn * (cap * fe + dec * (1. - fp));
        *ab = *em * safe_exp((omega - (b.mu_p + b.mu_e - b.mu_n)) / b.T);
    }
    else
    {
        const double Ep = omega - b.Qprime, Ee = -Ep;
        const double Ee2 = Ee * Ee, Ep2 = Ep * Ep;
        const double fe = fermi_distr(Ee, b.T, +b.mu_e);
        const double fp = fermi_distr(Ep, b.T, -b.mu_e);
        if (Ep - k::Me >= 0.)
            cap = Ep2 * sqrt(1. - m2 / Ep2) * Rbar;
        if (b.use_decay && Ee - k::Me >= 0.)
            dec = Ee2 * sqrt(1. - m2 / Ee2);
        *em = k::BetaConst * b.etanp * (cap * fp + dec * (1. - fe));
        *ab = *em * safe_exp((omega - (b.mu_n - b.mu_p - b.mu_e)) / b.T);
    }
}

// ---------------------------------------------------------------------------
// Iso-energetic scattering (formulas_beta_iso.hpp:371-564)
// ---------------------------------------------------------------------------

// formulas_beta_iso.hpp:371-395
BNSN_DI double eta_nn_sc(double nb, double temp, double yN)
{
    const double nN = yN * nb;
    if (nN <= 0.)
        return 0.;
    const double eFN = k::IsoEf * pow(nN, 2. / 3.);
    const double aux = 1.5 * temp / eFN;
    return nN * aux / sqrt(1. + aux * aux);
}

// formulas_beta_iso.hpp:411-507: IsoScattTotal with the two eta_NN factors
// precomputed per point.
BNSN_DI double iso_scatt_total(double omega, double eta_pp, double eta_nn,
                               bool use_wm)
{
    double R0p = 1., R1p = 1., R0n = 1., R1n = 1.;
    if (use_wm)
    {
        wm_scatt(omega, 1, &R0p, &R1p);
        wm_scatt(omega, 2, &R0n, &R1n);
    }
    constexpr double third = 1. / 3.;
    const double pr = eta_pp * ((k::IsoC0p * R0p) - (k::IsoC1p * R1p) * third);
    const double ne = eta_nn * ((k::IsoC0n * R0n) - (k::IsoC1n * R1n) * third);
    return pr + ne;
}

// formulas_beta_iso.hpp:523-564 (l = 0)
BNSN_DI double iso_scatt_leg0(double omega, double eta_pp, double eta_nn, bool use_wm)
{
    double R0p = 1., R1p = 1., R0n = 1., R1n = 1.;
    if (use_wm)
    {
        wm_scatt(omega, 1, &R0p, &R1p);
        wm_scatt(omega, 2, &R0n, &R1n);
    }
    return eta_pp * k::IsoC0p * R0p + eta_nn * k::IsoC0n * R0n;
}

// ---------------------------------------------------------------------------
// e+e- pair kernel (kernel_pair.hpp:16-198)
// ---------------------------------------------------------------------------

// Fermi integrals F_1..F_5 at eta - y (m) and eta + y (p) of one energy.
struct PairEnergyFdi
{
    double m[5], p[5];
};

// Psi_0(y, z) and Psi_0(z, y) of kernel_pair.hpp:16-120 from the per-energy
// Fermi integrals: fam[k-1] = F_k(eta - y), fap = F_k(eta + y), fbm / fbp the
// same for z; f3e / f4e are F_3(eta), F_4(eta).  Zero when eta - y - z > 200.
BNSN_DI void pair_psi(double eta, double y, double z, const double* fam, const double* fap,
                      const double* fbm, const double* fbp, double f3e, double f4e,
                      double* psi0, double* psi1)
{
    *psi0 = 0.;
    *psi1 = 0.;
    if (eta - y - z > 200.)
        return;
    double fmyz[3], fpyz[3];
    fdi_orders<3, 5>(eta - y - z, fmyz);
    fdi_orders<3, 5>(eta + y + z, fpyz);
    const double c0  = 20. * fam[3];
    const double c1  = 20. * fbp[3];
    const double c2  = 120. * fam[1] - 120. * fbp[1];
    const double c3  = -40. * fam[2] + 40. * fbp[2];
    const double c4  = 40. * f3e;
    const double c5  = 40. * fmyz[0] - c4;
    const double c6  = -20. * f4e;
    const double c7  = 20. * fmyz[1] + c6;
    const double c8  = -40. * fpyz[0] + c4;
    const double c9  = 20. * fpyz[1] + c6;
    const double c10 = -4. * fam[4] + 4. * fmyz[2] - 4. * fbm[4] + 4. * fap[4] -
                       4. * fpyz[2] + 4. * fbp[4];
    const double c11 = 20. * fap[3];
    const double c12 = 20. * fbm[3];
    const double c13 = -40. * fbm[2] + 40. * fap[2];
    const double c14 = 120. * fbm[1] - 120. * fap[1];
    const double yz  = y * z;
    const double den = 15. * (yz * yz);
    const double p0 =
        c10 +
        y * (-c0 + c1 + c7 +
             y * (c3 + c5 + z * (c2 + z * (-120. * fam[0] + 120. * fbp[0]))) +
             z * (80. * fam[2] - 80. * fbp[2] - c2 * z)) +
        z * (c0 - c1 + c9 + z * (c3 + c8));
    const double p1 =
        c10 + y * (-c11 + c12 + c9 + y * (c13 + c8)) +
        z * (c11 - c12 + c7 + y * (80. * fbm[2] - 80. * fap[2] - c14 * y) +
             z * (c13 + c5 + y * (c14 + y * (-120. * fbm[0] + 120. * fap[0]))));
    *psi0 = p0 / den;
    *psi1 = p1 / den;
}

// Pair kernel at (omega = y T, omega' = z T), kernel_pair.hpp:135-198:
// em[4] = Phi/2 per species, ab[4] = e^{(w + w')/T} em.
BNSN_DI void pair_kernel(double T, double eta, double omega, double omega_p,
                         double y, double z, const double* fam, const double* fap,
                         const double* fbm, const double* fbp, double f3e,
                         double f4e, double* em, double* ab)
{
    double psi0, psi1;
    pair_psi(eta, y, z, fam, fap, fbm, fbp, f3e, f4e, &psi0, &psi1);
    const double aux = k::PairPhi * (T * T) / (1. - safe_exp(y + z));
    const double phi0 = ((k::PairA1e * k::PairA1e) * psi0 + (k::PairA2e * k::PairA2e) * psi1) * aux;
    const double phi1 = ((k::PairA1e * k::PairA1e) * psi1 + (k::PairA2e * k::PairA2e) * psi0) * aux;
    const double phi2 = ((k::PairA1x * k::PairA1x) * psi0 + (k::PairA2x * k::PairA2x) * psi1) * aux;
    const double phi3 = ((k::PairA1x * k::PairA1x) * psi1 + (k::PairA2x * k::PairA2x) * psi0) * aux;
    em[0] = 0.5 * phi0;
    em[1] = 0.5 * phi1;
    em[2] = 0.5 * phi2;
    em[3] = 0.5 * phi3;
    const double ex = safe_exp((omega + omega_p) / T);
#pragma unroll
    for (int s = 0; s < 4; ++s)
        ab[s] = ex * em[s];
}

// ---------------------------------------------------------------------------
// HR98 bremsstrahlung (kernel_brem_HR98.hpp:33-393)
// ---------------------------------------------------------------------------

// Quantities of one NN channel that do not depend on the energy pair.
struct Hr98Channel
{
    double weight;  // n_nuc (x 28/3 for np) entering the channel sum
    double gamma;   // spin-fluctuation rate, Eq.(37)
    double hgg;     // 0.5 gamma g(y, eta*), Eq.(35) denominator
    double K1;      // 3 (pi/2)^2.5 eta*^-2.5 of s_d, Eq.(46)
    double f_u;     // f(u) of s_d
    double eta2p1;  // 1 + eta*^2 of F, Eq.(50)
    double sqe;     // sqrt(eta*) of G
    double ep2;     // eta* + 0.2 of G
    double h;       // h(eta*) of C
};

// Channel-independent per-point quantities (y depends only on T).
struct Hr98Point
{
    double T, y, ey12, poly_y, y4p1, Dy, mp, minv, mcorr;
    Hr98Channel ch[3];
};

// kernel_brem_HR98.hpp:165-236: g(y, eta*) with the clamps of the fit.
BNSN_DI double hr98_g(double y, double eta_star)
{
    y        = (y > k::BremYmin) ? y : k::BremYmin;
    eta_star = (eta_star > k::BremEtamin) ? eta_star : k::BremEtamin;
    const double y2    = y * y;
    const double inv   = 1. / eta_star;
    const double a1den = 25. * y2 + 1.;
    const double a1    = (0.5 + inv) / (1. + inv) * (1. / a1den) +
                      (0.5 + eta_star / 15.6) * 25. * y2 / a1den;
    const double a2  = (0.63 + 0.04 * pow(eta_star, 1.45)) / (1. + 0.02 * pow(eta_star, 2.5));
    const double p15 = pow(eta_star, 1.5);
    const double a3  = 1.2 * safe_exp(0.6 * eta_star - 0.4 * p15);
    const double p1  = (1.8 + 0.45 * eta_star) / (1. + 0.15 * p15);
    const double p2  = 2.3 - 0.05 * eta_star / (1. + 0.025 * eta_star);
    return (a1 + a2 * pow(y, p1)) / (1. + a3 * pow(y, p2) + a2 * pow(y, p1 + 2.) / 13.75);
}

// Channel constants (kernel_brem_HR98.hpp:239-289 for everything but x);
// ch = 0: nn, 1: pp, 2: np.
BNSN_DI Hr98Channel hr98_channel(double nb, double yn, double yp, double T, int ch)
{
    Hr98Channel c;
    double n_nuc, m_nuc;
    if (ch == 0)
    {
        n_nuc    = nb * yn;
        m_nuc    = k::MnGrams;
        c.weight = n_nuc;
    }
    else if (ch == 1)
    {
        n_nuc    = nb * yp;
        m_nuc    = k::MpGrams;
        c.weight = n_nuc;
    }
    else
    {
        n_nuc    = nb * sqrt(yn * yp);
        m_nuc    = k::MAvgGrams;
        c.weight = (28. / 3.) * n_nuc;
    }
    const double T10  = T * 0.1;
    const double etas = pow(3. * k::PiSq * n_nuc, 2. / 3.) * k::BremAux1 / (2. * m_nuc * T);
    c.gamma           = 1.63 * pow(etas, 1.5) * T10;
    const double y    = 1.94 / T10;
    const double gb   = hr98_g(y, etas);
    c.hgg             = 0.5 * c.gamma * gb;
    // s-component constants (the fit clamps eta* from below)
    const double e    = (etas > k::BremEtamin) ? etas : k::BremEtamin;
    const double yc   = (y > k::BremYmin) ? y : k::BremYmin;
    const double u    = sqrt(yc / (2. * e)) + 1.e-10;
    const double u2   = u * u;
    const double uarg = u2 / (2. * sqrt(2. * u2 + 4.));
    double f_u        = (1. - 5. * u * atan(2. / u) / 6. + u2 / (3. * (u2 + 4.)) +
                  atan(1. / uarg) * uarg / 3.);
    c.f_u    = (fabs(f_u) < 1.e-14) ? 1.e-14 : f_u;
    c.K1     = 3. * k::PiHalf52 * pow(e, -2.5);
    c.eta2p1 = 1. + e * e;
    c.sqe    = sqrt(e);
    c.ep2    = e + 0.2;
    c.h      = 0.1 * e / (2.39 + 0.1 * pow(e, 1.1));
    return c;
}

// Channel-independent part; the channels are filled separately so that three
// lanes can compute them in parallel.
BNSN_DI void hr98_point_common(double nb, double T, bool medium, Hr98Point* P)
{
    P->T          = T;
    const double y = 1.94 / (T * 0.1);
    const double yc = (y > k::BremYmin) ? y : k::BremYmin;
    P->y          = yc;
    P->ey12       = safe_exp(-yc / 12.);
    P->poly_y     = 5. * (yc * yc) / 3.;
    P->y4p1       = 1. + yc * yc * yc * yc;
    P->Dy         = 0.8 + 0.06 * pow(yc, 1.05);
    const double p = 0.67 + 0.18 * pow(yc, 0.4);
    P->mp         = -p;
    P->minv       = -1. / p;
    if (medium)
    {
        const double q = (1. + cbrt(nb / k::SatN) / 3.);
        P->mcorr       = q * q * q * q * q * q;
    }
    else
    {
        P->mcorr = 1.;
    }
}

// l = 0 HR98 kernel (kernel_brem_HR98.hpp:342-393) at x = (w + w')/T:
// absorption and emission (detailed balance) kernels.
BNSN_DI void hr98_kernel(const Hr98Point& P, double omega, double omega_p,
                         double* em, double* ab)
{
    const double x  = (omega + omega_p) / P.T;
    const double xs = (x > k::BremXmin) ? x : k::BremXmin;
    const double y  = P.y;
    // s_nd, Eq.(45)
    const double snd_num = 2. * k::SqrtPi * pow(xs + 2. - P.ey12, 1.5) *
                           ((xs * xs) + 2. * xs * y + P.poly_y + 1.);
    const double q       = k::Pi18 + xs + y;
    const double s_nd    = snd_num / (k::SqrtPi + q * q * q * q);
    const double X2      = (xs * xs) + k::FourPiSq;
    const double den_sd  = k::FourPiSq * (1. - safe_exp(-xs));
    const double px11    = pow(xs, 1.1);
    const double xterm   = 3. + (xs - 1.2) * (xs - 1.2) + pow(xs, -4.);
    const double gpart   = 0.0044 * px11 * y / P.Dy;
    const double cnum    = 1.1 * px11;
    const double px093   = pow(xs, 0.93);
    const double px12    = 0.0001 * pow(xs, 1.2);
    const double cden2   = 30. + 0.005 * pow(xs, 2.8);
    const double snd_p   = pow(s_nd, P.mp);
    const double x2      = x * x;
    double tot           = 0.;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        const Hr98Channel& C = P.ch[c];
        const double s_d     = C.K1 * X2 * xs * C.f_u / den_sd;
        const double f_brem  = 1. + 1. / (xterm * C.eta2p1 * P.y4p1);
        const double g_brem  = 1. - gpart * C.sqe / C.ep2;
        const double c_brem  = cnum * C.h / (2.3 + C.h * px093 + px12) * 30. / cden2;
        const double s = pow(snd_p + pow(s_d, P.mp), P.minv) * f_brem * (1. + c_brem * g_brem);
        const double chan = C.gamma / (x2 + C.hgg * C.hgg) * s / P.T;
        tot += C.weight * chan;
    }
    double sab = k::BremConst * tot;
    sab        = sab / P.mcorr;
    sab        = 3. * sab;
    *ab        = sab;
    *em        = sab * safe_exp(-x);
}

// ---------------------------------------------------------------------------
// BRT06 bremsstrahlung (kernel_brem_BRT06.hpp:24-69)
// ---------------------------------------------------------------------------

// q_nb / T^7 with the leading constants (per point).
BNSN_DI double brt06_point(double nb, double T, double yn, double yp)
{
    const double rho = nb * k::Mb;
    const double q   = 2.0778e+02 * 0.5 * k::MeV *
                     ((yn * yn) + (yp * yp) + (28. / 3.) * yn * yp) * (rho * rho) *
                     pow(T, 5.5);
    const double T7 = T * T * T * T * T * T * T;
    return k::HC6FourPi2 * k::BremC4BRT06 * (q / T7);
}

BNSN_DI void brt06_kernel(double pre, double T, double omega, double omega_p,
                          double* em, double* ab)
{
    const double x   = 0.5 * (omega + omega_p) / T;
    const double tmp = pre * bessk1(x) / x;
    *em              = tmp * safe_exp(-x);
    *ab              = tmp * safe_exp(x);
}

// ---------------------------------------------------------------------------
// GP19 bremsstrahlung (kernel_brem_GP19.hpp:35-481), table in global memory
// ---------------------------------------------------------------------------

struct Gp19Table
{
    int d0, d1, d2, d3;
    const double *nb, *ye, *t, *w, *lognb, *logw, *data;
};

// First interval [ax[i], ax[i+1]] containing v (the reference's linear scan
// returns the first such i), by binary search; -1 outside the axis.
BNSN_DI int gp19_bracket(double v, const double* ax, int n, double* t)
{
    if (v < ax[0] || v > ax[n - 1])
        return -1;
    // smallest i in [0, n-2] with v <= ax[i+1]
    int lo = 0, hi = n - 2;
    while (lo < hi)
    {
        const int mid = (lo + hi) >> 1;
        if (v <= ax[mid + 1])
            hi = mid;
        else
            lo = mid + 1;
    }
    if (!(v >= ax[lo] && v <= ax[lo + 1]))
        return -1;
    *t = (v - ax[lo]) / (ax[lo + 1] - ax[lo]);
    return lo;
}

BNSN_DI double gp19_interp(const Gp19Table& G, double nb, double ye, double T, double w)
{
    double tx, ty, tz, tw;
    const int i = gp19_bracket(log(nb), G.lognb, G.d0, &tx);
    const int j = gp19_bracket(ye, G.ye, G.d1, &ty);
    const int kk = gp19_bracket(T, G.t, G.d2, &tz);
    const int l = gp19_bracket(log(w), G.logw, G.d3, &tw);
    if (i < 0 || j < 0 || kk < 0 || l < 0)
        return __longlong_as_double(0x7ff8000000000000LL);
    const double* g = G.data;
    const int D1 = G.d1, D2 = G.d2, D3 = G.d3;
    auto at = [&](int a, int b, int c, int e) {
        return __ldg(&g[(((int64_t)(a) * D1 + b) * D2 + c) * D3 + e]);
    };
    const double a0 = 1. - tx, a1 = tx, b0 = 1. - ty, b1 = ty;
    const double c0 = 1. - tz, c1 = tz, d0 = 1. - tw, d1 = tw;
    return at(i, j, kk, l) * a0 * b0 * c0 * d0 + at(i, j, kk, l + 1) * a0 * b0 * c0 * d1 +
           at(i, j, kk + 1, l) * a0 * b0 * c1 * d0 + at(i, j, kk + 1, l + 1) * a0 * b0 * c1 * d1 +
           at(i, j + 1, kk, l) * a0 * b1 * c0 * d0 + at(i, j + 1, kk, l + 1) * a0 * b1 * c0 * d1 +
           at(i, j + 1, kk + 1, l) * a0 * b1 * c1 * d0 +
           at(i, j + 1, kk + 1, l + 1) * a0 * b1 * c1 * d1 +
           at(i + 1, j, kk, l) * a1 * b0 * c0 * d0 + at(i + 1, j, kk, l + 1) * a1 * b0 * c0 * d1 +
           at(i + 1, j, kk + 1, l) * a1 * b0 * c1 * d0 +
           at(i + 1, j, kk + 1, l + 1) * a1 * b0 * c1 * d1 +
           at(i + 1, j + 1, kk, l) * a1 * b1 * c0 * d0 +
           at(i + 1, j + 1, kk, l + 1) * a1 * b1 * c0 * d1 +
           at(i + 1, j + 1, kk + 1, l) * a1 * b1 * c1 * d0 +
           at(i + 1, j + 1, kk + 1, l + 1) * a1 * b1 * c1 * d1;
}

BNSN_DI double gp19_in_range(const Gp19Table& G, double nb, double ye, double T, double w)
{
    return k::BremConst * (nb * 1e+18) * gp19_interp(G, nb, ye, T, w);
}

BNSN_DI double gp19_low_nb(const Gp19Table& G, double nb, double ye, double T, double w)
{
    const double nbmin = G.nb[0];
    const double r     = nb / nbmin;
    return gp19_in_range(G, nbmin, ye, T, w) * (r * r);
}

BNSN_DI double gp19_high_t(const Gp19Table& G, double nb, double ye, double T, double w)
{
    const double nbnm  = nb * 1e+18;
    const double nbnm2 = nbnm * nbnm;
    const double w2    = w * w;
    const double s50   = 7.0710678118654755;
    const double R48   = gp19_in_range(G, nb, ye, 48.0, w);
    const double R50   = gp19_in_range(G, nb, ye, 50.0, w);
    const double K     = 4. * k::BremConst * nbnm2;
    const double A     = 1. / R50;
    const double B     = 1. / (K * s50);
    const double m     = (R50 - R48) / (50.0 - 48.0);
    const double beta  = 8. * w2 * K * (B * B) / (2. * m * (A * A) * s50 + A * K * B);
    const double gamma = ((A * beta) - (4. * B * w2)) / (B * nbnm2 * 50.0);
    const double inv   = 1. / ((w / T) * (w / T) + (nbnm2 / (4. * T)) * gamma);
    const double S     = (beta * nbnm) / (T * sqrt(T)) * inv;
    return k::BremConst * nbnm * S;
}

// ---------------------------------------------------------------------------
// GP19 per point: for fixed (nb, Ye, T) the multilinear interpolation of
// kernel_brem_GP19.hpp:75-139 is linear in the table's w column, so a point
// needs at most two 1-D profiles over the w axis (computed once) and every
// (w, w') cell only brackets log w.  The regimes follow BremKernelAbsGP19
// (kernel_brem_GP19.hpp:357-481):
//   0 in range; 1 nb < nb_min (scaled by (nb/nb_min)^2); 2 nb < nb_min and
//   T < T_min; 3 nb < nb_min and T > T_max; 4 T < T_min; 5 T > T_max.
// Profiles: regimes 0, 1 use p0 at (nb', Ye', T); 2, 4 use p0 at T = 2 and
// p1 at T = 4; 3, 5 use p0 at T = 48 and p1 at T = 50 (nb' = nb_min for 1-3).
// ---------------------------------------------------------------------------
constexpr int kGp19MaxW = 64; // w-axis length handled with profiles

struct Gp19Point
{
    int regime;
    double C;     // BremConst * nb' * 1e18 (x (nb/nb_min)^2 in regimes 1, 2)
    double nbnm;  // nb' * 1e18 of the high-T extrapolation
    double r2;    // (nb/nb_min)^2 of regime 3
    double T;
    double pT[2]; // temperatures of the two profiles
    double nbp;   // nb' of the profiles [fm^-3]
    double yep;   // Ye' of the profiles
};

BNSN_DI void gp19_point(const Gp19Table& G, double nb_nm, double ye_in, double T, Gp19Point* P)
{
    double ye = ye_in, nb = nb_nm * 1e-18;
    const double nbmax = G.nb[G.d0 - 1], nbmin = G.nb[0];
    const double yemax = G.ye[G.d1 - 1];
    const double Tmax = G.t[G.d2 - 1], Tmin = G.t[0];
    if (ye > yemax)
        ye = yemax;
    if (nb > nbmax)
        nb = nbmax;
    P->T    = T;
    P->yep  = ye;
    P->r2   = 1.;
    P->pT[0] = P->pT[1] = T;
    if (nb < nbmin)
    {
        const double r = nb / nbmin;
        P->nbp  = nbmin;
        P->nbnm = nbmin * 1e+18;
        if (T < Tmin)
        {
            P->regime = 2;
            P->pT[0]  = 2.0;
            P->pT[1]  = 4.0;
            P->C      = k::BremConst * (nbmin * 1e+18) * (r * r);
        }
        else if (T > Tmax)
        {
            P->regime = 3;
            P->pT[0]  = 48.0;
            P->pT[1]  = 50.0;
            P->C      = k::BremConst * (nbmin * 1e+18);
            P->r2     = r * r;
        }
        else
        {
            P->regime = 1;
            P->C      = k::BremConst * (nbmin * 1e+18) * (r * r);
        }
    }
    else
    {
        P->nbp  = nb;
        P->nbnm = nb * 1e+18;
        P->C    = k::BremConst * (nb * 1e+18);
        if (T < Tmin)
        {
            P->regime = 4;
            P->pT[0]  = 2.0;
            P->pT[1]  = 4.0;
        }
        else if (T > Tmax)
        {
            P->regime = 5;
            P->pT[0]  = 48.0;
            P->pT[1]  = 50.0;
        }
        else
            P->regime = 0;
    }
}

// The (nb', Ye', T') corner of the table and the 8 trilinear weights of a
// profile, the same for every w column: the brackets are found once per
// profile instead of once per entry.  ok = 0 where the reference's
// interpolation brackets fail.
struct Gp19Corners
{
    int64_t base; // offset of corner (i, j, k) at column 0
    double w[8];  // weights of (di, dj, dk) = (0,0,0), (0,0,1), (0,1,0), ..., (1,1,1)
    int ok;
};

BNSN_DI void gp19_profile_corners(const Gp19Table& G, double nbp, double yep, double Tp,
                                  Gp19Corners* C)
{
    double tx, ty, tz;
    const int i  = gp19_bracket(log(nbp), G.lognb, G.d0, &tx);
    const int j  = gp19_bracket(yep, G.ye, G.d1, &ty);
    const int kk = gp19_bracket(Tp, G.t, G.d2, &tz);
    C->ok = i >= 0 && j >= 0 && kk >= 0;
    if (!C->ok)
        return;
    C->base = (((int64_t)i * G.d1 + j) * G.d2 + kk) * G.d3;
    const double a0 = 1. - tx, a1 = tx, b0 = 1. - ty, b1 = ty, c0 = 1. - tz, c1 = tz;
    C->w[0] = a0 * b0 * c0;
    C->w[1] = a0 * b0 * c1;
    C->w[2] = a0 * b1 * c0;
    C->w[3] = a0 * b1 * c1;
    C->w[4] = a1 * b0 * c0;
    C->w[5] = a1 * b0 * c1;
    C->w[6] = a1 * b1 * c0;
    C->w[7] = a1 * b1 * c1;
}

// Profile entry at w column l: the trilinear interpolation in (nb, Ye, T) of
// the reference (kernel_brem_GP19.hpp); NaN where the brackets fail.
BNSN_DI double gp19_profile_eval(const Gp19Table& G, const Gp19Corners& C, int l)
{
    if (!C.ok)
        return __longlong_as_double(0x7ff8000000000000LL);
    const int64_t S2 = G.d3, S1 = (int64_t)G.d2 * G.d3, S0 = (int64_t)G.d1 * S1;
    const double* g = G.data + C.base + l;
    return __ldg(g) * C.w[0] + __ldg(g + S2) * C.w[1] + __ldg(g + S1) * C.w[2] +
           __ldg(g + S1 + S2) * C.w[3] + __ldg(g + S0) * C.w[4] + __ldg(g + S0 + S2) * C.w[5] +
           __ldg(g + S0 + S1) * C.w[6] + __ldg(g + S0 + S1 + S2) * C.w[7];
}

// The high-temperature extrapolation (kernel_brem_GP19.hpp:285-355) from the
// in-range kernels at T = 48 and 50 MeV.
BNSN_DI double gp19_high_t_from(double R48, double R50, double nbnm, double T, double w)
{
    const double nbnm2 = nbnm * nbnm;
    const double w2    = w * w;
    const double s50   = 7.0710678118654755;
    const double K     = 4. * k::BremConst * nbnm2;
    const double A     = 1. / R50;
    const double B     = 1. / (K * s50);
    const double m     = (R50 - R48) / (50.0 - 48.0);
    const double beta  = 8. * w2 * K * (B * B) / (2. * m * (A * A) * s50 + A * K * B);
    const double gamma = ((A * beta) - (4. * B * w2)) / (B * nbnm2 * 50.0);
    const double inv   = 1. / ((w / T) * (w / T) + (nbnm2 / (4. * T)) * gamma);
    const double S     = (beta * nbnm) / (T * sqrt(T)) * inv;
    return k::BremConst * nbnm * S;
}

// One cell from the profiles: v0, v1 are the profile values interpolated at
// the clipped w; w0 = omega + omega' unclipped.
BNSN_DI void gp19_cell(const Gp19Point& P, double v0, double v1, double w, double w0,
                       double* em, double* ab)
{
    double s;
    switch (P.regime)
    {
    case 0:
    case 1: s = P.C * v0; break;
    case 2:
    {
        const double eps = 1e-30;
        double k2 = P.C * v0, k4 = P.C * v1;
        k2 = (k2 < eps) ? eps : k2;
        k4 = (k4 < eps) ? eps : k4;
        const double m = log(k4 / k2) * 1.4426950408889634;
        s = k2 * pow(P.T * 0.5, m);
        s = (s < eps) ? eps : s;
        break;
    }
    case 4:
    {
        const double k2 = P.C * v0, k4 = P.C * v1;
        const double m  = log(k4 / k2) * 1.4426950408889634;
        s = k2 * pow(P.T * 0.5, m);
        break;
    }
    default: // 3, 5
        s = gp19_high_t_from(P.C * v0, P.C * v1, P.nbnm, P.T, w) * P.r2;
        break;
    }
    s   = fabs(3. * s);
    *ab = s;
    *em = s * safe_exp(-w0 / P.T);
}

// kernel_brem_GP19.hpp:357-481
BNSN_DI void gp19_kernel(const Gp19Table& G, double nb_nm, double ye_in, double T,
                         double omega, double omega_p, double* em, double* ab)
{
    double ye       = ye_in;
    double w        = omega + omega_p;
    const double w0 = w;
    double nb       = nb_nm * 1e-18;
    const double nbmax = G.nb[G.d0 - 1], nbmin = G.nb[0];
    const double yemax = G.ye[G.d1 - 1];
    const double Tmax = G.t[G.d2 - 1], Tmin = G.t[0];
    const double wmax = G.w[G.d3 - 1], wmin = G.w[0];
    if (ye > yemax)
        ye = yemax;
    if (nb > nbmax)
        nb = nbmax;
    if (w > wmax)
        w = wmax;
    else if (w < wmin)
        w = wmin;
    double s = 0.;
    if (nb >= nbmin && T >= Tmin && T <= Tmax)
        s = gp19_in_range(G, nb, ye, T, w);
    if (nb < nbmin)
    {
        if (T < Tmin)
        {
            const double eps = 1e-30;
            double k2 = gp19_low_nb(G, nb, ye, 2.0, w);
            double k4 = gp19_low_nb(G, nb, ye, 4.0, w);
            k2 = (k2 < eps) ? eps : k2;
            k4 = (k4 < eps) ? eps : k4;
            const double m = log(k4 / k2) * 1.4426950408889634;
            s = k2 * pow(T * 0.5, m);
            s = (s < eps) ? eps : s;
        }
        else if (T > Tmax)
        {
            const double r = nb / nbmin;
            s = gp19_high_t(G, nbmin, ye, T, w) * (r * r);
        }
        else
        {
            s = gp19_low_nb(G, nb, ye, T, w);
        }
    }
    else if (T < Tmin)
    {
        const double k2 = gp19_in_range(G, nb, ye, 2.0, w);
        const double k4 = gp19_in_range(G, nb, ye, 4.0, w);
        const double m  = log(k4 / k2) * 1.4426950408889634;
        s = k2 * pow(T * 0.5, m);
    }
    else if (T > Tmax)
    {
        s = gp19_high_t(G, nb, ye, T, w);
    }
    s   = fabs(3. * s);
    *ab = s;
    *em = s * safe_exp(-w0 / T);
}

// ---------------------------------------------------------------------------
// Inelastic scattering on electrons / positrons (kernel_nes.hpp)
// ---------------------------------------------------------------------------

// Per-point quantities of the NES (e = 0, eta = mu_e/T) and NPS (e = 1,
// eta = -mu_e/T) kernels: F_0..F_5 at eta (fe0 / fe1, in shared memory) and
// FermiDistr(0, 1, eta).
struct NepsPoint
{
    double T, pre; // pre = NEPS constant x T^2
    double eta0, eta1;
    double fd00, fd01;
    const double* fe0;
    const double* fe1;
};

// kernel_nes.hpp:50-78
BNSN_DI double mb_int_out(double w, double wp, double x, double y, int sign,
                          double b1, double b2, const double* dw, const double* dabs)
{
    return (((b1 + b2) * (sign * dabs[2] - dw[4]) * 0.2 -
             b1 * (w + wp) * (dw[3] + 2. * ((w + wp) * dw[2] + 3. * w * wp * dw[1])) +
             sign * ((b1 * x - b2 * y) * dabs[1] + 2. * (b1 * x * x + b2 * y * y) * dabs[0])) /
                (w * w * wp * wp) -
            6. * b1 * dw[0]);
}

// kernel_nes.hpp:82-107
BNSN_DI double mb_int_one(double x, double y, int sign, double b1, double b2, const double* f)
{
    return -sign * y *
           (2. * (b1 + b2) * f[0] + (b1 * (y + 4. * x) + 3. * b2 * y) * f[1] +
            (b1 * (3. * y - 4. * x) + b2 * y) * f[2] +
            ((b1 + 6. * b2) * y * y * 0.2 + b1 * x * y + 2. * b1 * x * x) * f[3] -
            ((6. * b1 + b2) * y * y * 0.2 - 3. * b1 * x * y + 2. * b1 * x * x) * f[4]) /
           (x * x);
}

// kernel_nes.hpp:111-132
BNSN_DI double mb_int_two(double w, double wp, double x, double y, double b1,
                          double b2, const double* f)
{
    return y * (w - wp) *
           ((b1 + b2) * (4. * f[2] + f[0] * (11. * y * y - 25. * x * y + 20. * x * x) / 30.) +
            (b1 - b2) * (2. * x - y) * f[1]) /
           (x * x);
}

// (b1, b2) couplings of species s for electrons (e = 0) and positrons (e = 1),
// kernel_nes.hpp:164-233 and :266-336.
BNSN_DI void neps_couplings(int e, int s, double* b1, double* b2)
{
    const double bo = (s < 2) ? k::NepsBPlus : k::NepsBMinus;
    const bool first = ((s & 1) == 0) != (e == 1);
    *b1 = first ? bo : k::NepsBZero;
    *b2 = first ? k::NepsBZero : bo;
}

// NES + NPS kernels (kernel_nes.hpp:139-359) for both directions of one
// energy pair: k1 = R(nu, nub), k2 = R(nub, nu); em/ab[4] each.  The Fermi
// integrals at eta - w, eta - w', eta - |w - w'| are evaluated once and
// shared by the two directions and the four species.
BNSN_DI void neps_pair(const NepsPoint& P, double nu, double nub, double* em1,
                       double* ab1, double* em2, double* ab2)
{
    const double T  = P.T;
    const double w  = nu / T;
    const double wp = nub / T;
    const double x  = (w > wp) ? w : wp;
    const double y  = (w < wp) ? w : wp;
    double efa, efb; // NEPSExpFunc(wp - w), NEPSExpFunc(w - wp)
    neps_exp_pair(wp - w, w - wp, &efa, &efb);
    const int sign1 = 2 * (signbit(wp - w) != 0) - 1;
    const int sign2 = 2 * (signbit(w - wp) != 0) - 1;
#pragma unroll
    for (int s = 0; s < 4; ++s)
    {
        em1[s] = ab1[s] = em2[s] = ab2[s] = 0.;
    }
#pragma unroll 1
    for (int e = 0; e < 2; ++e)
    {
        const double eta  = e ? P.eta1 : P.eta0;
        const double* f0e = e ? P.fe1 : P.fe0;
        const double fd0  = e ? P.fd01 : P.fd00;
        double r1[4], r2[4];
        if (y > eta * 1e-3)
        {
            double fw[5], fwp[5], fa[3];
            fdi_orders<1, 5>(eta - w, fw);
            fdi_orders<1, 5>(eta - wp, fwp);
            fdi_orders<3, 5>(eta - fabs(w - wp), fa);
            double dw1[5], dw2[5], dabs[3];
#pragma unroll
            for (int kk = 0; kk < 5; ++kk)
            {
                dw1[kk] = fwp[kk] - fw[kk];
                dw2[kk] = fw[kk] - fwp[kk];
            }
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
                dabs[kk] = f0e[3 + kk] - fa[kk];
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                double b1, b2;
                neps_couplings(e, s, &b1, &b2);
                r1[s] = P.pre * mb_int_out(w, wp, x, y, sign1, b1, b2, dw1, dabs);
                r2[s] = P.pre * mb_int_out(wp, w, x, y, sign2, b1, b2, dw2, dabs);
            }
        }
        else if (x > eta * 1e-3)
        {
            double fx[3];
            fdi_orders<0, 2>(eta - x, fx);
            const double f[5] = {fx[2] - f0e[2], fx[1], f0e[1],
                                 fx[0] + y * fermi_distr(0., 1., eta - x) / 6.,
                                 f0e[0] - y * fd0 / 6.};
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                double b1, b2;
                neps_couplings(e, s, &b1, &b2);
                r1[s] = P.pre * mb_int_one(x, y, sign1, b1, b2, f);
                r2[s] = P.pre * mb_int_one(x, y, sign2, b1, b2, f);
            }
        }
        else
        {
            const double f[3] = {fd0, f0e[0], f0e[1]};
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                double b1, b2;
                neps_couplings(e, s, &b1, &b2);
                r1[s] = P.pre * mb_int_two(w, wp, x, y, b1, b2, f);
                r2[s] = P.pre * mb_int_two(wp, w, x, y, b1, b2, f);
            }
        }
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            em1[s] += -r1[s] * efb;
            ab1[s] += r1[s] * efa;
            em2[s] += -r2[s] * efa;
            ab2[s] += r2[s] * efb;
        }
    }
}

// NES + NPS kernel R(nu, nub) in one direction (kernel_nes.hpp:139-359) for
// the spectral integrals; fw0 / fw1 hold F_0..F_5 at eta - nu/T for electrons
// and positrons (per energy, shared by all nodes).
BNSN_DI void neps_one(const NepsPoint& P, double nu, double nub, const double* fw0,
                      const double* fw1, double* em, double* ab)
{
    const double T  = P.T;
    const double w  = nu / T;
    const double wp = nub / T;
    const double x  = (w > wp) ? w : wp;
    const double y  = (w < wp) ? w : wp;
    double efa, efb;
    neps_exp_pair(wp - w, w - wp, &efa, &efb);
    const int sign = 2 * (signbit(wp - w) != 0) - 1;
#pragma unroll
    for (int s = 0; s < 4; ++s)
        em[s] = ab[s] = 0.;
#pragma unroll 1
    for (int e = 0; e < 2; ++e)
    {
        const double eta  = e ? P.eta1 : P.eta0;
        const double* f0e = e ? P.fe1 : P.fe0;
        const double fd0  = e ? P.fd01 : P.fd00;
        const double* fw  = e ? fw1 : fw0;
        double r[4];
        if (y > eta * 1e-3)
        {
            double fwp[5], fa[3], dw[5], dabs[3];
            fdi_orders<1, 5>(eta - wp, fwp);
            fdi_orders<3, 5>(eta - fabs(w - wp), fa);
#pragma unroll
            for (int kk = 0; kk < 5; ++kk)
                dw[kk] = fwp[kk] - fw[1 + kk];
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
                dabs[kk] = f0e[3 + kk] - fa[kk];
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                double b1, b2;
                neps_couplings(e, s, &b1, &b2);
                r[s] = P.pre * mb_int_out(w, wp, x, y, sign, b1, b2, dw, dabs);
            }
        }
        else if (x > eta * 1e-3)
        {
            double fx[3];
            if (x == w)
            {
                fx[0] = fw[0];
                fx[1] = fw[1];
                fx[2] = fw[2];
            }
            else
                fdi_orders<0, 2>(eta - x, fx);
            const double f[5] = {fx[2] - f0e[2], fx[1], f0e[1],
                                 fx[0] + y * fermi_distr(0., 1., eta - x) / 6.,
                                 f0e[0] - y * fd0 / 6.};
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                double b1, b2;
                neps_couplings(e, s, &b1, &b2);
                r[s] = P.pre * mb_int_one(x, y, sign, b1, b2, f);
            }
        }
        else
        {
            const double f[3] = {fd0, f0e[0], f0e[1]};
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                double b1, b2;
                neps_couplings(e, s, &b1, &b2);
                r[s] = P.pre * mb_int_two(w, wp, x, y, b1, b2, f);
            }
        }
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            em[s] += -r[s] * efb;
            ab[s] += r[s] * efa;
        }
    }
}

#undef BNSN_DI

} // namespace fp64
} // namespace bnsn
