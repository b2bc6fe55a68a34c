// Test/measurement infrastructure only: the reference's own headers compiled
// with BS_REAL = a counting real type, to measure how many floating-point
// operations the reference algorithm performs per call of each of its
// kernels and per grey point.  The product never links or loads it.
//
// The reference makes its real type a macro (include/bns_nurates.hpp:29-34,
// REAL_TYPE), so defining REAL_TYPE as `cdouble` below turns every
// arithmetic operation and every math-library call on the path into a
// counted one.  A cdouble holds a double and rounds exactly as a double does
// (no contraction across operators), so results equal the plain build's.
// Two generated header copies make that hold: constants.hpp:204-206 would
// otherwise give a type that is neither float nor double the float exp
// cut-off, and integration.hpp:39-40 assigns reals to double locals.
//
// Attribution: the calls named in COUNTED below are renamed while their
// headers are parsed and replaced by wrappers that count the call and route
// the operations inside it to that function's counters; everything else a
// grey point does (distribution weights, blocking and stimulated-absorption
// factors, the integrand assembly and the quadrature sums of
// m1_opacities.hpp) lands in "assembly".
//
// Built and driven by oracle/opcount.py.

#include <stdint.h>
#include <string.h>

#include <cmath>
#include <type_traits>
#include <unordered_set>

struct OpCounts
{
    uint64_t add, mul, div, sqrt, exp, log, pow, transc, cmp, minmax;
};

extern OpCounts* g_cur;

#define CD_COUNT(field)                                                                            \
    do                                                                                             \
    {                                                                                              \
        if (!std::is_constant_evaluated())                                                         \
            ++g_cur->field;                                                                        \
    } while (0)

namespace cdm {

// Converts to arithmetic types only explicitly, so mixed expressions resolve
// to the counted operators (which have exact overloads for (cdouble,
// arithmetic) and (arithmetic, cdouble)), never to built-in double arithmetic.
struct cdouble
{
    double v;
    constexpr cdouble() : v(0.) {}
    constexpr cdouble(double x) : v(x) {}
    template <class T, class = std::enable_if_t<std::is_arithmetic_v<T>>>
    explicit constexpr operator T() const
    {
        return (T)v;
    }
    constexpr cdouble operator-() const { return cdouble(-v); }
    constexpr cdouble operator+() const { return *this; }
    constexpr cdouble& operator++()
    {
        CD_COUNT(add);
        v += 1.;
        return *this;
    }
    constexpr cdouble& operator--()
    {
        CD_COUNT(add);
        v -= 1.;
        return *this;
    }
    constexpr cdouble operator++(int)
    {
        cdouble t = *this;
        ++*this;
        return t;
    }
    constexpr cdouble operator--(int)
    {
        cdouble t = *this;
        --*this;
        return t;
    }
    constexpr cdouble& operator+=(cdouble b)
    {
        CD_COUNT(add);
        v += b.v;
        return *this;
    }
    constexpr cdouble& operator-=(cdouble b)
    {
        CD_COUNT(add);
        v -= b.v;
        return *this;
    }
    constexpr cdouble& operator*=(cdouble b)
    {
        CD_COUNT(mul);
        v *= b.v;
        return *this;
    }
    constexpr cdouble& operator/=(cdouble b)
    {
        CD_COUNT(div);
        v /= b.v;
        return *this;
    }
};

template <class T>
using if_arith = std::enable_if_t<std::is_arithmetic_v<T>, int>;

#define CD_BIN(op, field)                                                                          \
    constexpr cdouble operator op(cdouble a, cdouble b)                                            \
    {                                                                                              \
        CD_COUNT(field);                                                                           \
        return cdouble(a.v op b.v);                                                                \
    }                                                                                              \
    template <class T, if_arith<T> = 0>                                                            \
    constexpr cdouble operator op(cdouble a, T b)                                                  \
    {                                                                                              \
        return a op cdouble((double)b);                                                            \
    }                                                                                              \
    template <class T, if_arith<T> = 0>                                                            \
    constexpr cdouble operator op(T a, cdouble b)                                                  \
    {                                                                                              \
        return cdouble((double)a) op b;                                                            \
    }
CD_BIN(+, add)
CD_BIN(-, add)
CD_BIN(*, mul)
CD_BIN(/, div)
#undef CD_BIN

#define CD_CMP(op)                                                                                 \
    constexpr bool operator op(cdouble a, cdouble b)                                               \
    {                                                                                              \
        CD_COUNT(cmp);                                                                             \
        return a.v op b.v;                                                                         \
    }                                                                                              \
    template <class T, if_arith<T> = 0>                                                            \
    constexpr bool operator op(cdouble a, T b)                                                     \
    {                                                                                              \
        return a op cdouble((double)b);                                                            \
    }                                                                                              \
    template <class T, if_arith<T> = 0>                                                            \
    constexpr bool operator op(T a, cdouble b)                                                     \
    {                                                                                              \
        return cdouble((double)a) op b;                                                            \
    }
CD_CMP(<)
CD_CMP(>)
CD_CMP(<=)
CD_CMP(>=)
CD_CMP(==)
CD_CMP(!=)
#undef CD_CMP

#define CD_F1(name, field)                                                                         \
    inline cdouble name(cdouble a)                                                                 \
    {                                                                                              \
        CD_COUNT(field);                                                                           \
        return cdouble(std::name(a.v));                                                            \
    }
#define CD_F2(name, field)                                                                         \
    inline cdouble name(cdouble a, cdouble b)                                                      \
    {                                                                                              \
        CD_COUNT(field);                                                                           \
        return cdouble(std::name(a.v, b.v));                                                       \
    }                                                                                              \
    template <class T, if_arith<T> = 0>                                                            \
    inline cdouble name(cdouble a, T b)                                                            \
    {                                                                                              \
        return cdm::name(a, cdouble((double)b));                                                   \
    }                                                                                              \
    template <class T, if_arith<T> = 0>                                                            \
    inline cdouble name(T a, cdouble b)                                                            \
    {                                                                                              \
        return cdm::name(cdouble((double)a), b);                                                   \
    }
#define CD_MATH                                                                                    \
    CD_F1(exp, exp)                                                                                \
    CD_F1(log, log)                                                                                \
    CD_F1(sqrt, sqrt)                                                                              \
    CD_F2(pow, pow)                                                                                \
    CD_F1(log2, transc)                                                                            \
    CD_F1(log10, transc)                                                                           \
    CD_F1(atan, transc)                                                                            \
    CD_F2(atan2, transc)                                                                           \
    CD_F2(hypot, transc)                                                                           \
    CD_F1(cbrt, transc)                                                                            \
    CD_F1(tanh, transc)                                                                            \
    CD_F1(sinh, transc)                                                                            \
    CD_F1(cosh, transc)                                                                            \
    CD_F1(sin, transc)                                                                             \
    CD_F1(cos, transc)                                                                             \
    CD_F1(fabs, minmax)                                                                            \
    CD_F1(floor, minmax)                                                                           \
    CD_F1(ceil, minmax)                                                                            \
    CD_F1(round, minmax)                                                                           \
    CD_F2(fmin, minmax)                                                                            \
    CD_F2(fmax, minmax)

// unqualified calls find these by argument-dependent lookup
CD_MATH

inline bool signbit(cdouble a) { return std::signbit(a.v); }
inline bool isnan(cdouble a) { return std::isnan(a.v); }
inline bool isinf(cdouble a) { return std::isinf(a.v); }
inline bool isfinite(cdouble a) { return std::isfinite(a.v); }

} // namespace cdm

using cdm::cdouble;

// the reference calls the math library as Kokkos::name (its no-Kokkos shim,
// bns_nurates.hpp:39-53, adds the std:: overloads next to these)
namespace Kokkos {
using cdm::exp, cdm::log, cdm::sqrt, cdm::pow, cdm::log2, cdm::log10, cdm::atan, cdm::atan2,
    cdm::hypot, cdm::cbrt, cdm::tanh, cdm::sinh, cdm::cosh, cdm::sin, cdm::cos, cdm::fabs,
    cdm::floor, cdm::ceil, cdm::round, cdm::fmin, cdm::fmax;
}

#define REAL_TYPE cdouble

// Rename the counted kernels while their headers are parsed.
#define TotalNuF TotalNuF_ref
#define CalculateDistrParamsFromM1 CalculateDistrParamsFromM1_ref
#define AbsOpacity AbsOpacity_ref
#define StimAbsOpacity StimAbsOpacity_ref
#define IsoScattTotal IsoScattTotal_ref
#define PairKernels PairKernels_ref
#define BremKernelsLegCoeff BremKernelsLegCoeff_ref
#define BremKernelsBRT06 BremKernelsBRT06_ref
#define BremKernelAbsGP19 BremKernelAbsGP19_ref
#define InelasticScattKernels InelasticScattKernels_ref
#include "bns_nurates.hpp"
// the generated copies (opcount.py), before any other header includes them
#include "constants.hpp"
#include "integration.hpp"
#include "distribution.hpp"
#include "formulas_beta_iso.hpp"
#include "kernel_brem_BRT06.hpp"
#include "kernel_brem_GP19.hpp"
#include "kernel_brem_HR98.hpp"
#include "kernel_nes.hpp"
#include "kernel_pair.hpp"
#undef TotalNuF
#undef CalculateDistrParamsFromM1
#undef AbsOpacity
#undef StimAbsOpacity
#undef IsoScattTotal
#undef PairKernels
#undef BremKernelsLegCoeff
#undef BremKernelsBRT06
#undef BremKernelAbsGP19
#undef InelasticScattKernels

enum Counted
{
    kAssembly,
    kDistr,
    kTotalNuF,
    kAbs,
    kStimAbs,
    kIso,
    kPair,
    kHR98,
    kBRT06,
    kGP19,
    kInel,
    kNumCounted
};

static OpCounts g_counts[kNumCounted];
static uint64_t g_calls[kNumCounted];
OpCounts* g_cur = &g_counts[kAssembly];

struct Scope
{
    OpCounts* prev;
    explicit Scope(Counted c) : prev(g_cur)
    {
        g_cur = &g_counts[c];
        ++g_calls[c];
    }
    ~Scope() { g_cur = prev; }
};

// distinct (energy, species) arguments of TotalNuF within the current point
static std::unordered_set<uint64_t> g_nuf_seen;
static uint64_t g_nuf_distinct;

inline BS_REAL TotalNuF(const BS_REAL omega, const NuDistributionParams* d, const int nuid)
{
    uint64_t bits;
    memcpy(&bits, &omega.v, sizeof(bits));
    if (g_nuf_seen.insert(bits * 4u + (uint64_t)nuid).second)
        ++g_nuf_distinct;
    Scope s(kTotalNuF);
    return TotalNuF_ref(omega, d, nuid);
}
inline NuDistributionParams CalculateDistrParamsFromM1(const M1Quantities* m,
                                                       const MyEOSParams* e)
{
    Scope s(kDistr);
    return CalculateDistrParamsFromM1_ref(m, e);
}
inline MyOpacity AbsOpacity(const BS_REAL omega, OpacityParams* p, MyEOSParams* e)
{
    Scope s(kAbs);
    return AbsOpacity_ref(omega, p, e);
}
inline MyOpacity StimAbsOpacity(const BS_REAL omega, OpacityParams* p, MyEOSParams* e)
{
    Scope s(kStimAbs);
    return StimAbsOpacity_ref(omega, p, e);
}
inline BS_REAL IsoScattTotal(const BS_REAL omega, OpacityParams* p, MyEOSParams* e)
{
    Scope s(kIso);
    return IsoScattTotal_ref(omega, p, e);
}
inline MyKernelOutput PairKernels(const MyEOSParams* e, const PairKernelParams* k)
{
    Scope s(kPair);
    return PairKernels_ref(e, k);
}
inline void PairKernels(const MyEOSParams* e, const PairKernelParams* k, MyKernelOutput* a,
                        MyKernelOutput* b)
{
    Scope s(kPair);
    PairKernels_ref(e, k, a, b);
}
inline MyKernelOutput BremKernelsLegCoeff(BremKernelParams* k, MyEOSParams* e)
{
    Scope s(kHR98);
    return BremKernelsLegCoeff_ref(k, e);
}
inline MyKernelOutput BremKernelsBRT06(BremKernelParams* k, MyEOSParams* e)
{
    Scope s(kBRT06);
    return BremKernelsBRT06_ref(k, e);
}
inline MyKernelOutput BremKernelAbsGP19(const BremKernelParams* k, const MyEOSParams* e)
{
    Scope s(kGP19);
    return BremKernelAbsGP19_ref(k, e);
}
inline MyKernelOutput InelasticScattKernels(InelasticScattKernelParams* k, MyEOSParams* e)
{
    Scope s(kInel);
    return InelasticScattKernels_ref(k, e);
}

#include "m1_opacities.hpp"

extern "C" {

int opcount_n_counted(void) { return kNumCounted; }

// Per grey point (ComputeM1Opacities with stimulated absorption, the
// distribution parameters reconstructed from the M1 moments first) over
// npts points: calls[kNumCounted] and counts[kNumCounted][10] summed over the
// points (fields of OpCounts in order), *nuf_distinct the number of distinct
// (energy, species) arguments of TotalNuF summed over the points, and
// out[20][npts] the outputs.
int opcount_m1(int64_t npts, const double* eos, const double* m1, const int* flags,
               const int* pars, int nx, const double* x, const double* w, uint64_t* calls,
               uint64_t* counts, uint64_t* nuf_distinct, double* out)
{
    if (2 * nx > BS_N_MAX)
        return 2;
    memset(g_counts, 0, sizeof(g_counts));
    memset(g_calls, 0, sizeof(g_calls));
    g_nuf_distinct = 0;
    MyQuadrature q;
    memset(&q, 0, sizeof(q));
    q.type = kGauleg;
    q.dim  = 1;
    q.nx   = nx;
    q.ny   = 1;
    q.nz   = 1;
    q.x1   = 0.;
    q.x2   = 1.;
    q.y1 = q.y2 = q.z1 = q.z2 = -42.;
    for (int i = 0; i < nx; ++i)
    {
        q.points[i] = x[i];
        q.w[i]      = w[i];
    }
    for (int64_t p = 0; p < npts; ++p)
    {
        GreyOpacityParams g;
        memset(&g, 0, sizeof(g));
        g.opacity_flags.use_abs_em          = flags[0];
        g.opacity_flags.use_pair            = flags[1];
        g.opacity_flags.use_brem            = flags[2];
        g.opacity_flags.use_inelastic_scatt = flags[3];
        g.opacity_flags.use_iso             = flags[4];
        g.opacity_pars.use_dU               = pars[0] != 0;
        g.opacity_pars.use_dm_eff           = pars[1] != 0;
        g.opacity_pars.use_WM_ab            = pars[2] != 0;
        g.opacity_pars.use_WM_sc            = pars[3] != 0;
        g.opacity_pars.use_decay            = pars[4] != 0;
        g.opacity_pars.brem_implementation  = (BremImpl)pars[5];
        g.opacity_pars.use_NN_medium_corr   = pars[6] != 0;
        g.opacity_pars.neglect_blocking     = pars[7] != 0;
        BS_REAL* e[11] = {&g.eos_pars.nb,   &g.eos_pars.temp,  &g.eos_pars.ye, &g.eos_pars.yp,
                          &g.eos_pars.yn,   &g.eos_pars.mu_p,  &g.eos_pars.mu_n,
                          &g.eos_pars.mu_e, &g.eos_pars.mu_mu, &g.eos_pars.dU,
                          &g.eos_pars.dm_eff};
        for (int f = 0; f < 11; ++f)
            *e[f] = eos[f * npts + p];
        for (int s = 0; s < 4; ++s)
        {
            g.m1_pars.n[s]   = m1[(0 + s) * npts + p];
            g.m1_pars.J[s]   = m1[(4 + s) * npts + p];
            g.m1_pars.chi[s] = m1[(8 + s) * npts + p];
        }
        g_nuf_seen.clear();
        g.distr_pars   = CalculateDistrParamsFromM1(&g.m1_pars, &g.eos_pars);
        M1Opacities o  = ComputeM1Opacities(&q, &q, &g);
        for (int s = 0; s < 4; ++s)
        {
            out[(0 + s) * npts + p]  = o.eta_0[s].v;
            out[(4 + s) * npts + p]  = o.kappa_0_a[s].v;
            out[(8 + s) * npts + p]  = o.eta[s].v;
            out[(12 + s) * npts + p] = o.kappa_a[s].v;
            out[(16 + s) * npts + p] = o.kappa_s[s].v;
        }
    }
    *nuf_distinct = g_nuf_distinct;
    for (int c = 0; c < kNumCounted; ++c)
    {
        calls[c] = g_calls[c];
        memcpy(counts + 10 * c, &g_counts[c], sizeof(OpCounts));
    }
    return 0;
}

} // extern "C"
