// Double-float ("df") arithmetic on the FP32 pipes for the mixed-precision path.
//
// A df value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits (unit roundoff ~3.6e-15) over the FP32 exponent
// range.  GB300 runs FP32 at 64x its FP64 rate, so a df operation (6-20 FP32
// instructions) is several times cheaper than the FP64 one.  The
// error-free transformations are Knuth's TwoSum, Dekker's FastTwoSum and the
// FMA-based TwoProd; division is Dekker's long division with one correction.
// Nothing here relies on fast-math: the library is compiled without it, so
// the compiler keeps every addition below in IEEE order (FMA contraction only
// merges a product with an addition, and the sums below contain no products).
//
// df_exp uses Cody-Waite range reduction with a three-part ln 2, a Taylor
// polynomial for e^r - 1 on |r| <= ln2/32, and four exact-ish squarings of
// (1 + q) carried as q -> q (2 + q).
//
// fdi_df<KLO, KHI> evaluates the same Fukushima rational forms as
// fdi_orders (bnsn_fp64.cuh) with df coefficients.
#pragma once

#include <math.h>

#include "bnsn_fp64.cuh"

namespace bnsn {
namespace dfm {
namespace { // internal linkage: every translation unit has its own copy

#define BNSN_DI __device__ __forceinline__

struct df
{
    float hi, lo;
};

// Compile-time split of a double constant into a df.
struct dfc
{
    float hi, lo;
    __host__ __device__ constexpr dfc() : hi(0.f), lo(0.f) {}
    __host__ __device__ constexpr dfc(double v)
        : hi((float)v), lo((float)(v - (double)(float)v))
    {
    }
};

BNSN_DI df mk(const dfc& c) { return {c.hi, c.lo}; }
BNSN_DI df mk(float v) { return {v, 0.f}; }

BNSN_DI df from_double(double d)
{
    const float h = __double2float_rn(d);
    return {h, __double2float_rn(d - (double)h)};
}

BNSN_DI double to_double(df a) { return (double)a.hi + (double)a.lo; }

BNSN_DI df two_sum(float a, float b)
{
    const float s  = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

BNSN_DI df fast_two_sum(float a, float b)
{
    const float s = a + b;
    return {s, b - (s - a)};
}

BNSN_DI df add(df a, df b)
{
    df s       = two_sum(a.hi, b.hi);
    const df t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}

BNSN_DI df add(df a, float b)
{
    df s = two_sum(a.hi, b);
    s.lo += a.lo;
    return fast_two_sum(s.hi, s.lo);
}

BNSN_DI df neg(df a) { return {-a.hi, -a.lo}; }
BNSN_DI df neg_df(df a) { return {-a.hi, -a.lo}; }
BNSN_DI df sub(df a, df b) { return add(a, neg(b)); }

BNSN_DI df mul(df a, df b)
{
    const float p = a.hi * b.hi;
    float e       = fmaf(a.hi, b.hi, -p);
    e             = fmaf(a.hi, b.lo, e);
    e             = fmaf(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

BNSN_DI df mul(df a, float b)
{
    const float p = a.hi * b;
    float e       = fmaf(a.hi, b, -p);
    e             = fmaf(a.lo, b, e);
    return fast_two_sum(p, e);
}

// Exact product of two floats.
BNSN_DI df two_prod(float a, float b)
{
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}

BNSN_DI df div(df a, df b)
{
    const float rb = __frcp_rn(b.hi);
    const float q1 = a.hi * rb;
    const df r     = sub(a, mul(b, q1));
    const float q2 = r.hi * rb;
    const df r2    = sub(r, mul(b, q2));
    const float q3 = r2.hi * rb;
    const df q     = fast_two_sum(q1, q2);
    return add(q, q3);
}

// c + t p for the Horner steps of the rational forms: the product error and
// the addition error are gathered in one correction term (Dekker's addition),
// 14 FP32 instructions instead of a separate product and accurate sum; the
// polynomials on [0, 1] have no large internal cancellation.
BNSN_DI df fma_df(df t, df p, df c)
{
    const float ph = t.hi * p.hi;
    float pe       = fmaf(t.hi, p.hi, -ph);
    pe             = fmaf(t.hi, p.lo, pe);
    pe             = fmaf(t.lo, p.hi, pe);
    const float s  = ph + c.hi;
    const float bb = s - ph;
    float e        = (ph - (s - bb)) + (c.hi - bb);
    e += pe + c.lo;
    return fast_two_sum(s, e);
}

// a * 2^k for integer k (exact unless the result leaves the normal range).
BNSN_DI df ldexp_df(df a, int k) { return {ldexpf(a.hi, k), ldexpf(a.lo, k)}; }

// Horner evaluation with df coefficients: c[0] + t c[1] + ... + t^{N-1} c[N-1].
template <int N>
BNSN_DI df horner(const dfc (&c)[N], df t)
{
    df p = mk(c[N - 1]);
#pragma unroll
    for (int i = N - 2; i >= 0; --i)
        p = add(mk(c[i]), mul(t, p));
    return p;
}

// e^x.  Results below the FP32 normal range lose precision (and are 0 for
// x < -104); callers only use them as negligible contributions.
BNSN_DI df exp_df(df x)
{
    if (x.hi < -104.f)
        return {0.f, 0.f};
    // k = round(x / ln2); r = x - k ln2 with ln2 = L1 + L2 + L3, L1 exact in
    // 16 bits so that k L1 is exact for |k| < 256.
    constexpr float kInvLn2 = 1.44269504088896341f;
    constexpr float L1      = 0.693145751953125f;
    constexpr dfc L23(0.693147180559945309417232121458 - 0.693145751953125);
    const float k = rintf(x.hi * kInvLn2);
    df r          = two_sum(x.hi - k * L1, x.lo); // x.hi - k L1 is exact (Sterbenz)
    r             = sub(r, two_prod(k, L23.hi));
    r             = add(r, -k * L23.lo);
    // e^r = (e^{r/16})^16; q = e^{r/16} - 1 by Taylor to degree 7 (|r/16| <= 0.0217,
    // truncation < 1e-17)
    const df s = {r.hi * 0.0625f, r.lo * 0.0625f};
    constexpr dfc c7(1. / 5040.), c6(1. / 720.), c5(1. / 120.), c4(1. / 24.), c3(1. / 6.);
    df q = mk(c7);
    q    = add(mk(c6), mul(s, q));
    q    = add(mk(c5), mul(s, q));
    q    = add(mk(c4), mul(s, q));
    q    = add(mk(c3), mul(s, q));
    q    = add(mk(0.5f), mul(s, q));
    q    = add(mk(1.f), mul(s, q));
    q    = mul(s, q);
#pragma unroll
    for (int i = 0; i < 4; ++i)
        q = mul(q, add(q, 2.f)); // (1 + q)^2 - 1
    const df e = add(q, 1.f);
    return ldexp_df(e, (int)k);
}

// ---------------------------------------------------------------------------
// Fermi-Dirac integrals F_K, K = KLO..KHI, in df (the forms of fdi_orders).
// ---------------------------------------------------------------------------
__device__ constexpr dfc kAN0[5] = {22696.2126132366633, 5222.0667923565138, 357.623326425354522, 6.9167792879948140, 0.00200096064827815813};
__device__ constexpr dfc kAD0[5] = {45392.4252264733267, 14539.5980679273792, 1611.36476693109675, 71.072178562726798, 1.0};
__device__ constexpr dfc kBN0[9] = {159.601717762460980, 23.7193942338278703, 0.377783268730614356, 10.5181677709577503, 3.78181326142271599, -0.441998676614933572, -0.450072959113928254, -0.0734798777056723512, 0.000915454570009894267};
__device__ constexpr dfc kBD0[8] = {284.26032127745967, 315.2592651624449, 310.2713981221035, 206.21640678892182, 96.77898293084927, 35.456591489081173, 8.1762315442738975, 1.0};
__device__ constexpr dfc kAN1[5] = {22189.1070807945062, 4915.92700908746777, 322.901386168881348, 5.9897442965804548, 0.00397641173774375092};
__device__ constexpr dfc kAD1[5] = {88756.428323178025, 25002.3197546553836, 2389.06277237306633, 88.376214553692756, 1.0};
__device__ constexpr dfc kBN1[9] = {145.488167182330098, 251.392824471576922, 56.6537141912783024, 17.9918985363509694, 20.1369115558099802, 7.09659390228556164, 0.199701180197912643, -0.403173132925886253, -0.0792966701498222697};
__device__ constexpr dfc kBD1[9] = {606.0757707716040, 374.1806357435014, 252.1367051536344, 27.2746245830016, -61.57766112137513, -53.72117554363975, -25.678454878692950, -7.1995819520154718, -1.0};
__device__ constexpr dfc kAN2[4] = {1914.06748184935743, 273.085756700981399, 8.5861610217850095, 0.0161890243763741414};
__device__ constexpr dfc kAD2[4] = {7656.2699273974454, 1399.35442210906621, 72.929152915475392, 1.0};
__device__ constexpr dfc kBN2[9] = {2711.49678259128843, 1299.85460914884154, 222.606134197895041, 172.881855215582924, 112.951038040682055, 24.0376482128898634, -2.68393549333878715, -2.14077421411719935, -0.326188299771397236};
__device__ constexpr dfc kBD2[9] = {2517.1726659917047, 3038.7689794575778, 2541.7823512372631, 1428.0589853413436, 531.62378035996132, 122.54595216479181, 8.395768655115050, -3.9142702096919080, -1.0};
__device__ constexpr dfc kAN3[4] = {5121.6401850302408, 664.28706260743472, 19.0856927562699544, 0.0410982603688952131};
__device__ constexpr dfc kAD3[4] = {13657.7071600806539, 2136.54222460571183, 92.376788603062645, 1.0};
__device__ constexpr dfc kBN3[8] = {7881.24597452900838, 4323.07526636309661, 1260.13125873282465, 653.359212389160499, 354.630774329461644, 113.373708671587772, 19.9559488532742796, 1.59407954898394322};
__device__ constexpr dfc kBD3[8] = {2570.7250703533430, 2972.7443644211129, 2393.9995533270879, 1259.0724833462608, 459.86413596901097, 112.60906419590854, 16.468882811659000, 1.0};
__device__ constexpr dfc kAN4[4] = {18247.2542465629199, 2120.56302902849207, 54.659507299984584, 0.121876197098273914};
__device__ constexpr dfc kAD4[4] = {24329.6723287505678, 3261.01909656925521, 117.071576489684022, 1.0};
__device__ constexpr dfc kBN4[8] = {33093.9102025608137, 19031.4783357798975, 5431.08357152245897, 2393.94262931609398, 1268.40017257978070, 418.662172475927160, 77.4108960876508190, 6.67374311450268357};
__device__ constexpr dfc kBD4[8] = {2645.4885670047153, 3236.2237702166948, 2500.5977847175497, 1278.0109577275445, 448.99020896813485, 105.86020755838874, 15.216887271751039, 1.0};
__device__ constexpr dfc kAN5[4] = {81190.938912603315, 8368.4990332049831, 190.753830813273698, 0.413800735538960261};
__device__ constexpr dfc kAD5[4] = {43301.8340867217726, 4977.68099709243407, 148.484432990224213, 1.0};
__device__ constexpr dfc kBN5[8] = {159651.547840031111, 96307.2005742063042, 26923.5693307648389, 9274.54751848368696, 4445.76333033698006, 1461.45267097859337, 272.164427980501432, 23.6526046298891619};
__device__ constexpr dfc kBD5[8] = {2522.7839609396783, 3244.5527999477567, 2403.0532924519756, 1176.7202478443275, 397.7596246691212, 91.84661231161838, 13.491911254479298, 1.0};

template <int K> struct Fdi;

#define BNSN_DF_FDI(K, A0)                                                                         \
    template <> struct Fdi<K>                                                                      \
    {                                                                                              \
        static constexpr float a0 = A0;                                                            \
        BNSN_DI static df low(df ex, df t)                                                         \
        {                                                                                          \
            return mul(ex, sub(mk(a0), mul(ex, div(horner(kAN##K, t), horner(kAD##K, t)))));       \
        }                                                                                          \
        BNSN_DI static df mid(df s, df t) { return div(horner(kBN##K, t), horner(kBD##K, s)); }   \
    };
BNSN_DF_FDI(0, 1.f)
BNSN_DF_FDI(1, 1.f)
BNSN_DF_FDI(2, 2.f)
BNSN_DF_FDI(3, 6.f)
BNSN_DF_FDI(4, 24.f)
BNSN_DF_FDI(5, 120.f)
#undef BNSN_DF_FDI

// Reflection for y > 0 (the polynomials of FdiCoef<K>::reflect).
template <int K>
BNSN_DI df reflect(df f, df y)
{
    constexpr dfc r1a(1.64493406684822644);
    constexpr dfc r2a(3.28986813369645287), r2b(0.333333333333333333);
    constexpr dfc r3a(11.3643939539669510), r3b(4.93480220054467931);
    constexpr dfc r4a(45.4575758158678040), r4b(6.57973626739290575), r4c(0.2);
    constexpr dfc r5a(236.532261911384425), r5b(113.643939539669510), r5c(8.22467033424113218),
        r5d(0.166666666666666667);
    if (K == 0)
        return add(f, y);
    const df y2 = mul(y, y);
    if (K == 1)
        return add(neg(f), add(mk(r1a), mul(y2, 0.5f)));
    if (K == 2)
        return add(f, mul(y, add(mk(r2a), mul(y2, mk(r2b)))));
    if (K == 3)
        return add(neg(f), add(mk(r3a), mul(y2, add(mk(r3b), mul(y2, 0.25f)))));
    if (K == 4)
        return add(f, mul(y, add(mk(r4a), mul(y2, add(mk(r4b), mul(y2, mk(r4c)))))));
    return add(neg(f),
               add(mk(r5a), mul(y2, add(mk(r5b), mul(y2, add(mk(r5c), mul(y2, mk(r5d))))))));
}

// F_K(y), K = KLO..KHI, into out[K - KLO]; regimes as fdi_orders (x = -|y|).
template <int KLO, int KHI>
BNSN_DI void fdi_df(df y, df* out)
{
    const df x = (y.hi > 0.f) ? neg(y) : y;
    if (!(x.hi <= 0.f)) // NaN argument: 0, as fdi_orders
    {
#pragma unroll
        for (int kk = 0; kk <= KHI - KLO; ++kk)
            out[kk] = {0.f, 0.f};
        return;
    }
    if (x.hi < -2.f)
    {
        constexpr dfc e2(7.38905609893065023);
        const df ex = exp_df(x);
        const df t  = mul(ex, mk(e2));
#define BNSN_DF_LOW(K)                                                                             \
    if (KLO <= K && K <= KHI)                                                                      \
        out[K - KLO] = Fdi<K>::low(ex, t);
        BNSN_DF_LOW(0) BNSN_DF_LOW(1) BNSN_DF_LOW(2) BNSN_DF_LOW(3) BNSN_DF_LOW(4) BNSN_DF_LOW(5)
#undef BNSN_DF_LOW
    }
    else
    {
        const df s = {-0.5f * x.hi, -0.5f * x.lo};
        const df t = add(neg(s), 1.f);
#define BNSN_DF_MID(K)                                                                             \
    if (KLO <= K && K <= KHI)                                                                      \
        out[K - KLO] = Fdi<K>::mid(s, t);
        BNSN_DF_MID(0) BNSN_DF_MID(1) BNSN_DF_MID(2) BNSN_DF_MID(3) BNSN_DF_MID(4) BNSN_DF_MID(5)
#undef BNSN_DF_MID
    }
    if (y.hi > 0.f)
    {
#define BNSN_DF_REF(K)                                                                             \
    if (KLO <= K && K <= KHI)                                                                      \
        out[K - KLO] = reflect<K>(out[K - KLO], y);
        BNSN_DF_REF(0) BNSN_DF_REF(1) BNSN_DF_REF(2) BNSN_DF_REF(3) BNSN_DF_REF(4) BNSN_DF_REF(5)
#undef BNSN_DF_REF
    }
}

// ---------------------------------------------------------------------------
// Compact table-driven F_k, k = 1..5, for the NES item loop.  All five orders
// share one Horner loop over __constant__ coefficients (padded to 9 terms
// with zeros), so the code stays small enough for the instruction cache; the
// numerator and denominator chains run interleaved.
// ---------------------------------------------------------------------------
struct FdiTab
{
    dfc num[2][5][9]; // [0: x < -2 (in t = e^{x+2}), 1: -2 <= x <= 0 (in 1 - s)][k-1]
    dfc den[2][5][9]; // [regime][k-1]; mid-regime denominators in s = -x/2
};

#define BNSN_Z 0.0
__constant__ FdiTab kFdiTab = {
    {{{22189.1070807945062, 4915.92700908746777, 322.901386168881348, 5.9897442965804548, 0.00397641173774375092, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z},
      {1914.06748184935743, 273.085756700981399, 8.5861610217850095, 0.0161890243763741414, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z},
      {5121.6401850302408, 664.28706260743472, 19.0856927562699544, 0.0410982603688952131, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z},
      {18247.2542465629199, 2120.56302902849207, 54.659507299984584, 0.121876197098273914, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z},
      {81190.938912603315, 8368.4990332049831, 190.753830813273698, 0.413800735538960261, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z}},
     {{145.488167182330098, 251.392824471576922, 56.6537141912783024, 17.9918985363509694, 20.1369115558099802, 7.09659390228556164, 0.199701180197912643, -0.403173132925886253, -0.0792966701498222697},
      {2711.49678259128843, 1299.85460914884154, 222.606134197895041, 172.881855215582924, 112.951038040682055, 24.0376482128898634, -2.68393549333878715, -2.14077421411719935, -0.326188299771397236},
      {7881.24597452900838, 4323.07526636309661, 1260.13125873282465, 653.359212389160499, 354.630774329461644, 113.373708671587772, 19.9559488532742796, 1.59407954898394322, BNSN_Z},
      {33093.9102025608137, 19031.4783357798975, 5431.08357152245897, 2393.94262931609398, 1268.40017257978070, 418.662172475927160, 77.4108960876508190, 6.67374311450268357, BNSN_Z},
      {159651.547840031111, 96307.2005742063042, 26923.5693307648389, 9274.54751848368696, 4445.76333033698006, 1461.45267097859337, 272.164427980501432, 23.6526046298891619, BNSN_Z}}},
    {{{88756.428323178025, 25002.3197546553836, 2389.06277237306633, 88.376214553692756, 1.0, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z},
      {7656.2699273974454, 1399.35442210906621, 72.929152915475392, 1.0, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z},
      {13657.7071600806539, 2136.54222460571183, 92.376788603062645, 1.0, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z},
      {24329.6723287505678, 3261.01909656925521, 117.071576489684022, 1.0, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z},
      {43301.8340867217726, 4977.68099709243407, 148.484432990224213, 1.0, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z, BNSN_Z}},
     {{606.0757707716040, 374.1806357435014, 252.1367051536344, 27.2746245830016, -61.57766112137513, -53.72117554363975, -25.678454878692950, -7.1995819520154718, -1.0},
      {2517.1726659917047, 3038.7689794575778, 2541.7823512372631, 1428.0589853413436, 531.62378035996132, 122.54595216479181, 8.395768655115050, -3.9142702096919080, -1.0},
      {2570.7250703533430, 2972.7443644211129, 2393.9995533270879, 1259.0724833462608, 459.86413596901097, 112.60906419590854, 16.468882811659000, 1.0, BNSN_Z},
      {2645.4885670047153, 3236.2237702166948, 2500.5977847175497, 1278.0109577275445, 448.99020896813485, 105.86020755838874, 15.216887271751039, 1.0, BNSN_Z},
      {2522.7839609396783, 3244.5527999477567, 2403.0532924519756, 1176.7202478443275, 397.7596246691212, 91.84661231161838, 13.491911254479298, 1.0, BNSN_Z}}}};
#undef BNSN_Z

// r[k-1] = F_k(-|y|), k = kmin..5 (the unreflected part of fdi_orders; NaN ->
// 0); entries below kmin are not written.  `tab` is kFdiTab or a copy of it in
// shared memory (lanes in different regimes read different coefficients: from
// shared memory that costs at most a bank conflict, from the constant cache a
// serialised access per distinct address).
__device__ __noinline__ void fdi_raw15(df y, df* r, int kmin = 1, const FdiTab* tab = nullptr)
{
    if (!tab)
        tab = &kFdiTab;
    const df x = (y.hi > 0.f) ? neg(y) : y;
    if (!(x.hi <= 0.f))
    {
#pragma unroll
        for (int k = 0; k < 5; ++k)
            r[k] = {0.f, 0.f};
        return;
    }
    const int reg = (x.hi < -2.f) ? 0 : 1;
    df ex = {0.f, 0.f}, tn, td;
    if (reg == 0)
    {
        constexpr dfc e2(7.38905609893065023);
        ex = exp_df(x);
        tn = mul(ex, mk(e2));
        td = tn;
    }
    else
    {
        td = {-0.5f * x.hi, -0.5f * x.lo};
        tn = add(neg(td), 1.f);
    }
    // terms of the forms: x < -2: 5 (k = 1), 4 (k = 2..5); else 9, 9, 8, 8, 8
#pragma unroll 1
    for (int k = kmin - 1; k < 5; ++k)
    {
        const dfc* cn = tab->num[reg][k];
        const dfc* cd = tab->den[reg][k];
        const int top = reg == 0 ? (k == 0 ? 4 : 3) : (k < 2 ? 8 : 7);
        df pn = mk(cn[top]), pd = mk(cd[top]);
#pragma unroll 1
        for (int i = top - 1; i >= 0; --i)
        {
            pn = fma_df(tn, pn, mk(cn[i]));
            pd = fma_df(td, pd, mk(cd[i]));
        }
        const df q = div(pn, pd);
        if (reg == 0)
        {
            const float a0 = k == 0 ? 1.f : k == 1 ? 2.f : k == 2 ? 6.f : k == 3 ? 24.f : 120.f;
            r[k] = mul(ex, sub(mk(a0), mul(ex, q)));
        }
        else
            r[k] = q;
    }
}

// Full F_k(y), k = 1..5, from the unreflected values (reflection for y > 0).
BNSN_DI void fdi_full15(const df* r, df y, df* f)
{
    if (y.hi > 0.f)
    {
        f[0] = reflect<1>(r[0], y);
        f[1] = reflect<2>(r[1], y);
        f[2] = reflect<3>(r[2], y);
        f[3] = reflect<4>(r[3], y);
        f[4] = reflect<5>(r[4], y);
    }
    else
    {
#pragma unroll
        for (int k = 0; k < 5; ++k)
            f[k] = r[k];
    }
}

// Divided differences (P_k(b) - P_k(a)) / (b - a) of the reflection
// polynomials, k = 1..5; every term is positive for a, b > 0.
BNSN_DI void fdi_dd15(df a, df b, df* d)
{
    constexpr dfc c2a(3.28986813369645287), c3b(4.93480220054467931), c4a(45.4575758158678040),
        c4b(6.57973626739290575), c5b(113.643939539669510), c5c(8.22467033424113218),
        third(1. / 3.), fifth(0.2), sixth(1. / 6.);
    const df s = add(a, b), a2 = mul(a, a), b2 = mul(b, b), ab = mul(a, b);
    const df q2   = add(add(a2, ab), b2); // a^2 + ab + b^2
    const df p2   = add(a2, b2);          // a^2 + b^2
    const df a2b2 = mul(a2, b2);
    const df a4b4 = add(mul(a2, a2), mul(b2, b2));
    const df q4   = add(add(a4b4, mul(ab, p2)), a2b2); // (b^5 - a^5) / (b - a)
    d[0] = mul(s, 0.5f);
    d[1] = add(mk(c2a), mul(q2, mk(third)));
    d[2] = mul(s, add(mk(c3b), mul(p2, 0.25f)));
    d[3] = add(mk(c4a), add(mul(mk(c4b), q2), mul(q4, mk(fifth))));
    d[4] = mul(s, add(mk(c5b), add(mul(mk(c5c), p2), mul(add(a4b4, a2b2), mk(sixth)))));
}

// F_k(b) - F_k(a), k = 1..5, from the unreflected values at a and b and an
// accurate delta = b - a.  With a, b > 0 the reflection polynomials are
// differenced analytically (delta times their divided difference) instead
// of subtracting two values of size ~|a|^{k+1}.
BNSN_DI void fdi_diff15(const df* ra, const df* rb, df a, df b, df delta, df* dw)
{
    if (a.hi > 0.f && b.hi > 0.f)
    {
        df d[5];
        fdi_dd15(a, b, d);
        // reflect<K>: F = -F(-y) + P for odd K, F(-y) + P for even K
        dw[0] = add(sub(ra[0], rb[0]), mul(delta, d[0]));
        dw[1] = add(sub(rb[1], ra[1]), mul(delta, d[1]));
        dw[2] = add(sub(ra[2], rb[2]), mul(delta, d[2]));
        dw[3] = add(sub(rb[3], ra[3]), mul(delta, d[3]));
        dw[4] = add(sub(ra[4], rb[4]), mul(delta, d[4]));
    }
    else
    {
        df fa[5], fb[5];
        fdi_full15(ra, a, fa);
        fdi_full15(rb, b, fb);
#pragma unroll
        for (int k = 0; k < 5; ++k)
            dw[k] = sub(fb[k], fa[k]);
    }
}

#undef BNSN_DI

} // namespace
} // namespace dfm
} // namespace bnsn
