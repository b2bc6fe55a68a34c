// Mixed-precision device helpers shared by the grey and spectral kernels.
#pragma once

#include "bnsn_df.cuh"
#include "bnsn_fp64.cuh"

namespace bnsn {
namespace {

using namespace fp64;

// Bracket of lw on a log-w axis of d3 entries (binary search, first interval).
template <class R>
__device__ __forceinline__ int bracket_sorted(R lw, const R* ax, int d3, R* t)
{
    int lo = 0, hi = d3 - 2;
    while (lo < hi)
    {
        const int mid = (lo + hi) >> 1;
        if (lw <= ax[mid + 1])
            hi = mid;
        else
            lo = mid + 1;
    }
    *t = (lw - ax[lo]) / (ax[lo + 1] - ax[lo]);
    return lo;
}

// Interval of w on the GP19 w axis and its interpolation weight in FP32, for
// an FP64 w already clipped to the axis.  The interval comes from an FP32
// search of log w; the weight from log1p of the offset to the interval's first
// node, (w - w_l) / w_l, so that it keeps the relative precision of that
// offset: logf(w) itself is off by up to an ulp of log w (~5e-7 at w ~ 400
// MeV), which moved the weight by 1e-6 and the brem cell by up to 1.4e-6.
// wax, iw: the axis and 1 / axis (FP64); lwf: log axis (FP32); idl:
// 1 / (log w_{l+1} - log w_l) (FP32).
__device__ __forceinline__ int gp19_bracket32(double w, const float* lwf, const double* wax,
                                              const double* iw, const float* idl, int d3,
                                              float* tw)
{
    float t;
    const int l = bracket_sorted<float>(logf((float)w), lwf, d3, &t);
    *tw         = log1pf((float)((w - wax[l]) * iw[l])) * idl[l];
    return l;
}

// Per-point data of the mixed item loop.
struct NepsMixed
{
    dfm::df reta[2][5]; // unreflected F_1..F_5 at eta for e- (0) and e+ (1)
    dfm::df eta[2];
    double invTt[4], etat[4], lbf[4], invTf[4], cf[4]; // exponent arguments in FP64
};

// NEPSExpFunc (functions.hpp:4401-4413) in FP32 for the FP64 argument d;
// e^{-|d|} takes the FP32 exponential of the rounded argument times the
// first-order correction for its remainder, expm1 keeps 1 - e^{-|d|}
// accurate for small |d|.
__device__ __forceinline__ float neps_exp_f32(double d, bool neg)
{
    const double ad = fabs(d);
    const float a   = (float)ad;
    const float alo = (float)(ad - (double)a); // e^{-alo} = 1 - alo to FP32 precision
    const float ea  = expf(-a);
    const float e   = ea * (1.f - alo);
    const float dn  = -expm1f(-a) + ea * alo + (d == 0. ? 1.f : 0.f);
    return (neg ? 1.f : -e) / dn;
}

// Taylor branches of neps_pair (kernel_nes.hpp:82-132) for w or w' near 0,
// in FP64: dimensionless r1 = R(w, w'), r2 = R(w', w) of lepton e.  Rare in the
// item loop, so kept out of line to keep the loop's code small.
__device__ __noinline__ void neps_taylor(const NepsPoint& P, int e, double w, double wp,
                                         double x, double y, int sign1, int sign2, double* r1,
                                         double* r2)
{
    const double eta  = e ? P.eta1 : P.eta0;
    const double* f0e = e ? P.fe1 : P.fe0;
    const double fd0  = e ? P.fd01 : P.fd00;
    if (x > eta * 1e-3)
    {
        double fx[3];
        fdi_orders<0, 2>(eta - x, fx);
        const double f[5] = {fx[2] - f0e[2], fx[1], f0e[1],
                             fx[0] + y * fermi_distr(0., 1., eta - x) / 6., f0e[0] - y * fd0 / 6.};
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            double b1, b2;
            neps_couplings(e, s, &b1, &b2);
            r1[s] = mb_int_one(x, y, sign1, b1, b2, f);
            r2[s] = mb_int_one(x, y, sign2, b1, b2, f);
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
            r1[s] = mb_int_two(w, wp, x, y, b1, b2, f);
            r2[s] = mb_int_two(wp, w, x, y, b1, b2, f);
        }
    }
}

} // namespace
} // namespace bnsn

namespace bnsn {
namespace {

// Spectral NES/NPS kernel of neps_one (one direction) before the detailed-
// balance factors: R[s] = sum over e-, e+ of R(w, w') for species s, with the
// Fermi integrals and brackets in df, dimensionless (the caller applies the
// NEPS prefactor, NEPSExpFunc and the occupations).  rw[e] are the
// unreflected F_1..F_5 at aw[e] = eta_e - nu/T, staged per energy.  DF: R in
// df (the accurate pass), else rounded to FP32 per lepton.
// W, WP are w, wp in df.
template <bool DF>
__device__ __forceinline__ void neps_r_core(const NepsPoint& P, const NepsMixed& Q,
                                            const dfm::FdiTab* ftab, double w, double wp,
                                            dfm::df W, dfm::df WP, const dfm::df (*rw)[5],
                                            const dfm::df* aw, dfm::df* Rd, float* Rf)
{
    using namespace dfm;
    const double x = (w > wp) ? w : wp;
    const double y = (w < wp) ? w : wp;
    const bool n1     = w > wp; // sign of wp - w
    const float sign1 = n1 ? 1.f : -1.f;
#pragma unroll
    for (int s = 0; s < 4; ++s)
    {
        if (DF)
            Rd[s] = mk(0.f);
        else
            Rf[s] = 0.f;
    }
    const df S = add(W, WP), Pp = mul(W, WP), Dn = mul(Pp, Pp);
    const df X = n1 ? W : WP, Y = n1 ? WP : W;
    // bracket arguments from FP64 differences (eta up to ~1e3 needs 53 bits)
    const double dd = w - wp, ad = fabs(dd);
    const df dlt    = from_double(dd);    // w - wp
    const df adw    = n1 ? dlt : neg(dlt); // |w - wp|
    const int nlep = P.eta0 > 30. ? 1 : 2; // e+ terms below 1e-13 of e- for eta_e > 30
#pragma unroll 1
    for (int e = 0; e < nlep; ++e)
    {
        const double eta = e ? P.eta1 : P.eta0;
        if (y > eta * 1e-3)
        {
            const df awp = from_double(eta - wp);
            const df aab = from_double(eta - ad);
            df rwp[5], rab[5];
            fdi_raw15(awp, rwp, 1, ftab);
            fdi_raw15(aab, rab, 3, ftab);
            rab[0] = rab[1] = Q.reta[e][0];
            df dw[5], d5[5];
            fdi_diff15(rw[e], rwp, aw[e], awp, dlt, dw);
            fdi_diff15(rab, Q.reta[e], aab, Q.eta[e], adw, d5);
            const df dabs[3] = {d5[2], d5[3], d5[4]};
            const df T1 = add(dw[3], mul(add(mul(S, dw[2]), mul(mul(Pp, 3.f), dw[1])), 2.f));
            const df U  = add(mul(X, dabs[1]), mul(mul(mul(X, X), 2.f), dabs[0]));
            const df V  = add(neg(mul(Y, dabs[1])), mul(mul(mul(Y, Y), 2.f), dabs[0]));
            constexpr dfc kFifth(0.2);
            const df c1 = sub(mul(mul(dabs[2], mk(kFifth)), sign1), mul(dw[4], mk(kFifth)));
            const df A1 = sub(div(add(sub(c1, mul(S, T1)), mul(U, sign1)), Dn), mul(dw[0], 6.f));
            const df B1 = div(add(c1, mul(V, sign1)), Dn);
            constexpr dfc kBp(k::NepsBPlus), kBm(k::NepsBMinus), kBz(k::NepsBZero);
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                const df bo      = (s < 2) ? mk(kBp) : mk(kBm);
                const bool first = ((s & 1) == 0) != (e == 1);
                const df r = first ? add(mul(A1, bo), mul(B1, mk(kBz)))
                                   : add(mul(A1, mk(kBz)), mul(B1, bo));
                if (DF)
                    Rd[s] = add(Rd[s], r);
                else
                    Rf[s] += r.hi;
            }
        }
        else
        {
            double t1[4], t2[4];
            neps_taylor(P, e, w, wp, x, y, (int)sign1, n1 ? -1 : 1, t1, t2);
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                if (DF)
                    Rd[s] = add(Rd[s], from_double(t1[s]));
                else
                    Rf[s] += (float)t1[s];
            }
        }
    }
}

__device__ __forceinline__ void neps_r_mixed(const NepsPoint& P, const NepsMixed& Q,
                                             const dfm::FdiTab* ftab, double w, double wp,
                                             dfm::df W, dfm::df WP, const dfm::df (*rw)[5],
                                             const dfm::df* aw, float* R)
{
    neps_r_core<false>(P, Q, ftab, w, wp, W, WP, rw, aw, nullptr, R);
}

} // namespace
} // namespace bnsn

namespace bnsn {
namespace {

// ---------------------------------------------------------------------------
// Spectral NES/NPS in FP32 with exponent scaling.
//
// At a fixed energy w = nu/T the NES emissivity integrand carries
// e^{-(w - w')} g(w') (w' < w) and the absorption integrand e^{-(w' - w)}
// (1 - g(w')) (w' > w): for w of tens to hundreds both leave the FP32 range
// while the integral itself is an ordinary FP64 number.  The occupation
// factors are therefore formed as exponentials of double-float arguments
// minus a per-energy shift sigma (an upper estimate of the largest log
// factor over the nodes), the terms are summed in those scaled units, and
// e^{sigma} is applied in FP64.  Components whose scaled value falls below
// 2^-120 are dropped and their bound is returned, so that the caller can
// recompute in FP64 when dropped or denormal terms could matter.
// ---------------------------------------------------------------------------
constexpr float kNesDrop    = 7.52316385e-37f; // 2^-120
constexpr float kNesDropArg = -83.1777f;       // log 2^-120

struct NesSpec
{
    dfm::df invTt[4], etat[4], invTf[4], cf[4], lbf[4], lwt[4], lwf[4];
    int has_t;  // bit s: w_t of species s nonzero
    int has_fe; // bit s: free part of species s nonzero (w_f > 0, beta_f > 0)
    int has_fa; // bit s: w_f of species s nonzero (enters 1 - g)
};

// Species data of one point (call for s = 0..3; the masks come from nes_spec_masks).
__device__ __forceinline__ void nes_spec_species(const Distr& d, int s, NesSpec* Z)
{
    Z->invTt[s] = dfm::from_double(1. / d.temp_t[s]);
    Z->etat[s]  = dfm::from_double(d.eta_t[s]);
    Z->invTf[s] = dfm::from_double(1. / d.temp_f[s]);
    Z->cf[s]    = dfm::from_double(d.c_f[s]);
    Z->lbf[s]   = dfm::from_double(d.beta_f[s] > 0. ? log(d.beta_f[s]) : 0.);
    Z->lwt[s]   = dfm::from_double(d.w_t[s] > 0. ? log(d.w_t[s]) : 0.);
    Z->lwf[s]   = dfm::from_double(d.w_f[s] > 0. ? log(d.w_f[s]) : 0.);
}

__device__ __forceinline__ void nes_spec_masks(const Distr& d, NesSpec* Z)
{
    int mt = 0, mfe = 0, mfa = 0;
#pragma unroll
    for (int s = 0; s < 4; ++s)
    {
        mt |= (d.w_t[s] > 0.) << s;
        mfe |= (d.w_f[s] > 0. && d.beta_f[s] > 0.) << s;
        mfa |= (d.w_f[s] > 0.) << s;
    }
    Z->has_t  = mt;
    Z->has_fe = mfe;
    Z->has_fa = mfa;
}

// Largest estimated log occupation factor over nodes a0, a0 + step, ... < 2n
// of energy nu (w = nu/T): sig[0] for emission (g e^{-(w - w')^+}), sig[1]
// for absorption ((1 - g) e^{-(w' - w)^+}); -inf when there are no nodes.
// FP32 throughout: sigma is only a scale, its error cancels exactly.
__device__ __forceinline__ void nes_spec_scan(const NesSpec& Z, float w, float nu, float lnu,
                                              const double* x, const dfm::df* lx, int n, int a0,
                                              int step, bool nbb, float* sig)
{
    float se = -INFINITY, sa = -INFINITY;
    for (int a = a0; a < 2 * n; a += step)
    {
        const bool first = a < n;
        const int i      = first ? a : a - n;
        const float xi = (float)x[i], li = lx[i].hi;
        const float wp  = first ? w * xi : w / xi;
        const float nub = first ? nu * xi : nu / xi;
        const float lnb = first ? lnu + li : lnu - li;
        const float D   = fabsf(w - wp);
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            const bool ht = (Z.has_t >> s) & 1, hfe = (Z.has_fe >> s) & 1;
            const bool hfa = (Z.has_fa >> s) & 1;
            const float A  = nub * Z.invTt[s].hi - Z.etat[s].hi;
            const float Fn = Z.lbf[s].hi + Z.cf[s].hi * lnb - nub * Z.invTf[s].hi;
            const float le = fmaxf(ht ? Z.lwt[s].hi - fmaxf(A, 0.f) : -INFINITY,
                                   hfe ? Z.lwf[s].hi + Fn : -INFINITY);
            const float la = nbb ? 0.f
                                 : fmaxf(ht ? Z.lwt[s].hi - fmaxf(-A, 0.f) : -INFINITY,
                                         hfa ? Z.lwf[s].hi : -INFINITY);
            se = fmaxf(se, first ? le - D : le);
            sa = fmaxf(sa, first ? la : la - D);
        }
    }
    sig[0] = se;
    sig[1] = sa;
}

// exp of a double-float argument in FP32 (first-order remainder factor).
__device__ __forceinline__ float exp_of(dfm::df x) { return expf(x.hi) * (1.f + x.lo); }

// NES/NPS terms of one spectral node for the four species, in scaled units:
//   te[s] = wa w'^2 R_s (+-E/dn) g_s e^{-sig_e},
//   ta[s] = wa w'^2 R_s (+-E/dn) (1 - g_s) e^{-sig_a},
// where E = e^{-|w - w'|} sits in the emission factor for w' < w and in the
// absorption factor for w' > w, and dn = 1 - E (NEPSExpFunc,
// functions.hpp:4401-4413).  de[s], da[s] bound the dropped components of
// te[s], ta[s].
// Node arguments in df: W = nu/T, WP = nubar/T, NB = nubar, LB = log nubar
// (w, wp the same in FP64 for the branch tests of the kernel).
__device__ __forceinline__ void nes_spec_node(const NepsPoint& P, const NepsMixed& Q,
                                              const NesSpec& Z, const dfm::FdiTab* ftab,
                                              double w, double wp, dfm::df W, dfm::df WP,
                                              dfm::df NB, dfm::df LB, float wa, float sig_e,
                                              float sig_a, bool nbb, const dfm::df (*rw)[5],
                                              const dfm::df* aw, float* te, float* ta, float* de,
                                              float* da)
{
    using namespace dfm;
    float R[4];
    neps_r_mixed(P, Q, ftab, w, wp, W, WP, rw, aw, R);
    const bool first = wp < w;
    const df D       = first ? sub(W, WP) : sub(WP, W); // |w - wp|
    const float ea   = expf(-D.hi);
    const float dn   = -expm1f(-D.hi) + ea * D.lo; // 1 - e^{-D}
    const df Se = first ? add(D, sig_e) : mk(sig_e);
    const df Sa = first ? mk(sig_a) : add(D, sig_a);
    const float c = (first ? wa : -wa) * (WP.hi * WP.hi) / dn;
    float gnb = 0.f, unb = 0.f; // neglected blocking: (1 - g) -> 1
    if (nbb)
    {
        const df x = neg(Sa);
        if (x.hi < kNesDropArg)
            unb = kNesDrop;
        else
            gnb = exp_of(x);
    }
#pragma unroll
    for (int s = 0; s < 4; ++s)
    {
        const bool ht = (Z.has_t >> s) & 1, hfe = (Z.has_fe >> s) & 1;
        const bool hfa = (Z.has_fa >> s) & 1;
        float ge = 0.f, gm = nbb ? gnb : 0.f, le = 0.f, la = nbb ? unb : 0.f;
        if (ht)
        {
            const df A      = sub(mul(NB, Z.invTt[s]), Z.etat[s]);
            const float inv = 1.f / (1.f + expf(-fabsf(A.hi)));
            const bool pos  = A.hi > 0.f;
            const df x1     = sub(pos ? sub(Z.lwt[s], A) : Z.lwt[s], Se);
            if (x1.hi < kNesDropArg)
                le += kNesDrop;
            else
                ge += exp_of(x1) * inv;
            if (!nbb)
            {
                const df x3 = sub(pos ? Z.lwt[s] : add(Z.lwt[s], A), Sa);
                if (x3.hi < kNesDropArg)
                    la += kNesDrop;
                else
                    gm += exp_of(x3) * inv;
            }
        }
        df Fn = mk(0.f);
        if (hfe)
        {
            Fn          = add(Z.lbf[s], sub(mul(Z.cf[s], LB), mul(NB, Z.invTf[s])));
            const df x2 = add(Fn, sub(Z.lwf[s], Se));
            if (x2.hi < kNesDropArg)
                le += kNesDrop;
            else
                ge += exp_of(x2);
        }
        if (hfa && !nbb)
        {
            const df x4 = sub(Z.lwf[s], Sa);
            // 1 - f_free = -expm1(log f_free), accurate when f_free is near 1
            const float omf = hfe ? -(expm1f(Fn.hi) + expf(Fn.hi) * Fn.lo) : 1.f;
            if (x4.hi < kNesDropArg)
                la += kNesDrop;
            else
                gm += exp_of(x4) * omf;
        }
        const float k = c * R[s];
        te[s] = k * ge;
        ta[s] = k * gm;
        de[s] = fabsf(k) * le;
        da[s] = fabsf(k) * la;
    }
}

// nes_spec_node with every product after the Fermi integrals in df (the
// accurate pass over energies whose FP32 terms cancel): te, ta in the same
// scaled units, rounded to FP64.
__device__ __forceinline__ void nes_spec_node_df(const NepsPoint& P, const NepsMixed& Q,
                                                 const NesSpec& Z, const dfm::FdiTab* ftab,
                                                 double w, double wp, dfm::df W, dfm::df WP,
                                                 dfm::df NB, dfm::df LB, double wa, float sig_e,
                                                 float sig_a, bool nbb, const dfm::df (*rw)[5],
                                                 const dfm::df* aw, double* te, double* ta,
                                                 float* de, float* da)
{
    using namespace dfm;
    df R[4];
    neps_r_core<true>(P, Q, ftab, w, wp, W, WP, rw, aw, R, nullptr);
    const bool first = wp < w;
    const df D       = first ? sub(W, WP) : sub(WP, W);
    const df dn      = add(neg(exp_df(neg(D))), 1.f); // 1 - e^{-D}, D > 0
    const df Se = first ? add(D, sig_e) : mk(sig_e);
    const df Sa = first ? mk(sig_a) : add(D, sig_a);
    const df c  = div(mul(from_double(first ? wa : -wa), mul(WP, WP)), dn);
    df gnb = mk(0.f);
    float unb = 0.f;
    if (nbb)
    {
        const df x = neg(Sa);
        if (x.hi < kNesDropArg)
            unb = kNesDrop;
        else
            gnb = exp_df(x);
    }
#pragma unroll 1
    for (int s = 0; s < 4; ++s)
    {
        const bool ht = (Z.has_t >> s) & 1, hfe = (Z.has_fe >> s) & 1;
        const bool hfa = (Z.has_fa >> s) & 1;
        df ge = mk(0.f), gm = nbb ? gnb : mk(0.f);
        float le = 0.f, la = nbb ? unb : 0.f;
        if (ht)
        {
            const df A     = sub(mul(NB, Z.invTt[s]), Z.etat[s]);
            const bool pos = A.hi > 0.f;
            const df t     = exp_df(pos ? neg(A) : A); // e^{-|A|}
            const df inv   = div(mk(1.f), add(t, 1.f));
            const df x1    = sub(pos ? sub(Z.lwt[s], A) : Z.lwt[s], Se);
            if (x1.hi < kNesDropArg)
                le += kNesDrop;
            else
                ge = add(ge, mul(exp_df(x1), inv));
            if (!nbb)
            {
                const df x3 = sub(pos ? Z.lwt[s] : add(Z.lwt[s], A), Sa);
                if (x3.hi < kNesDropArg)
                    la += kNesDrop;
                else
                    gm = add(gm, mul(exp_df(x3), inv));
            }
        }
        df Fn = mk(0.f);
        if (hfe)
        {
            Fn          = add(Z.lbf[s], sub(mul(Z.cf[s], LB), mul(NB, Z.invTf[s])));
            const df x2 = add(Fn, sub(Z.lwf[s], Se));
            if (x2.hi < kNesDropArg)
                le += kNesDrop;
            else
                ge = add(ge, exp_df(x2));
        }
        if (hfa && !nbb)
        {
            const df x4  = sub(Z.lwf[s], Sa);
            const df omf = hfe ? add(neg(exp_df(Fn)), 1.f) : mk(1.f);
            if (x4.hi < kNesDropArg)
                la += kNesDrop;
            else
                gm = add(gm, mul(exp_df(x4), omf));
        }
        const df k = mul(c, R[s]);
        te[s]      = to_double(mul(k, ge));
        ta[s]      = to_double(mul(k, gm));
        de[s]      = fabsf(k.hi) * le;
        da[s]      = fabsf(k.hi) * la;
    }
}

} // namespace
} // namespace bnsn
