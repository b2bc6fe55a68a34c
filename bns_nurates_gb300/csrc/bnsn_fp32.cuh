// Single-precision device physics of the mixed-precision path.
//
// Only bounded, cancellation-free shape functions run in FP32; their
// dimensionful prefactors, every Fermi-Dirac integral and the distribution
// algebra stay in FP64 (bnsn_fp64.cuh).
#pragma once

#include <math.h>

#include "bnsn_constants.h"
#include "bnsn_df.cuh"
#include "bnsn_fp64.cuh"

namespace bnsn {
namespace fp32 {

#define BNSN_DI __device__ __forceinline__

// HR98 bremsstrahlung (kernel_brem_HR98.hpp:33-338) split into per-point FP64
// constants (below, rounded to FP32 or kept as double-float) and an FP32
// shape of x = (w + w')/T:
//   s_abs(x) = outer * sum_ch pre_ch * S_ch(x) / (x^2 + hgg_ch^2)
// with outer = 3 C_brem / medium correction and pre_ch = n_ch gamma_ch / T.
// The non-degenerate part s_nd (Eq. 45: a ratio of powers up to x^4) and the
// factors x (x^2 + 4 pi^2) / (1 - e^-x) of s_d run in double-float from the
// double-float x: in FP32 their rounding (and that of x itself, amplified up
// to 4x by q^4) reached 8.5e-7 of the shape.
struct Hr98Mixed
{
    float y, poly_y, y4p1, Dy, p, pinv;
    float K1fu[3], eta2p1[3], sqe[3], ep2[3], h[3], hgg2[3], pre[3];
    dfm::df cX, cq, cp, y2; // 2 - e^{-y/12}, pi^(1/8) + y, 5 y^2 / 3 + 1, 2 y
    double outer;
};

BNSN_DI void hr98_mixed_from(const fp64::Hr98Point& P, Hr98Mixed* M)
{
    M->y      = (float)P.y;
    M->poly_y = (float)P.poly_y;
    M->y4p1   = (float)P.y4p1;
    M->Dy     = (float)P.Dy;
    M->p      = (float)(-P.mp);
    M->pinv   = (float)(-P.minv);
    M->cX     = dfm::from_double(2. - P.ey12);
    M->cq     = dfm::from_double(k::Pi18 + P.y);
    M->cp     = dfm::from_double(P.poly_y + 1.);
    M->y2     = dfm::from_double(2. * P.y);
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        const fp64::Hr98Channel& C = P.ch[c];
        M->K1fu[c]   = (float)(C.K1 * C.f_u / k::FourPiSq);
        M->eta2p1[c] = (float)C.eta2p1;
        M->sqe[c]    = (float)C.sqe;
        M->ep2[c]    = (float)C.ep2;
        M->h[c]      = (float)C.h;
        M->hgg2[c]   = (float)(C.hgg * C.hgg);
        M->pre[c]    = (float)(C.weight * C.gamma / P.T);
    }
    M->outer = 3. * k::BremConst / P.mcorr;
}

// x^p for x > 0 to about 1 ulp: log2 x = k + log2 m with the binary exponent
// k exact and m in [1, 2); p log2 x is carried as hi + lo (exact product of p
// and k), split into an integer n and a fraction f, and x^p = 2^n exp2(f).
// exp(p log x) in FP32 loses |p log x| ulps in the rounded argument.
BNSN_DI float powf_acc(float x, float p)
{
    int k;
    const float m  = frexpf(x, &k); // x = m 2^k, m in [0.5, 1)
    const float lm = log2f(m);      // in [-1, 0)
    const float kf = (float)k;
    const float hi = p * kf;
    const float lo = fmaf(p, kf, -hi) + p * lm; // p k - hi exactly, plus p log2 m
    const float n  = rintf(hi);
    const float f  = (hi - n) + lo;             // hi - n exact
    return ldexpf(exp2f(f), (int)n);
}

// Sum over the three NN channels of n gamma S(x) / (T (x^2 + (gamma g/2)^2))
// at x = xh + xl (double-float).  The interpolation (s_nd^-p + s_d^-p)^(-1/p)
// of Eq.(49) is evaluated as min * (1 + (max/min)^-p)^(-1/p): the same value,
// but the outer power acts on a number in [1, 2], which keeps its FP32
// rounding error at the ulp level instead of growing with |p log s|.
BNSN_DI float hr98_shape(const Hr98Mixed& M, float xh_in, float xl_in)
{
    using namespace dfm;
    constexpr dfc kSqrtPi(k::SqrtPi), kTwoSqrtPi(2. * k::SqrtPi), kFourPiSq(k::FourPiSq);
    const bool clamp = xh_in < (float)k::BremXmin;
    const df X1      = clamp ? mk((float)k::BremXmin) : df{xh_in, xl_in}; // x clamped
    const float x    = X1.hi;
    const float y    = M.y;
    // s_nd = 2 sqrt(pi) X^1.5 (x^2 + 2 x y + 5 y^2 / 3 + 1) / (sqrt(pi) + q^4)
    const df Xd   = add(X1, M.cX);                       // X = x + 2 - e^{-y/12}
    const float sx = sqrtf(Xd.hi);
    const df sX   = {sx, (fmaf(-sx, sx, Xd.hi) + Xd.lo) / (2.f * sx)}; // sqrt(X), one Newton step
    const df poly = add(mul(X1, add(X1, M.y2)), M.cp);
    const df q    = add(X1, M.cq);
    const df q2   = mul(q, q);
    const df den  = add(mul(q2, q2), mk(kSqrtPi));
    const df sndd = div(mul(mul(mul(Xd, sX), poly), mk(kTwoSqrtPi)), den);
    const float snd = sndd.hi + sndd.lo;
    // x (x^2 + 4 pi^2) / (1 - e^-x) of s_d
    const float ex   = expf(-x);
    const float em1  = -expm1f(-x) + ex * X1.lo;
    const df X2x     = mul(add(mul(X1, X1), mk(kFourPiSq)), X1);
    const float sdx  = (X2x.hi + X2x.lo) / em1;
    const float px11  = powf_acc(x, 1.1f);
    const float px093 = powf_acc(x, 0.93f);
    const float px12  = powf_acc(x, 1.2f);
    const float px28  = powf_acc(x, 2.8f);
    const float x2    = x * x;
    const float xterm = 3.f + (x - 1.2f) * (x - 1.2f) + 1.f / (x2 * x2);
    const float gpart = 0.0044f * px11 * y / M.Dy;
    const float cden2 = 30.f + 0.005f * px28;
    const df XS       = {xh_in, xl_in}; // x unclamped, as the reference's x^2
    const df xs2d     = mul(XS, XS);
    const float xs2   = xs2d.hi + xs2d.lo;
    float tot         = 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        const float s_d    = M.K1fu[c] * sdx;
        const float lo     = fminf(snd, s_d);
        const float hi     = fmaxf(snd, s_d);
        const float t      = powf_acc(hi / lo, -M.p);
        const float s_base = lo * expf(-log1pf(t) * M.pinv);
        const float f_brem = 1.f + 1.f / (xterm * M.eta2p1[c] * M.y4p1);
        const float g_brem = 1.f - gpart * M.sqe[c] / M.ep2[c];
        const float c_brem =
            1.1f * px11 * M.h[c] / (2.3f + M.h[c] * px093 + 0.0001f * px12) * 30.f / cden2;
        const float s = s_base * f_brem * (1.f + c_brem * g_brem);
        tot += M.pre[c] * s / (xs2 + M.hgg2[c]);
    }
    return tot;
}

// K_1(x) e^{x} for x > 0 (the BRT06 brem kernel's Bessel factor with its
// detailed-balance exponential folded in): the polynomial approximations of
// Abramowitz & Stegun 9.8.3, 9.8.7 and 9.8.8 that the FP64 bessk1 uses
// (functions.hpp:99-180), evaluated in FP32; e^{x} multiplies K_1 for
// x <= 2 and cancels the e^{-x} of the large-x form otherwise, so the result
// stays O(x^{-1/2}) at any x.
BNSN_DI float bessk1e(float x)
{
    if (x <= 2.f)
    {
        const float t  = x * (1.f / 3.75f);
        const float u  = t * t;
        const float i1 = x * (0.5f + u * (0.87890594f + u * (0.51498869f + u * (0.15084934f +
                         u * (0.2658733e-1f + u * (0.301532e-2f + u * 0.32411e-3f))))));
        const float y  = 0.25f * (x * x);
        const float k1 = logf(0.5f * x) * i1 +
                         (1.f / x) * (1.f + y * (0.15443144f + y * (-0.67278579f +
                         y * (-0.18156897f + y * (-0.1919402e-1f + y * (-0.110404e-2f +
                         y * (-0.4686e-4f)))))));
        return k1 * expf(x);
    }
    const float y = 2.f / x;
    return (1.25331414f + y * (0.23498619f + y * (-0.3655620e-1f + y * (0.1504268e-1f +
            y * (-0.780353e-2f + y * (0.325614e-2f + y * (-0.68245e-3f))))))) /
           sqrtf(x);
}

// The iso-energetic scattering kernel's weak-magnetism factor of one nucleon
// (reac 1: protons, 2: neutrons) in FP32: (C0 R0 - C1 R1 / 3) / IsoConst of
// formulas_beta_iso.hpp:411-507 with R0, R1 of weak_magnetism.hpp:165-210 and
// the form factors of weak_magnetism.hpp:45-104.  All its terms are positive
// (cv F2 >= 0 for both nucleons), so FP32 keeps ~1e-7; 1 - 1/(1 + 5.6 tau) is
// formed as 5.6 tau / (1 + 5.6 tau), without the cancellation at small tau.
BNSN_DI float iso_wm_factor(float omega, int reac)
{
    constexpr float lamp = 1.793f, lamn = -1.913f;
    constexpr float cw   = (float)(0.5 - 2. * k::SinThW2);
    const float e    = omega * (float)k::WmEScale;
    const float tau  = 0.5f * (e * e) / (1.f + e);
    const float eta  = 1.f / (1.f + 5.6f * tau);
    const float gq   = 1.f + 4.97f * tau;
    const float Gt   = 1.f / ((gq * gq) * (1.f + tau));
    const float Fp1  = (1.f + tau * (1.f + lamp)) * Gt;
    const float Fp2  = lamp * Gt;
    const float Fn1  = tau * lamn * (5.6f * tau * eta) * Gt;
    const float Fn2  = lamn * (1.f + tau * eta) * Gt;
    const float d3   = 1.f + 3.53f * tau;
    const float cv   = reac == 1 ? cw * Fp1 - 0.5f * Fn1 : cw * Fn1 - 0.5f * Fp1;
    const float ca   = (reac == 1 ? 0.5f * (float)(k::Ga - k::Gs) : -0.5f * (float)(k::Ga + k::Gs)) /
                     (d3 * d3);
    const float F2   = reac == 1 ? cw * Fp2 - 0.5f * Fn2 : cw * Fn2 - 0.5f * Fp2;
    const float ef   = e * F2;
    const float A0   = (cv * cv) + 3.f * (ca * ca) + 1.5f * (ef * ef) + 2.f * (e * e) * cv * F2;
    const float A1   = (cv * cv) - (ca * ca) - 2.f * (ef * ef) - 4.f * (e * e) * cv * F2;
    return A0 - A1 * (1.f / 3.f);
}

#undef BNSN_DI

} // namespace fp32
} // namespace bnsn
