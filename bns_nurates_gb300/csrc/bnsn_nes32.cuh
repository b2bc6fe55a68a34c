// NES/NPS kernels of the mixed path as cancellation-free FP32 integrals.
//
// The reference's out-kernel integral MezzacappaIntOut(w, w')
// (kernel_nes.hpp:50-78) combines F_1..F_5 at eta - w', eta - w, eta and
// eta - |w - w'| with polynomial coefficients over w^2 w'^2, linearly in the
// couplings b1, b2.  Writing F_k(eta + c) = int_{-c}^inf (u + c)^k f(u - eta) du
// (f(t) = 1/(1 + e^t)) turns it into
//
//   MezzacappaIntOut = sign * [b1 I_1 + b2 I_2] / (x^2 y^2),
//   I_l = int_0^inf K_l(u) f(u - eta) du,
//
// with x = max(w, w'), y = min(w, w'), sign = +1 for w > w' and -1 otherwise
// (the reference's `sign`), and K_l >= 0 piecewise polynomial: quintics on
// [0, m], [m, m + e], [m + e, x] (m = min(y, x - y), e = |x - 2y|) and linear
// on [x, inf).  In the Bernstein basis of each finite piece the coefficients
// are polynomials in m and e with non-negative coefficients
// (bns_nurates_gb300/nes_forms.py derives them from the reference formula and
// checks that), so the kernel evaluates with no cancellation; the reference
// formula cancels catastrophically in degenerate matter and at small energies.
// The reverse direction needs no second integral: MezzacappaIntOut(w', w) =
// -MezzacappaIntOut(w, w').
//
// Quadrature in u (eta = the lepton's degeneracy, e- or e+), as for the pair
// kernel (bnsn_pair32.cuh): Gauss-Legendre with 8 nodes on panels 4 wide
// within +-16 of the Fermi edge u = eta; 3-node Gauss-Legendre below it (f = 1
// to 1e-7, exact for quintics); above it f = e^{eta - u}: 3-node
// Gauss-Laguerre from the segment start where the piece extends >= 30 beyond
// it (the remainder past the piece end is below 1e-8), else Gauss-Legendre
// panels 6 wide.  The linear piece on [x, inf) is integrated in closed
// form, A F_0(eta - x) + B F_1(eta - x).  Everything is scaled by e^{-Lref},
// Lref = min(eta, 0), so the integrand's largest value is O(1) in FP32.
//
// Panels are exactly kPanel (kFall) wide from the segment start, the last
// one the remainder, so the occupation factor at a node of a full panel is
//   phi = 1 / (A + e^{v_c} E_k),  E_k = e^{hw t_k} a correctly rounded table,
// with e^{v_c} at the panel centre from expf: one FMA and one approximate
// reciprocal per node.  The quintic is the homogeneous Horner form in
// (tau, rho) = (t, r) / L, both formed by one FMA from the panel's centre.
// Nothing in a node's evaluation subtracts: its rounding errors stay a few
// 1e-8 and are independent from node to node.

#pragma once

#include "bnsn_df.cuh"

namespace bnsn {
namespace nes32 {

constexpr float kEdge     = 16.f; // half-width of the Fermi-edge zone
constexpr float kPanel    = 4.f;  // panel width in the edge zone
constexpr float kFall     = 6.f;  // panel width above the edge zone
constexpr float kLagSpan  = 30.f; // Laguerre from a segment start if the piece reaches this far

__device__ __constant__ const float kG8t[4] = {0.18343464249564978f, 0.525532409916329f,
                                               0.7966664774136267f, 0.9602898564975362f};
__device__ __constant__ const float kG8w[4] = {0.36268378337836166f, 0.3137066458778869f,
                                               0.22238103445337443f, 0.10122853629037706f};
// e^{hw t} at the 8 nodes (+t_k, -t_k pairs) of a full panel, hw = 2 and 3
__device__ __constant__ const float kE2[8] = {
    1.4432092905044556f, 0.6929002404212952f, 2.8606956005096436f, 0.349565327167511f,
    4.9201202392578125f, 0.2032470554113388f, 6.824913501739502f,  0.14652200043201447f};
__device__ __constant__ const float kE3[8] = {
    1.733779788017273f,  0.5767744779586792f,  4.83846378326416f,   0.2066771686077118f,
    10.913488388061523f, 0.09162972867488861f, 17.829769134521484f, 0.0560859739780426f};
constexpr float kG3t = 0.7745966692414834f, kG3w0 = 0.8888888888888888f,
                kG3w1 = 0.5555555555555556f;
__device__ __constant__ const float kLagT[3] = {0.4157745567834791f, 2.294280360279042f,
                                                6.2899450829374794f};
__device__ __constant__ const float kLagW[3] = {0.7110930099291729f, 0.278517733569241f,
                                                0.010389256501586133f};
// R(t) = F_1(t) / F_0(t) on [-2, 2] as a Chebyshev series in t / 2 (c_0
// halved), F_0(t) = ln(1 + e^t), F_1(t) = -Li_2(-e^t) (nes_forms.py, mpmath;
// truncation below 4e-9 relative).
__device__ __constant__ const float kRcheb[13] = {
    1.2661236754389507f,     0.30499188429691676f,    0.07771025854852331f,
    0.005195668746712225f,   -0.0017622100274969996f, -0.0002334905678526031f,
    7.758964026037337e-05f,  1.2508351105798513e-05f, -4.231493146199279e-06f,
    -7.418171543928765e-07f, 2.57367408166754e-07f,   4.704674539515587e-08f,
    -1.6724525594697865e-08f};

__device__ __forceinline__ float dsub(dfm::df a, dfm::df b)
{
    return (a.hi - b.hi) + (a.lo - b.lo);
}

// e^{a - b} for df a, b to FP32 accuracy at any |a - b|: the exponent's
// float value and its remainder (a float difference alone loses |a - b| x
// 6e-8 of relative accuracy in the exponential).
__device__ __forceinline__ float exp_diff(dfm::df a, dfm::df b)
{
    const dfm::df d = dfm::two_sum(a.hi, -b.hi);
    const dfm::df s = dfm::fast_two_sum(d.hi, d.lo + (a.lo - b.lo));
    return expf(s.hi) * (1.f + s.lo);
}

// Bernstein coefficients (times C(5, j)) of K_1 (g1) and K_2 (g2) on piece k.
__device__ __forceinline__ void piece_coeffs(int k, bool dgy, float m, float e, float* g1,
                                             float* g2)
{
    const float m2 = m * m, m3 = m2 * m, e2 = e * e;
    const float em = e + m, e2m = e + 2.f * m;
    const float q51  = fmaf(10.f, e2, fmaf(45.f, e * m, 51.f * m2)); // 10e^2+45em+51m^2
    const float q6   = fmaf(10.f, e2, fmaf(15.f, e * m, 6.f * m2));  // 10e^2+15em+6m^2
    if (k == 0)
    {
        g1[0] = g1[1] = g1[2] = 0.f;
        g1[3] = 2.f * m3 * e2m * e2m;
        g1[4] = m3 * e2m * fmaf(4.f, e, 9.f * m);
        g1[5] = 0.2f * m3 * q51;
        g2[0] = g2[1] = g2[2] = 0.f;
        if (dgy)
        {
            const float m5 = m3 * m2;
            g2[3] = 2.f * m5;
            g2[4] = 3.f * m5;
            g2[5] = 1.2f * m5;
        }
        else
        {
            g2[3] = 2.f * m3 * em * em;
            g2[4] = m3 * em * fmaf(4.f, e, 3.f * m);
            g2[5] = 0.2f * m3 * q6;
        }
        return;
    }
    if (dgy)
    {
        if (k == 1)
        {
            g1[0] = 0.2f * m3 * q51;
            g1[1] = m3 * fmaf(14.f, e2, fmaf(54.f, e * m, 51.f * m2));
            g1[2] = 2.f * m3 * fmaf(19.f, e2, fmaf(63.f, e * m, 51.f * m2));
            g1[3] = 2.f * m3 * fmaf(25.f, e2, fmaf(72.f, e * m, 51.f * m2));
            g1[4] = m3 * fmaf(32.f, e2, fmaf(81.f, e * m, 51.f * m2));
            g1[5] = 0.2f * m3 * fmaf(40.f, e2, fmaf(90.f, e * m, 51.f * m2));
            g2[0] = 1.2f * m3 * m2;
            g2[1] = 3.f * m2 * m2 * e2m;
            g2[2] = 2.f * m3 * fmaf(e, e + 6.f * m, 6.f * m2);
            g2[3] = 6.f * m3 * em * e2m;
            g2[4] = 6.f * m3 * em * em;
            g2[5] = 0.2f * m3 * q6;
        }
        else
        {
            g1[0] = 0.2f * m3 * fmaf(40.f, e2, fmaf(90.f, e * m, 51.f * m2));
            g1[1] = 2.f * m3 * fmaf(4.f, e, 5.f * m) * fmaf(5.f, e, 6.f * m);
            g1[2] = 4.f * m3 * fmaf(4.f, e, 5.f * m) * fmaf(5.f, e, 7.f * m);
            g1[3] = 2.f * m3 * fmaf(39.f, e2, fmaf(110.f, e * m, 77.f * m2));
            g1[4] = 3.f * m3 * fmaf(3.f, e, 5.f * m) * fmaf(4.f, e, 5.f * m);
            g1[5] = m3 * em * fmaf(6.f, e, 11.f * m);
            g2[0] = 0.2f * m3 * q6;
            g2[1] = m3 * em * fmaf(10.f, e, 9.f * m);
            g2[2] = 2.f * m3 * em * fmaf(10.f, e, 13.f * m);
            g2[3] = 2.f * m3 * em * fmaf(10.f, e, 17.f * m);
            g2[4] = m3 * em * fmaf(10.f, e, 21.f * m);
            g2[5] = m3 * em * fmaf(2.f, e, 5.f * m);
        }
        return;
    }
    const float e3 = e2 * e, e4 = e2 * e2, m4 = m2 * m2;
    // 55e^4+230e^3m+340e^2m^2+210em^3+51m^4 and 15e^4+50e^3m+60e^2m^2+30em^3+6m^4
    const float p55 = fmaf(55.f, e4, fmaf(230.f, e3 * m, fmaf(340.f, e2 * m2,
                                                              fmaf(210.f, e * m3, 51.f * m4))));
    const float p15 = fmaf(15.f, e4, fmaf(50.f, e3 * m, fmaf(60.f, e2 * m2,
                                                             fmaf(30.f, e * m3, 6.f * m4))));
    const float em3 = em * em * em;
    if (k == 1)
    {
        g1[0] = 0.2f * m3 * q51;
        g1[1] = m2 * fmaf(6.f, e3, fmaf(38.f, e2 * m, fmaf(78.f, e * m2, 51.f * m3)));
        g1[2] = 2.f * m * fmaf(3.f, e4, fmaf(27.f, e3 * m, fmaf(85.f, e2 * m2,
                                                                fmaf(111.f, e * m3, 51.f * m4))));
        g1[3] = 2.f * m * fmaf(11.f, e4, fmaf(68.f, e3 * m, fmaf(151.f, e2 * m2,
                                                                 fmaf(144.f, e * m3, 51.f * m4))));
        g1[4] = m * fmaf(27.f, e4, fmaf(134.f, e3 * m, fmaf(236.f, e2 * m2,
                                                            fmaf(177.f, e * m3, 51.f * m4))));
        g1[5] = 0.2f * m * p55;
        g2[0] = 0.2f * m3 * q6;
        g2[1] = 6.f * m2 * em3;
        g2[2] = 6.f * m * em3 * e2m;
        g2[3] = 2.f * m * em * em * fmaf(7.f, e2, fmaf(12.f, e * m, 6.f * m2));
        g2[4] = m * em * fmaf(11.f, e3, fmaf(27.f, e2 * m, fmaf(21.f, e * m2, 6.f * m3)));
        g2[5] = 0.2f * m * p15;
    }
    else
    {
        g1[0] = 0.2f * m * p55;
        g1[1] = m * fmaf(49.f, e4, fmaf(222.f, e3 * m, fmaf(358.f, e2 * m2,
                                                            fmaf(242.f, e * m3, 60.f * m4))));
        g1[2] = 2.f * m * fmaf(43.f, e4, fmaf(208.f, e3 * m, fmaf(361.f, e2 * m2,
                                                                  fmaf(265.f, e * m3, 70.f * m4))));
        g1[3] = 2.f * m * em * fmaf(37.f, e3, fmaf(151.f, e2 * m, fmaf(194.f, e * m2, 77.f * m3)));
        g1[4] = m * em * em * fmaf(31.f, e2, fmaf(100.f, e * m, 75.f * m2));
        g1[5] = m * em3 * fmaf(5.f, e, 11.f * m);
        g2[0] = 0.2f * m * p15;
        g2[1] = 3.f * m * em3 * fmaf(5.f, e, 3.f * m);
        g2[2] = 2.f * m * em3 * fmaf(15.f, e, 13.f * m);
        g2[3] = 2.f * m * em3 * fmaf(15.f, e, 17.f * m);
        g2[4] = 3.f * m * em3 * fmaf(5.f, e, 7.f * m);
        g2[5] = m * em3 * fmaf(3.f, e, 5.f * m);
    }
}

// K on a piece from its Bernstein coefficients at tau = t / L, rho = r / L.
__device__ __forceinline__ void bern2(const float* g1, const float* g2, float tau, float rho,
                                      float& k1, float& k2)
{
    const float r2 = rho * rho, r3 = r2 * rho, r4 = r2 * r2, r5 = r4 * rho;
    float a = g1[5], b = g2[5];
    a = fmaf(a, tau, g1[4] * rho);
    b = fmaf(b, tau, g2[4] * rho);
    a = fmaf(a, tau, g1[3] * r2);
    b = fmaf(b, tau, g2[3] * r2);
    a = fmaf(a, tau, g1[2] * r3);
    b = fmaf(b, tau, g2[2] * r3);
    a = fmaf(a, tau, g1[1] * r4);
    b = fmaf(b, tau, g2[1] * r4);
    k1 = fmaf(a, tau, g1[0] * r5);
    k2 = fmaf(b, tau, g2[0] * r5);
}

// 1/k^2 for the dilogarithm series.
__device__ __constant__ const float kInvK2[12] = {
    1.f,           0.25f,         0.11111111f,  0.0625f,       0.04f,        0.027777778f,
    0.020408163f,  0.015625f,     0.012345679f, 0.01f,         0.008264462f, 0.0069444445f};

// F_1(t) = -Li_2(-e^t) and F_0(t) = ln(1 + e^t), times e^{-sh} with sh the
// caller's scale (Lref, e^{-sh} = esh): the closed-form tail.  etsh = e^{t - sh}
// from the caller to FP32 accuracy (it sets the magnitude where t < -2).
__device__ __forceinline__ void fermi01_scaled(float t, float etsh, float esh, float& f0,
                                               float& f1)
{
    if (t < -2.f)
    {
        // F_k = z S_k(z), z = e^t <= e^-2: alternating series, first term dominant
        const float z = expf(t);
        float s1 = 0.f, zp = 1.f;
#pragma unroll
        for (int k = 1; k <= 12; ++k)
        {
            const float term = zp * kInvK2[k - 1];
            s1 += (k & 1) ? term : -term;
            zp *= z;
        }
        const float s0 = z < 1e-4f ? fmaf(-0.5f, z, 1.f) : log1pf(z) / z;
        f0 = etsh * s0;
        f1 = etsh * s1;
        return;
    }
    const float F0 = t > 0.f ? t + log1pf(expf(-t)) : log1pf(expf(t));
    float F1;
    if (t <= 2.f)
    {
        // Clenshaw for R = F_1 / F_0 at s = t / 2
        const float s = 0.5f * t;
        float bk1 = 0.f, bk2 = 0.f;
#pragma unroll
        for (int k = 12; k >= 1; --k)
        {
            const float bk = fmaf(2.f * s, bk1, kRcheb[k] - bk2);
            bk2 = bk1;
            bk1 = bk;
        }
        const float R = fmaf(s, bk1, kRcheb[0] - bk2);
        F1 = F0 * R;
    }
    else
    {
        // reflection: F_1(t) = t^2/2 + pi^2/6 - F_1(-t), the last term small
        const float z = expf(-t);
        float s1 = 0.f, zp = z;
#pragma unroll
        for (int k = 1; k <= 12; ++k)
        {
            const float term = zp * kInvK2[k - 1];
            s1 += (k & 1) ? term : -term;
            zp *= z;
        }
        F1 = fmaf(0.5f * t, t, 1.6449340668482264f - s1);
    }
    f0 = F0 * esh;
    f1 = F1 * esh;
}

// Approximate 1/x (one special-function instruction, about 1 ulp); a
// denormal result flushes to zero.
__device__ __forceinline__ float rcpa(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 1/x to 1/2 ulp: the approximate reciprocal and one Newton step.
__device__ __forceinline__ float rcp_nr(float x)
{
    const float r = rcpa(x);
    return fmaf(r, fmaf(-x, r, 1.f), r);
}

// Per-point constants of one lepton (e- with eta = mu_e/T, e+ with -eta).
// The integrand's occupation factor, scaled by e^{-Lref} with
// Lref = min(eta, 0) so that its largest value is O(1), is written
//   phi(u) = e^{-Lref} / (1 + e^{u - eta}) = 1 / (A + e^v),  v = u - vsh,
// with (A, vsh) = (1, eta) for eta >= 0 and (e^eta, 0) below: the exponent
// v stays small where phi matters.
struct Lepton
{
    dfm::df eta, vsh;
    float A, iA;  // e^{Lref}, e^{-Lref}
    float z1, z2; // Fermi-edge zone eta -+ kEdge
    dfm::df thr;  // 1e-3 eta: the reference's Taylor branches below y = thr
};

__device__ __forceinline__ Lepton make_lepton(double eta)
{
    Lepton Lp;
    const double lref = eta < 0. ? eta : 0.;
    Lp.eta = dfm::from_double(eta);
    Lp.vsh = dfm::from_double(eta - lref);
    Lp.A   = (float)exp(lref);
    Lp.iA  = (float)exp(-lref);
    Lp.z1  = Lp.eta.hi - kEdge;
    Lp.z2  = Lp.eta.hi + kEdge;
    Lp.thr = dfm::from_double(eta * 1e-3);
    return Lp;
}

// Geometry of one (w, w') pair, shared by both leptons.
struct Geo
{
    dfm::df E1, E2, X; // piece ends m, m + e, x
    dfm::df Y;         // y = min(w, w')
    float m, e;        // piece lengths m (pieces 0, 2) and e (piece 1)
    bool dgy;          // x - y > y
};

__device__ __forceinline__ bool df_gt(dfm::df a, dfm::df b)
{
    return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}

__device__ __forceinline__ Geo make_geo(dfm::df W, dfm::df WP)
{
    using namespace dfm;
    Geo G;
    const bool wg = df_gt(W, WP);
    G.X           = wg ? W : WP;
    G.Y           = wg ? WP : W;
    const df D    = sub(G.X, G.Y);
    G.dgy         = df_gt(D, G.Y);
    G.E1          = G.dgy ? G.Y : D;
    G.E2          = G.dgy ? D : G.Y;
    // the correctly rounded lengths (the coefficients' m and e)
    G.m           = G.E1.hi;
    G.e           = sub(G.E2, G.E1).hi;
    return G;
}

__device__ __forceinline__ Geo make_geo(double w, double wp)
{
    return make_geo(dfm::from_double(w), dfm::from_double(wp));
}

// Reference's branch condition y > 1e-3 eta, on the df values.
__device__ __forceinline__ bool above_taylor(const Geo& G, const Lepton& Lp)
{
    return df_gt(G.Y, Lp.thr);
}

// Ihat_1, Ihat_2 of one lepton: I_l = A * Ihat_l (A = e^{Lref}).
__device__ __forceinline__ void lepton_integrals(const Geo& G, const Lepton& Lp, float& I1,
                                                 float& I2)
{
    using namespace dfm;
    df A1 = mk(0.f), A2 = mk(0.f);
#pragma unroll 1
    for (int k = 0; k < 3; ++k)
    {
        const df P    = k == 0 ? mk(0.f) : (k == 1 ? G.E1 : G.E2);
        const df Q    = k == 0 ? G.E1 : (k == 1 ? G.E2 : G.X);
        const df Ld   = sub(Q, P);
        if (!(Ld.hi > 0.f))
            continue;
        // 1/L of the df length: tau = t/L and rho = r/L from the df positions
        // sum to 1 within an ulp, so the quintic carries no common scale error
        const float iLh = 1.f / Ld.hi;
        const float iLl = (fmaf(-Ld.hi, iLh, 1.f) - Ld.lo * iLh) * iLh;
        float g1[6], g2[6];
        piece_coeffs(k, G.dgy, G.m, G.e, g1, g2);
        df U = P;
#pragma unroll 1
        for (int j = 0; j <= 2; ++j)
        {
            df V = Q;
            if (j < 2)
            {
                const float zc = j == 0 ? Lp.z1 : Lp.z2;
                if (!(zc > U.hi && zc < Q.hi))
                    continue;
                V = mk(zc);
            }
            const float len = dsub(V, U);
            const float mid = U.hi + 0.5f * len;
            float s1 = 0.f, s2 = 0.f;
            if (mid < Lp.z1)
            {
                // below the edge (eta > E, Lref = 0): phi = 1, exact for quintics
                const float hw = 0.5f * len;
                const df CM    = add(U, hw);
                const float tc = dsub(CM, P), rc = dsub(Q, CM);
                const float dt = hw * kG3t;
                float k1, k2;
                bern2(g1, g2, fmaf(tc, iLh, tc * iLl), fmaf(rc, iLh, rc * iLl), k1, k2);
                s1 = kG3w0 * k1;
                s2 = kG3w0 * k2;
                const float ta = tc + dt, ra = rc - dt, tb = tc - dt, rb = rc + dt;
                bern2(g1, g2, fmaf(ta, iLh, ta * iLl), fmaf(ra, iLh, ra * iLl), k1, k2);
                s1 = fmaf(kG3w1, k1, s1);
                s2 = fmaf(kG3w1, k2, s2);
                bern2(g1, g2, fmaf(tb, iLh, tb * iLl), fmaf(rb, iLh, rb * iLl), k1, k2);
                s1 = hw * fmaf(kG3w1, k1, s1);
                s2 = hw * fmaf(kG3w1, k2, s2);
            }
            else if (mid > Lp.z2 && dsub(Q, U) >= kLagSpan)
            {
                // above the edge: phi = e^{-v}, Laguerre from U
                const float tu = dsub(U, P), ru = dsub(Q, U);
#pragma unroll
                for (int i = 0; i < 3; ++i)
                {
                    const float ta = tu + kLagT[i], ra = ru - kLagT[i];
                    float k1, k2;
                    bern2(g1, g2, fmaf(ta, iLh, ta * iLl), fmaf(ra, iLh, ra * iLl), k1, k2);
                    s1 = fmaf(kLagW[i], k1, s1);
                    s2 = fmaf(kLagW[i], k2, s2);
                }
                const float sc = exp_diff(Lp.vsh, U);
                s1 *= sc;
                s2 *= sc;
            }
            else
            {
                // panels of exactly kPanel (kFall above the zone) from U, the
                // last one the remainder: e^{(u - u_c)} at the nodes of a full
                // panel is a table, correctly rounded
                const bool fall = mid > Lp.z2;
                const float hn  = fall ? kFall : kPanel;
                float E[8];
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    E[i] = fall ? kE3[i] : kE2[i];
                float hw = 0.5f * hn;
                df pu    = U;
#pragma unroll 1
                while (true)
                {
                    const float rem = dsub(V, pu);
                    if (!(rem > 0.f))
                        break;
                    const bool last = rem < hn;
                    if (last)
                    {
                        hw = 0.5f * rem;
#pragma unroll
                        for (int i = 0; i < 4; ++i)
                        {
                            const df x     = two_prod(hw, kG8t[i]);
                            const float ep = expf(x.hi);
                            E[2 * i]       = fmaf(ep, x.lo, ep);
                            E[2 * i + 1]   = rcp_nr(E[2 * i]);
                        }
                    }
                    const df CM    = add(pu, hw);
                    const float ec = exp_diff(CM, Lp.vsh); // e^v at the panel centre
                    const float tc = dsub(CM, P), rc = dsub(Q, CM);
                    const float tcL = fmaf(tc, iLh, tc * iLl), rcL = fmaf(rc, iLh, rc * iLl);
                    const float hwL = fmaf(hw, iLh, hw * iLl);
                    float p1 = 0.f, p2 = 0.f;
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                    {
                        const float tq = (i & 1) ? -kG8t[i >> 1] : kG8t[i >> 1];
                        const float ph = kG8w[i >> 1] * rcpa(fmaf(ec, E[i], Lp.A));
                        float k1, k2;
                        bern2(g1, g2, fmaf(tq, hwL, tcL), fmaf(-tq, hwL, rcL), k1, k2);
                        p1 = fmaf(ph, k1, p1);
                        p2 = fmaf(ph, k2, p2);
                    }
                    s1 = fmaf(hw, p1, s1);
                    s2 = fmaf(hw, p2, s2);
                    if (last)
                        break;
                    pu = add(pu, hn);
                }
            }
            A1 = add(A1, s1);
            A2 = add(A2, s2);
            U  = V;
            if (j == 2)
                break;
        }
    }
    // [x, inf): K = A + B (u - x), in closed form
    {
        const float m = G.m, e = G.e, em = e + m;
        float a1, a2, bb;
        if (G.dgy)
        {
            const float c = m * m * m * em;
            a1 = c * fmaf(6.f, e, 11.f * m);
            a2 = c * fmaf(2.f, e, 5.f * m);
            bb = 4.f * c;
        }
        else
        {
            const float c = m * em * em * em;
            a1 = c * fmaf(5.f, e, 11.f * m);
            a2 = c * fmaf(3.f, e, 5.f * m);
            bb = 4.f * c;
        }
        float f0, f1;
        fermi01_scaled(dsub(Lp.eta, G.X), exp_diff(Lp.vsh, G.X), Lp.iA, f0, f1);
        A1 = add(A1, fmaf(a1, f0, bb * f1));
        A2 = add(A2, fmaf(a2, f0, bb * f1));
    }
    I1 = A1.hi + A1.lo;
    I2 = A2.hi + A2.lo;
}

// One lepton at given (w, w', eta) (the test entry): I_l = e^{lref} Ihat_l.
__device__ __noinline__ void lepton_integrals(double w, double wp, double eta, float& I1,
                                              float& I2, double& lref)
{
    const Geo G      = make_geo(w, wp);
    const Lepton Lp  = make_lepton(eta);
    lepton_integrals(G, Lp, I1, I2);
    lref = eta < 0. ? eta : 0.;
}

} // namespace nes32
} // namespace bnsn
