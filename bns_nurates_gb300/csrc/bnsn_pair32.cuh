// e+e- pair kernel of the mixed path as a cancellation-free FP32 integral.
//
// The reference's Psi_0(y, z) (kernel_pair.hpp:16-120) is a combination of
// Fermi integrals F_1..F_5 at eta, eta +- y, eta +- z, eta +- (y + z) with
// polynomial coefficients, divided by 15 y^2 z^2.  Writing each
// F_k(eta + c) = int_{-c}^inf (u + c)^k f(u - eta) du  (f(t) = 1/(1 + e^t))
// turns the combination into  int K(u) f(u - eta) du  with a piecewise
// polynomial K supported on [-s, s], s = y + z (the pieces beyond s sum to
// zero identically), and K(u - s) = -K(u) on [0, s].  With
// f(a) - f(a - s) = (1 - e^s) f(a) f(s - a) this gives
//
//   Psi_0(y, z) / (1 - e^s) = J_0 = 1/(15 y^2 z^2) int_0^s H_0(x) g(x) dx,
//   g(x) = f(x - eta) f(eta + s - x)   (the e- and e+ occupations),
//
// with H_0 >= 0 a quintic on each of [0, a], [a, b], [b, s]
// (a = min(y, z), b = max(y, z)), and Psi_0(z, y) the same with H_1 = H_0
// with y and z exchanged.  The integrand is positive: no cancellation, so
// FP32 suffices, whereas the reference formula cancels catastrophically
// (its FP64 value is rounding noise once eta - s exceeds ~35, which is why
// the reference zeroes it for eta - s > 200).  Checked against 90-digit and
// higher evaluations of the reference formula on 320 cells: at most 4.1e-7
// relative per cell, median 9e-8.
//
// Quadrature.  ln g is concave with slope in [-1, 1]: it rises like x - eta
// below the e- Fermi edge at x = eta, is flat up to the e+ edge at
// x = eta + s and falls beyond.  Each polynomial piece is cut at
// eta +- E and eta + s +- E (E = 16):
//   edge zones        Gauss-Legendre, 8 nodes on panels of width <= 4
//                     (f has poles at distance pi from the real axis)
//   plateau           g = 1 to 1e-7: 3-node Gauss-Legendre, exact for quintics
//   rising / falling  g = e^{+-(x - edge)}: 3-node Gauss-Laguerre from the
//                     segment's upper end minus e^{-(length)} times the same
//                     from its lower end, exact for quintic x exponential;
//                     segments shorter than 4 go to the edge rule
// Everything is scaled by e^{-Lref}, Lref = max over [0, s] of the linear
// part of ln g + s (so the integrand's largest value is O(1) in FP32); the
// linear part of each node's exponent is formed from per-panel constants
// relative to that maximum (exact where it matters), the edge corrections
// ln(1 + e^{-|d|}) from the node's own distances.

#pragma once

#include "bnsn_constants.h"
#include "bnsn_df.cuh"

namespace bnsn {
namespace pair32 {

constexpr float kEdge  = 16.f; // half-width of the Fermi-edge zones
constexpr float kPanel = 4.f;  // widest Gauss-Legendre panel in an edge zone
constexpr float kRamp  = 4.f;  // shortest segment taken by the Laguerre rule

// Gauss-Legendre on [-1, 1]: 8 nodes (+-t, weight w) and 3 nodes.
__device__ __constant__ const float kG8t[4] = {0.18343464249564978f, 0.525532409916329f,
                                               0.7966664774136267f, 0.9602898564975362f};
__device__ __constant__ const float kG8w[4] = {0.36268378337836166f, 0.3137066458778869f,
                                               0.22238103445337443f, 0.10122853629037706f};
constexpr float kG3t = 0.7745966692414834f, kG3w0 = 0.8888888888888888f,
                kG3w1 = 0.5555555555555556f;
// Gauss-Laguerre, 3 nodes: int_0^inf P(t) e^{-t} dt, exact for deg P <= 5.
__device__ __constant__ const float kLagT[3] = {0.4157745567834791f, 2.294280360279042f,
                                                6.2899450829374794f};
__device__ __constant__ const float kLagW[3] = {0.7110930099291729f, 0.278517733569241f,
                                                0.010389256501586133f};

// One cell (y = omega / T, z = omega' / T) at eta = mu_e / T.  Positions
// that enter an exponent or a polynomial's local coordinate are kept as
// double-float pairs: in FP32 alone, y ~ 20 carries an absolute rounding
// error ~1e-6, which e^{+-x} factors turn into a relative error of the cell.
struct Cell
{
    float y, z;          // polynomial coefficients (relative accuracy suffices)
    bool ylz;            // y < z
    dfm::df A, B, S;     // piece ends a = min(y, z), b = max(y, z), s = y + z
    dfm::df ETA, ES;     // eta, eta + s
    dfm::df R1, R2;      // eta + Lref and eta + s - Lref
    float e1, e2, e3, e4; // zone cuts eta - E, eta + E, eta + s - E, eta + s + E
    float k00;           // -Lref
};

// a - b of two double-float values, rounded to FP32 (exact where a ~ b).
__device__ __forceinline__ float dsub(dfm::df a, dfm::df b)
{
    return (a.hi - b.hi) + (a.lo - b.lo);
}

// H_0 and H_1 on piece k at a node: x the node, r = (right end of the
// piece) - x.  Every form is a sum of positive terms or positive definite.
__device__ __forceinline__ void hpair(int k, const Cell& c, float x, float r, float& h0,
                                      float& h1)
{
    if (k == 0)
    {
        const float x3 = 4.f * x * x * x;
        h0 = x3 * fmaf(x, x - 5.f * c.z, 10.f * c.z * c.z);
        h1 = x3 * fmaf(x, x - 5.f * c.y, 10.f * c.y * c.y);
    }
    else if (k == 1)
    {
        const float m  = c.ylz ? c.y : c.z;
        const float m3 = 4.f * m * m * m;
        const float hs = m3 * fmaf(r, fmaf(10.f, r, 15.f * m), 6.f * m * m); // 10r^2+15rm+6m^2
        const float hb = m3 * fmaf(x, fmaf(10.f, x, -5.f * m), m * m);       // 10x^2-5xm+m^2
        h0 = c.ylz ? hs : hb;
        h1 = c.ylz ? hb : hs;
    }
    else
    {
        const float t3 = 4.f * r * r * r;
        h0 = t3 * fmaf(r, r - 5.f * c.y, 10.f * c.y * c.y);
        h1 = t3 * fmaf(r, r - 5.f * c.z, 10.f * c.z * c.z);
    }
}

// Edge-zone panel [pu, pv] of piece k (right end Q): 8 Gauss-Legendre nodes
// with the full occupation factor.
__device__ __forceinline__ void edge_panel(int k, const Cell& c, dfm::df pu, dfm::df pv,
                                           dfm::df Q, float& q0, float& q1)
{
    const float hw  = 0.5f * dsub(pv, pu);
    const dfm::df CM = dfm::add(pu, hw);     // panel centre
    const float b1  = dsub(CM, c.ETA);       // node distance to the e- edge: b1 + ht
    const float b2  = dsub(CM, c.ES);        // to the e+ edge
    const float k10 = dsub(CM, c.R1);        // linear exponent below the e- edge
    const float k01 = dsub(c.R2, CM);        // beyond the e+ edge
    const float rq  = dsub(Q, CM);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i)
    {
        const float t  = (i & 1) ? -kG8t[i >> 1] : kG8t[i >> 1];
        const float ht = hw * t;
        const float d1 = b1 + ht, d2 = b2 + ht;
        const bool n1 = d1 < 0.f, p2 = d2 > 0.f;
        const float arg = n1 ? k10 + ht : (p2 ? k01 - ht : c.k00);
        const float corr = (1.f + __expf(-fabsf(d1))) * (1.f + __expf(-fabsf(d2)));
        float rc;  // 1 / corr, corr in [1, 4]: approximate reciprocal (1 ulp)
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rc) : "f"(corr));
        const float gh = __expf(arg) * rc;
        float h0, h1;
        hpair(k, c, CM.hi + ht, rq - ht, h0, h1);
        const float w = kG8w[i >> 1] * gh;
        s0 = fmaf(w, h0, s0);
        s1 = fmaf(w, h1, s1);
    }
    q0 = hw * s0;
    q1 = hw * s1;
}

// int_0^s H_l g e^{s - Lref} dx for l = 0, 1 (segment sums accumulated in
// double-float).
__device__ __forceinline__ void cell_integrals(const Cell& c, double& Q0, double& Q1)
{
    dfm::df A0 = dfm::mk(0.f), A1 = dfm::mk(0.f);
    // zone cuts in increasing order (e1 < e2, e3 < e4; e2 vs e3 depends on s)
    const float zc[4] = {c.e1, fminf(c.e2, c.e3), fmaxf(c.e2, c.e3), c.e4};
#pragma unroll 1
    for (int k = 0; k < 3; ++k)
    {
        const dfm::df P = k == 0 ? dfm::mk(0.f) : (k == 1 ? c.A : c.B);
        const dfm::df Q = k == 0 ? c.A : (k == 1 ? c.B : c.S);
        if (!(dsub(Q, P) > 0.f))
            continue;
        dfm::df U = P;
#pragma unroll 1
        for (int j = 0; j <= 4; ++j)
        {
            dfm::df V = Q;
            if (j < 4)
            {
                if (!(zc[j] > U.hi && zc[j] < Q.hi))
                    continue;
                V = dfm::mk(zc[j]);
            }
            // segment [U, V]
            const float len = dsub(V, U);
            const float mid = U.hi + 0.5f * len;
            const float d1m = mid - c.ETA.hi, d2m = d1m - c.S.hi;
            float q0 = 0.f, q1 = 0.f;
            if (d1m < -kEdge && len >= kRamp)
            {
                // rising: e^{x - eta - Lref}; Laguerre from V down, minus from U down
                const float rv = dsub(Q, V), ru = dsub(Q, U);
                float lv0 = 0.f, lv1 = 0.f, lu0 = 0.f, lu1 = 0.f;
#pragma unroll
                for (int i = 0; i < 3; ++i)
                {
                    float h0, h1;
                    hpair(k, c, V.hi - kLagT[i], rv + kLagT[i], h0, h1);
                    lv0 = fmaf(kLagW[i], h0, lv0);
                    lv1 = fmaf(kLagW[i], h1, lv1);
                    hpair(k, c, U.hi - kLagT[i], ru + kLagT[i], h0, h1);
                    lu0 = fmaf(kLagW[i], h0, lu0);
                    lu1 = fmaf(kLagW[i], h1, lu1);
                }
                const float sc = expf(dsub(V, c.R1));
                const float ed = expf(-len);
                q0 = sc * fmaf(-ed, lu0, lv0);
                q1 = sc * fmaf(-ed, lu1, lv1);
            }
            else if (d2m > kEdge && len >= kRamp)
            {
                // falling: e^{eta + s - Lref - x}; Laguerre from U up, minus from V up
                const float rv = dsub(Q, V), ru = dsub(Q, U);
                float lu0 = 0.f, lu1 = 0.f, lv0 = 0.f, lv1 = 0.f;
#pragma unroll
                for (int i = 0; i < 3; ++i)
                {
                    float h0, h1;
                    hpair(k, c, U.hi + kLagT[i], ru - kLagT[i], h0, h1);
                    lu0 = fmaf(kLagW[i], h0, lu0);
                    lu1 = fmaf(kLagW[i], h1, lu1);
                    hpair(k, c, V.hi + kLagT[i], rv - kLagT[i], h0, h1);
                    lv0 = fmaf(kLagW[i], h0, lv0);
                    lv1 = fmaf(kLagW[i], h1, lv1);
                }
                const float sc = expf(dsub(c.R2, U));
                const float ed = expf(-len);
                q0 = sc * fmaf(-ed, lv0, lu0);
                q1 = sc * fmaf(-ed, lv1, lu1);
            }
            else if (d1m > kEdge && d2m < -kEdge)
            {
                // plateau (Lref = 0 there): the quintic exactly
                const float hw = 0.5f * len;
                const dfm::df CM = dfm::add(U, hw);
                const float rq = dsub(Q, CM);
                float h0, h1, s0, s1;
                hpair(k, c, CM.hi, rq, h0, h1);
                s0 = kG3w0 * h0;
                s1 = kG3w0 * h1;
                hpair(k, c, CM.hi + hw * kG3t, rq - hw * kG3t, h0, h1);
                s0 = fmaf(kG3w1, h0, s0);
                s1 = fmaf(kG3w1, h1, s1);
                hpair(k, c, CM.hi - hw * kG3t, rq + hw * kG3t, h0, h1);
                s0 = fmaf(kG3w1, h0, s0);
                s1 = fmaf(kG3w1, h1, s1);
                q0 = hw * s0 * __expf(c.k00);
                q1 = hw * s1 * __expf(c.k00);
            }
            else
            {
                const int npan = max(1, (int)ceilf(len * (1.f / kPanel)));
                const float h  = len / (float)npan;
                dfm::df pu     = U;
#pragma unroll 1
                for (int pn = 0; pn < npan; ++pn)
                {
                    const dfm::df pv = pn == npan - 1 ? V : dfm::add(U, (float)(pn + 1) * h);
                    float a0, a1;
                    edge_panel(k, c, pu, pv, Q, a0, a1);
                    q0 += a0;
                    q1 += a1;
                    pu = pv;
                }
            }
            A0 = dfm::add(A0, q0);
            A1 = dfm::add(A1, q1);
            U = V;
            if (j == 4)
                break;
        }
    }
    Q0 = dfm::to_double(A0);
    Q1 = dfm::to_double(A1);
}

// Which reference Lref the cell uses: Lref = s - eta (eta >= s), eta + s
// (eta <= -s) or 0.
enum LrefCase
{
    kLrefZero = 0,
    kLrefAbove, // eta >= s
    kLrefBelow  // eta <= -s
};

// The cell's set-up from double-float y, z (nodes) and eta.  Returns false
// when the reference zeroes Psi (eta - y - z > 200, kernel_pair.hpp:40-44);
// lcase receives the Lref case, whose factor e^{Lref} the caller forms.
__device__ __forceinline__ bool make_cell(dfm::df Y, dfm::df Z, dfm::df ETA, Cell& c,
                                          int& lcase)
{
    using namespace dfm;
    const df S = add(Y, Z);
    if (dsub(ETA, S) > 200.f)
        return false;
    const float es = dsub(ETA, S), emns = (ETA.hi + S.hi) + (ETA.lo + S.lo);
    lcase = es >= 0.f ? kLrefAbove : (emns <= 0.f ? kLrefBelow : kLrefZero);
    c.y   = Y.hi;
    c.z   = Z.hi;
    c.ylz = dsub(Y, Z) < 0.f;
    c.A   = c.ylz ? Y : Z;
    c.B   = c.ylz ? Z : Y;
    c.S   = S;
    c.ETA = ETA;
    c.ES  = add(ETA, S);
    // R1 = eta + Lref, R2 = eta + s - Lref
    c.R1  = lcase == kLrefAbove ? S : (lcase == kLrefBelow ? add(add(ETA, ETA), S) : ETA);
    c.R2  = lcase == kLrefAbove ? add(ETA, ETA) : (lcase == kLrefBelow ? mk(0.f) : c.ES);
    c.k00 = lcase == kLrefAbove ? es : (lcase == kLrefBelow ? -emns : 0.f); // -Lref
    c.e1  = ETA.hi - kEdge;
    c.e2  = ETA.hi + kEdge;
    c.e3  = c.ES.hi - kEdge;
    c.e4  = c.ES.hi + kEdge;
    return true;
}

// Set-up from FP64 values (the unit-test entry point): lref receives Lref.
__device__ __forceinline__ bool make_cell(double y, double z, double eta, Cell& c,
                                          double& lref)
{
    int lcase;
    if (!make_cell(dfm::from_double(y), dfm::from_double(z), dfm::from_double(eta), c, lcase))
        return false;
    const double s = y + z;
    lref = lcase == kLrefAbove ? s - eta : (lcase == kLrefBelow ? eta + s : 0.);
    return true;
}

// The pair kernel of one cell for the four species: em and ab of
// kernel_pair.hpp:135-198 times (nu nubar)^2, from the FP32 integral:
// ab = (Phi T^2 / 2) alpha . (Psi / (1 - e^s)) e^{s}, em = ab / SafeExp(s).
// Y, Z: nu / T and nubar / T as double-float; eh = e^{y - |eta| / 2} and
// dn = e^{-y} of each side (e^{Lref} = eh_y eh_z where Lref != 0, e^{-s} =
// dn_y dn_z for s <= 700); sc = (Phi T^2 / 2) T^4 / 15, the point's factor.
__device__ __forceinline__ void kernel_q(dfm::df Y, dfm::df Z, double ehy, double ehz,
                                         double dny, double dnz, dfm::df ETA, double sc,
                                         double* em, double* ab)
{
    Cell c;
    int lcase;
    if (!make_cell(Y, Z, ETA, c, lcase))
    {
#pragma unroll
        for (int q = 0; q < 4; ++q)
            em[q] = ab[q] = 0.;
        return;
    }
    double Q0, Q1;
    cell_integrals(c, Q0, Q1);
    const double f = lcase == kLrefZero ? sc : sc * (ehy * ehz);
    ab[0] = f * ((k::PairA1e * k::PairA1e) * Q0 + (k::PairA2e * k::PairA2e) * Q1);
    ab[1] = f * ((k::PairA1e * k::PairA1e) * Q1 + (k::PairA2e * k::PairA2e) * Q0);
    ab[2] = f * ((k::PairA1x * k::PairA1x) * Q0 + (k::PairA2x * k::PairA2x) * Q1);
    ab[3] = f * ((k::PairA1x * k::PairA1x) * Q1 + (k::PairA2x * k::PairA2x) * Q0);
    const double ems = c.S.hi <= 700.f ? dny * dnz : 9.8596765437597708e-305; // e^-700
#pragma unroll
    for (int q = 0; q < 4; ++q)
        em[q] = ab[q] * ems;
}

} // namespace pair32
} // namespace bnsn
