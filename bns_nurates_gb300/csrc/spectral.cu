// Spectral opacity kernels (sm_103a), FP64 and mixed precision.
//
// Restates ComputeSpectralOpacities{NotStimulatedAbs,StimulatedAbs} and
// SpectralIntegrand (m1_opacities.hpp:1317-1660).
//
// Phases per chunk of points, each a persistent launch with one warp per
// point (the phase split keeps every kernel's code small enough for the
// instruction cache; a single fused kernel spent most cycles waiting on
// instruction fetch):
//   prelude   NuDistributionParams of each point -> chunk scratch;
//   pb        pair + brem sums of every (point, energy) -> records;
//   nes       NES/NPS sums -> records;
//   assemble  beta, iso, the outer factors and the stimulated-absorption
//             correction -> the caller's outputs.
// In pb and nes the antineutrino grid of the integral (t x_i, t / x_i with
// t = 2.182 T for pair/brem, nu x_i, nu / x_i for NES) is staged per point
// and per energy in shared memory; lanes take (energy, node group) tasks with
// groups of G consecutive lanes per energy (G a power of two) and combine the
// group sums with an xor-shuffle inside each segment.  Each integrand is
// evaluated once per node; the reference evaluates the full integrand once
// per (output, node) (integration.hpp:524-543), which only repeats identical
// values.
//
// MIXED: pb evaluates the pair kernel as the cancellation-free FP32 integral
// of the grey path (bnsn_pair32.cuh) and the brem kernel in FP32 (HR98
// shape, GP19 profiles) with the factor e^{-nu/T} of the emissivity applied
// in FP64 (BRT06 and the GP19 high-T extrapolation stay FP64), and nes uses
// double-float Fermi integrals and brackets with FP32 occupation factors
// formed as exponentials of double-float arguments minus a per-energy scale
// (nes_spec_node), so that e^{-(w - w')} g(w') stays in range at any nu/T;
// per-point data stay FP64 and every term is summed in FP64.  Both record an
// error bound per output: the FP32 rounding bound (sum|t| over 1.25 for
// brem, over 2.5 for the pair integrals, over 2 for NES) plus 1e9 x the
// components dropped below 2^-120.
// assemble compares the bounds with each output's total.  Where their sum
// exceeds it (terms that cancel), or where a part could not run in FP32
// (bound = inf: occupations outside the FP32 range, NES at nu/T < 0.05 where
// the brackets lose double-float accuracy), it flags the part whose bound
// exceeds half the total.  Flagged pair + brem parts are recomputed in FP64,
// flagged NES parts with every product in double-float (sum|t| up to 1e5
// |total|); assemble checks again with the remaining bounds and flags what
// is left, and an FP64 round finishes those.  The FP64 passes pack each
// point's flagged energies into full rounds.

#include <cuda_runtime.h>

#include "bnsn_df.cuh"
#include "bnsn_fp32.cuh"
#include "bnsn_fp64.cuh"
#include "bnsn_internal.h"
#include "bnsn_mixed.cuh"
#include "bnsn_pair32.cuh"

namespace bnsn {
namespace {

using namespace fp64;

constexpr int kWarps  = 4;
constexpr int kEChunk = 32; // energies staged per pass

constexpr double kSpecCancelBrem = 1.25;    // sum|t| / |total| of the FP32 brem terms
// same for the FP32 pair integrals: their terms are positive with at most
// 4.1e-7 relative error per cell (bnsn_pair32.cuh), so sum|t| / 2.5 is 1e6 x
// a bound on the error of their sum, the scale of the other bounds
constexpr double kSpecCancelPair = 2.5;
constexpr double kSpecCancelNes  = 2.0;     // same for the NES/NPS terms
constexpr double kSpecCancelDf   = 1e5;     // same for the double-float NES pass
constexpr double kSpecNesMinW    = 0.05;    // NES in FP64 below nu/T = 0.05
constexpr double kSpecFloor      = 7.2e-34; // 1e9 x the denormal floor of a sum

// Per (point, energy) record of the chunk scratch.
struct EnergyRec
{
    double pb[8];   // pair + brem: sum over nodes of w nubar^2 kernel x occupation
    double nes[8];  // NES/NPS: the same
    double bpb[8];  // mixed: error bound of pb[] (inf: recompute in FP64)
    double bnes[8]; // mixed: error bound of nes[]
};

// Kernel modes.
enum SpecMode
{
    kSpecFp64 = 0, // plain path: every energy in FP64
    kSpecMixed,    // mixed path, first pass over every energy
    kSpecRedo,     // FP64 over the flagged energies; assemble re-checks and flags again
    kSpecFinal,    // assemble only: the energies flagged twice, no guard
    kSpecAcc       // nes only: double-float products over the flagged energies
};

// Mixed-path statistics: [0] (point, energy) pairs evaluated, [1] of those
// recomputed in FP64 in any part, [2] pair + brem recomputations, [3] NES
// recomputations.
__device__ unsigned long long g_spec_counts[4];

// (point, energy) pairs whose outputs hold a NaN or Inf.
__device__ unsigned long long g_spec_nonfinite;

// Lane group size for ne energy tasks of M nodes each (power of two <= 32)
// minimising rounds x nodes per task.
__host__ __device__ inline int pick_groups(int ne, int M)
{
    int best       = 1;
    long best_cost = -1;
    for (int G = 1; G <= 32 && G <= M; G <<= 1)
    {
        const int per_round = 32 / G;
        const long rounds   = (ne + per_round - 1) / per_round;
        const long cost     = rounds * ((M + G - 1) / G);
        if (best_cost < 0 || cost < best_cost)
        {
            best_cost = cost;
            best      = G;
        }
    }
    return best;
}

__device__ __forceinline__ double seg_sum(double v, int G)
{
    for (int o = 1; o < G; o <<= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float seg_sum(float v, int G)
{
    for (int o = 1; o < G; o <<= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// kq-th set bit of m (0-based).
__device__ __forceinline__ int nth_bit(uint64_t m, int kq)
{
    for (int j = 0; j < kq && j < 64; ++j)
        m &= m - 1ull;
    return __ffsll((long long)m) - 1;
}

// Distribution of a point from the chunk scratch into shared memory.
__device__ __forceinline__ void load_distr(const double* dsc, int64_t q, Distr* d, int lane)
{
    if (lane < 28)
        (&d->w_t[0])[lane] = dsc[q * 28 + lane];
}

__device__ __forceinline__ bool same_cf_of(const Distr& d)
{
    const double c0 = d.c_f[0];
    return (d.c_f[1] == c0) && (d.c_f[2] == c0) && (d.c_f[3] == c0);
}

// Occupations of every species at their peaks far inside the FP32 range.
__device__ __forceinline__ bool fp32_envelope(const Distr& d, double eta_e)
{
    bool env = isfinite(eta_e);
#pragma unroll
    for (int s = 0; s < 4; ++s)
        env = env && (d.w_t[s] == 0. || d.eta_t[s] > -60.) &&
              (d.w_f[s] == 0. || d.beta_f[s] > 1e-30) && (d.temp_t[s] > 0.) &&
              (d.temp_f[s] > 0.) && isfinite(d.eta_t[s]) && isfinite(d.beta_f[s]);
    return env;
}

__device__ __forceinline__ uint64_t all_energies(int ne)
{
    return ne >= 64 ? ~0ull : ((1ull << ne) - 1ull);
}

// Energies of point q that a pb/nes pass works on (bit e: energy e of the launch).
__device__ __forceinline__ uint64_t energy_mask(int mode, const uint64_t* flags, int64_t q, int ne)
{
    return (mode == kSpecRedo || mode == kSpecAcc) ? flags[q] & all_energies(ne)
                                                   : all_energies(ne);
}

// ---------------------------------------------------------------------------
// prelude: NuDistributionParams per point (distribution.hpp:51-243)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128)
    spec_prelude_kernel(const __grid_constant__ OpacityLaunch L, int64_t p0, int64_t np,
                        double* __restrict__ dsc)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= np * 4)
        return;
    const int64_t q = t >> 2;
    const int s     = (int)(t & 3);
    const int64_t p = p0 + q;
    double* d       = dsc + q * 28;
    if (L.has_distr)
    {
        for (int k = 0; k < 7; ++k)
            d[k * 4 + s] = L.distr[k * 4 + s][p];
        return;
    }
    distr_species(L.m1[s][p], L.m1[4 + s][p], L.m1[8 + s][p], L.gamma36, &d[s], &d[4 + s],
                  &d[8 + s], &d[12 + s], &d[16 + s], &d[20 + s], &d[24 + s]);
}

// ---------------------------------------------------------------------------
// pb: pair annihilation + NN bremsstrahlung
// ---------------------------------------------------------------------------
struct PbWarp
{
    Distr d;
    double fe3, fe4; // F_3, F_4 at eta_e
    Hr98Point hr;
    double brt06_pre;
    int same_cf;
    double nb[kMaxM], zb[kMaxM]; // nubar and nubar / T
    double gb[kMaxM][4];
    double fmz[kMaxM][5], fpz[kMaxM][5];
    double fmy[kEChunk][5], fpy[kEChunk][5];
    Gp19Point gp;
    Gp19Corners gc[2];
    double gpp[2][kGp19MaxW];
};

struct PbWarpMixed
{
    fp32::Hr98Mixed hm;
    float yeh[kEChunk], yel[kEChunk]; // nu / T as hi + lo
    float ybh[kMaxM], ybl[kMaxM];     // nubar / T as hi + lo
    double ehy[kEChunk], dny[kEChunk]; // pair: e^{y - |eta|/2}, e^{-y} of the energies
    double ehz[kMaxM], dnz[kMaxM];     // the same of the nodes
    float gb32[kMaxM][4], gbm32[kMaxM][4];
    float gp32[2][kGp19MaxW];
};

template <int MODE>
struct PbShared
{
    double x[kMaxQ], B1[kMaxM];
    dfm::df B1d[kMaxM]; // mixed: weights as double-float
    double lw[kGp19MaxW], wax[kGp19MaxW], iw[kGp19MaxW];
    float lwf[kGp19MaxW], idl[kGp19MaxW];
    PbWarp w[kWarps];
    PbWarpMixed m[MODE == kSpecMixed ? kWarps : 1];
};

// GP19 kernel of one node from the per-point profiles in FP64.
__device__ __forceinline__ void gp19_profile_node(const Gp19Point& gp,
                                                  const double (*gpp)[kGp19MaxW],
                                                  const double* lw, int d3, double wmin,
                                                  double wmax, double nu, double nub, double* be,
                                                  double* ba)
{
    double w = nu + nub;
    w        = w > wmax ? wmax : (w < wmin ? wmin : w);
    double tw;
    const int l     = bracket_sorted<double>(log(w), lw, d3, &tw);
    const double v0 = gpp[0][l] * (1. - tw) + gpp[0][l + 1] * tw;
    const double v1 = gp.regime >= 2 ? gpp[1][l] * (1. - tw) + gpp[1][l + 1] * tw : 0.;
    gp19_cell(gp, v0, v1, w, nu + nub, be, ba);
}

template <int MODE>
__global__ void __launch_bounds__(kWarps * 32)
    spec_pb_kernel(const __grid_constant__ OpacityLaunch L, int64_t p0, int64_t np,
                   const double* __restrict__ dsc, EnergyRec* __restrict__ rec,
                   const uint64_t* __restrict__ flags, int G)
{
    constexpr bool MIX = MODE == kSpecMixed;
    extern __shared__ __align__(16) unsigned char s_raw[];
    PbShared<MODE>& S   = *reinterpret_cast<PbShared<MODE>*>(s_raw);
    const Gp19Table G19 = {L.gp19.d0, L.gp19.d1, L.gp19.d2, L.gp19.d3, L.gp19.nb,
                           L.gp19.ye, L.gp19.t,  L.gp19.w,  L.gp19.lognb,
                           L.gp19.logw, L.gp19.data};
    const bool prof   = L.use_brem && L.brem_impl == 2 && G19.d3 <= kGp19MaxW;
    const double wmin = prof ? G19.w[0] : 0., wmax = prof ? G19.w[G19.d3 - 1] : 0.;
    for (int k = threadIdx.x; k < kMaxQ; k += blockDim.x)
        S.x[k] = L.x1[k];
    for (int k = threadIdx.x; k < kMaxM; k += blockDim.x)
    {
        S.B1[k]  = L.B1[k];
        S.B1d[k] = dfm::from_double(L.B1[k]);
    }
    if (prof)
        for (int k = threadIdx.x; k < G19.d3; k += blockDim.x)
        {
            S.lw[k]  = G19.logw[k];
            S.lwf[k] = (float)G19.logw[k];
            S.wax[k] = G19.w[k];
            S.iw[k]  = 1. / G19.w[k];
            S.idl[k] = k + 1 < G19.d3 ? (float)(1. / (G19.logw[k + 1] - G19.logw[k])) : 0.f;
        }
    __syncthreads();

    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    PbWarp& W      = S.w[wid];
    PbWarpMixed& X = S.m[MIX ? wid : 0];
    const int n = L.n1, M = 2 * n, ne = L.n_energies;
    const bool nbb      = L.neglect_blocking != 0;
    const int64_t nwarp = (int64_t)gridDim.x * kWarps;

    for (int64_t q = (int64_t)blockIdx.x * kWarps + wid; q < np; q += nwarp)
    {
        const uint64_t emask = energy_mask(MODE, flags, q, ne);
        if (emask == 0ull)
            continue;
        // the redo passes pack this point's flagged energies into full rounds
        const int Gq        = MODE == kSpecRedo ? pick_groups(__popcll(emask), M) : G;
        const int grp       = lane % Gq;
        const int per_round = 32 / Gq;
        const int64_t p     = p0 + q;
        const double nbar = L.eos[0][p], T = L.eos[1][p], ye = L.eos[2][p];
        const double yp = L.eos[3][p], yn = L.eos[4][p], mu_e = L.eos[7][p];
        const double eta_e = mu_e / T;
        EnergyRec* R       = rec + q * ne;
        __syncwarp();
        load_distr(dsc, q, &W.d, lane);
        if (lane == 28 && L.use_pair)
        {
            double f[2];
            fdi_orders<3, 4>(eta_e, f);
            W.fe3 = f[0];
            W.fe4 = f[1];
        }
        if (L.use_brem && L.brem_impl == 0)
        {
            if (lane >= 6 && lane < 9)
                W.hr.ch[lane - 6] = hr98_channel(nbar, yn, yp, T, lane - 6);
            if (lane == 29)
                hr98_point_common(nbar, T, L.use_medium != 0, &W.hr);
        }
        if (lane == 30 && L.use_brem && L.brem_impl == 1)
            W.brt06_pre = brt06_point(nbar, T, yn, yp);
        if (lane == 31 && prof)
            gp19_point(G19, nbar, ye, T, &W.gp);
        __syncwarp();
        if (lane == 0)
        {
            W.same_cf = same_cf_of(W.d);
            if (MIX && L.use_brem && L.brem_impl == 0)
                fp32::hr98_mixed_from(W.hr, &X.hm);
        }
        if (prof)
        {
            const int np19 = (W.gp.regime >= 2) ? 2 : 1;
            if (lane < np19)
                gp19_profile_corners(G19, W.gp.nbp, W.gp.yep, W.gp.pT[lane], &W.gc[lane]);
            __syncwarp();
            for (int e = lane; e < np19 * G19.d3; e += 32)
            {
                const int pr = e / G19.d3, l = e - pr * G19.d3;
                const double v = gp19_profile_eval(G19, W.gc[pr], l);
                W.gpp[pr][l] = v;
                if (MIX)
                    X.gp32[pr][l] = (float)v;
            }
        }
        __syncwarp();
        const bool same_cf = W.same_cf != 0;
        // mixed pair: eta and the point's factor (Phi T^2 / 2) T^4 / 15
        const dfm::df ETA = dfm::from_double(eta_e);
        const double T2   = T * T;
        const double scq  = 0.5 * k::PairPhi * T2 * (T2 * T2) / 15.;
        // antineutrino grid of the pair/brem integral (m1_opacities.hpp:1542)
        const double ts = k::TempMultiple * T;
        for (int a = lane; a < M; a += 32)
        {
            const int i     = a < n ? a : a - n;
            const double nu = a < n ? ts * S.x[i] : ts / S.x[i];
            W.nb[a]         = nu;
            W.zb[a]         = nu / T;
            total_nu_f4(nu, W.d, same_cf, W.gb[a]);
            if (MIX)
            {
                const dfm::df yd = dfm::from_double(nu / T);
                X.ybh[a] = yd.hi;
                X.ybl[a] = yd.lo;
                if (L.use_pair)
                {
                    X.ehz[a] = exp(W.zb[a] - 0.5 * fabs(eta_e));
                    X.dnz[a] = exp(-W.zb[a]);
                }
#pragma unroll
                for (int s = 0; s < 4; ++s)
                {
                    X.gb32[a][s]  = (float)W.gb[a][s];
                    X.gbm32[a][s] = (float)(1. - W.gb[a][s]);
                }
            }
        }
        // the FP64 pair kernel's Fermi integrals (the mixed pass uses the
        // FP32 integral, bnsn_pair32.cuh)
        if (L.use_pair && !MIX)
            for (int t = lane; t < 2 * M; t += 32)
            {
                const int a    = t >> 1;
                const int i    = a < n ? a : a - n;
                const double z = (a < n ? ts * S.x[i] : ts / S.x[i]) / T;
                if (t & 1)
                    fdi_orders<1, 5>(eta_e + z, W.fpz[a]);
                else
                    fdi_orders<1, 5>(eta_e - z, W.fmz[a]);
            }
        // mixed: FP32 brem for HR98 and the GP19 profiles (not the high-T
        // extrapolation) inside the FP32 range envelope
        bool b32  = false;
        double sb = 0.;
        float thr = 0.f, lt2 = 0.f;
        if (MIX && L.use_brem)
        {
            b32 = (L.brem_impl == 0 || (prof && W.gp.regime != 3 && W.gp.regime != 5)) &&
                  fp32_envelope(W.d, eta_e);
            if (L.brem_impl == 0)
                sb = (T * T) * X.hm.outer;
            else if (prof)
            {
                sb  = (T * T) * (3. * W.gp.C);
                thr = (float)(1e-30 / W.gp.C);
                lt2 = (float)log2(T * 0.5);
            }
        }
        // brem in FP64 here when FP32 does not apply, except the full-table GP19
        // kernel (w axis longer than the profiles hold), left to the FP64 redo
        const bool skip = MIX && L.use_brem && !b32 && L.brem_impl == 2 && !prof;

        for (int e0 = 0; e0 < ne; e0 += kEChunk)
        {
            const int nec     = (ne - e0) < kEChunk ? (ne - e0) : kEChunk;
            const uint32_t cm = (uint32_t)(emask >> e0) &
                                (nec == 32 ? 0xffffffffu : ((1u << nec) - 1u));
            if (cm == 0u)
                continue;
            __syncwarp();
            for (int c = lane; c < nec; c += 32)
            {
                if (!((cm >> c) & 1u))
                    continue;
                const double y = L.energies[e0 + c] / T;
                if (L.use_pair && !skip && !MIX)
                {
                    fdi_orders<1, 5>(eta_e - y, W.fmy[c]);
                    fdi_orders<1, 5>(eta_e + y, W.fpy[c]);
                }
                if (MIX)
                {
                    const dfm::df yd = dfm::from_double(y);
                    X.yeh[c] = yd.hi;
                    X.yel[c] = yd.lo;
                    if (L.use_pair)
                    {
                        X.ehy[c] = exp(y - 0.5 * fabs(eta_e));
                        X.dny[c] = exp(-y);
                    }
                }
            }
            __syncwarp();
            const int nt = __popc(cm);
            for (int r0 = 0; r0 < nt; r0 += per_round)
            {
                const int kq    = r0 + lane / Gq;
                const bool act  = kq < nt;
                const int c     = act ? nth_bit(cm, kq) : 0;
                const double nu = act ? L.energies[e0 + c] : 1.;
                const double w  = nu / T;
                double acc[8];
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                    acc[kk] = 0.;
                float gl[8]; // mixed: sum|t| / 1.25 + 1e9 x dropped
                double gp[8]; // mixed: sum|t| of the FP32 pair terms
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                {
                    gl[kk] = 0.f;
                    gp[kk] = 0.;
                }
                const double sbe = sb * exp(-w); // brem emission carries e^{-nu/T}
                const double inu2 = MIX ? 1. / (nu * nu) : 0.;
                if (act && !skip)
                {
                    for (int a = grp; a < M; a += Gq)
                    {
                        const double wa  = S.B1[a];
                        const double nub = W.nb[a];
                        const double* gb = W.gb[a];
                        double pe[4] = {0., 0., 0., 0.}, pa[4] = {0., 0., 0., 0.};
                        double be = 0., ba = 0.;
                        if (L.use_pair && !MIX)
                            pair_kernel(T, eta_e, nu, nub, w, W.zb[a], W.fmy[c], W.fpy[c],
                                        W.fmz[a], W.fpz[a], W.fe3, W.fe4, pe, pa);
                        if (L.use_brem && !b32)
                        {
                            if (L.brem_impl == 0)
                                hr98_kernel(W.hr, nu, nub, &be, &ba);
                            else if (L.brem_impl == 1)
                                brt06_kernel(W.brt06_pre, T, nu, nub, &be, &ba);
                            else if (prof)
                                gp19_profile_node(W.gp, W.gpp, S.lw, G19.d3, wmin, wmax, nu,
                                                  nub, &be, &ba);
                            else if (!MIX)
                                gp19_kernel(G19, nbar, ye, T, nu, nub, &be, &ba);
                        }
                        const double nb2 = nub * nub;
                        if (!MIX || (L.use_brem && !b32))
                        {
#pragma unroll
                            for (int s = 0; s < 4; ++s)
                            {
                                const int ps    = s ^ 1;
                                const double bf = nbb ? 1. : 1. - gb[ps];
                                acc[s] += wa * (nb2 * ((pe[s] + be) * bf));
                                acc[4 + s] += wa * (nb2 * ((pa[s] + ba) * gb[ps]));
                            }
                        }
                        if (MIX && L.use_pair)
                        {
                            // FP32 pair integral: (em, ab) (nu nubar)^2, positive
                            double qe[4], qa[4];
                            pair32::kernel_q(dfm::df{X.yeh[c], X.yel[c]},
                                             dfm::df{X.ybh[a], X.ybl[a]}, X.ehy[c], X.ehz[a],
                                             X.dny[c], X.dnz[a], ETA, scq, qe, qa);
                            const double wq = wa * inu2;
#pragma unroll
                            for (int s = 0; s < 4; ++s)
                            {
                                const int ps    = s ^ 1;
                                const double bf = nbb ? 1. : 1. - gb[ps];
                                const double te = wq * (qe[s] * bf);
                                const double ta = wq * (qa[s] * gb[ps]);
                                acc[s] += te;
                                acc[4 + s] += ta;
                                gp[s] += fabs(te);
                                gp[4 + s] += fabs(ta);
                            }
                        }
                        if (MIX && b32)
                        {
                            // kernel shape at x = (nu + nubar) / T (hi + lo)
                            const dfm::df xs = dfm::add(dfm::df{X.yeh[c], X.yel[c]},
                                                        dfm::df{X.ybh[a], X.ybl[a]});
                            float kab;
                            bool slow = false;
                            if (L.brem_impl == 0)
                                kab = fp32::hr98_shape(X.hm, xs.hi, xs.lo);
                            else
                            {
                                double wv = nu + nub;
                                wv        = wv > wmax ? wmax : (wv < wmin ? wmin : wv);
                                float tw;
                                const int l = gp19_bracket32(wv, S.lwf, S.wax, S.iw, S.idl,
                                                             G19.d3, &tw);
                                const float v0 =
                                    X.gp32[0][l] + tw * (X.gp32[0][l + 1] - X.gp32[0][l]);
                                if (W.gp.regime <= 1)
                                    kab = v0;
                                else
                                {
                                    const float v1 =
                                        X.gp32[1][l] + tw * (X.gp32[1][l + 1] - X.gp32[1][l]);
                                    kab = v0 * exp2f(log2f(v1 / v0) * lt2);
                                    // regime 2 clips at 1e-30: exact FP64 node
                                    slow = W.gp.regime == 2 &&
                                           (v0 < thr || v1 < thr || kab < thr);
                                }
                                kab = fabsf(kab);
                            }
                            // e^{-nubar/T}; below 2^-120 the term is dropped
                            const bool far = X.ybh[a] > -kNesDropArg;
                            float kem = far ? 0.f : kab * (expf(-X.ybh[a]) * (1.f - X.ybl[a]));
                            if (slow)
                            {
                                double em, abv;
                                gp19_profile_node(W.gp, W.gpp, S.lw, G19.d3, wmin, wmax, nu,
                                                  nub, &em, &abv);
                                kab = (float)(abv / (3. * W.gp.C));
                                kem = (float)(em * exp(w) / (3. * W.gp.C));
                            }
                            // w nubar^2 / T^2 rounded once from double-float factors
                            const dfm::df yb  = {X.ybh[a], X.ybl[a]};
                            const dfm::df wyd = dfm::mul(S.B1d[a], dfm::mul(yb, yb));
                            const float wy2   = wyd.hi + wyd.lo;
#pragma unroll
                            for (int s = 0; s < 4; ++s)
                            {
                                const int ps = s ^ 1;
                                float bf32   = nbb ? 1.f : X.gbm32[a][ps];
                                float g32    = X.gb32[a][ps];
                                float dre    = far ? wy2 * kab * kNesDrop : 0.f;
                                float dra    = 0.f;
                                if (fabsf(bf32) < kNesDrop)
                                {
                                    dre += wy2 * kem * kNesDrop;
                                    bf32 = 0.f;
                                }
                                if (g32 < kNesDrop)
                                {
                                    dra += wy2 * kab * kNesDrop;
                                    g32 = 0.f;
                                }
                                const float te = wy2 * (kem * bf32);
                                const float ta = wy2 * (kab * g32);
                                acc[s]     = fma(sbe, (double)te, acc[s]);
                                acc[4 + s] = fma(sb, (double)ta, acc[4 + s]);
                                gl[s] += fabsf(te) * (float)(1. / kSpecCancelBrem) + 1e9f * dre;
                                gl[4 + s] +=
                                    fabsf(ta) * (float)(1. / kSpecCancelBrem) + 1e9f * dra;
                            }
                        }
                    }
                }
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                {
                    acc[kk] = seg_sum(acc[kk], Gq);
                    if (MIX)
                    {
                        gl[kk] = seg_sum(gl[kk], Gq);
                        if (L.use_pair)
                            gp[kk] = seg_sum(gp[kk], Gq);
                    }
                }
                if (act && grp == 0)
                {
                    EnergyRec& E = R[e0 + c];
#pragma unroll
                    for (int kk = 0; kk < 8; ++kk)
                    {
                        E.pb[kk] = acc[kk];
                        if (MIX)
                            E.bpb[kk] = skip ? INFINITY
                                             : (b32 ? (kk < 4 ? sbe : sb) *
                                                          ((double)gl[kk] + kSpecFloor)
                                                    : 0.) +
                                                   gp[kk] * (1. / kSpecCancelPair);
                        else if (MODE == kSpecRedo)
                            E.bpb[kk] = 0.;
                    }
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// nes: inelastic neutrino-electron / -positron scattering
// ---------------------------------------------------------------------------
struct NesWarp
{
    Distr d;
    double fe[2][6];
    double fd0[2];
    int same_cf;
    double fw[kEChunk][2][6];
};

struct NesWarpMixed
{
    NepsMixed Q; // eta and F_k(eta) of e-, e+
    NesSpec Z;
    dfm::df rw[kEChunk][2][5]; // unreflected F_1..F_5 at eta_e - nu/T per energy and lepton
    dfm::df aw[kEChunk][2];
    dfm::df lnu[kEChunk];
};

template <int MODE>
struct NesShared
{
    double x[kMaxQ], xinv[kMaxQ], B1[kMaxM];
    dfm::df lxd[kMaxQ];
    dfm::FdiTab ftab;
    NesWarp w[kWarps];
    NesWarpMixed m[(MODE == kSpecMixed || MODE == kSpecAcc) ? kWarps : 1];
};

template <int MODE>
__global__ void __launch_bounds__(kWarps * 32, MODE == kSpecMixed ? 4 : 1)
    spec_nes_kernel(const __grid_constant__ OpacityLaunch L, int64_t p0, int64_t np,
                    const double* __restrict__ dsc, EnergyRec* __restrict__ rec,
                    const uint64_t* __restrict__ flags, int G)
{
    constexpr bool ACC = MODE == kSpecAcc;
    constexpr bool MIX = MODE == kSpecMixed || ACC;
    extern __shared__ __align__(16) unsigned char s_raw[];
    NesShared<MODE>& S = *reinterpret_cast<NesShared<MODE>*>(s_raw);
    for (int k = threadIdx.x; k < kMaxQ; k += blockDim.x)
    {
        S.x[k]    = L.x1[k];
        S.xinv[k] = 1. / L.x1[k];
        S.lxd[k]  = dfm::from_double(L.lx1[k]);
    }
    for (int k = threadIdx.x; k < kMaxM; k += blockDim.x)
        S.B1[k] = L.B1[k];
    if (MIX)
        for (int k = threadIdx.x; k < (int)(sizeof(dfm::FdiTab) / sizeof(float)); k += blockDim.x)
            ((float*)&S.ftab)[k] = ((const float*)&dfm::kFdiTab)[k];
    __syncthreads();

    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    NesWarp& W      = S.w[wid];
    NesWarpMixed& X = S.m[MIX ? wid : 0];
    const int n = L.n1, M = 2 * n, ne = L.n_energies;
    const bool nbb      = L.neglect_blocking != 0;
    const int64_t nwarp = (int64_t)gridDim.x * kWarps;

    for (int64_t q = (int64_t)blockIdx.x * kWarps + wid; q < np; q += nwarp)
    {
        const uint64_t emask = energy_mask(MODE, flags, q, ne);
        if (emask == 0ull)
            continue;
        const int Gq        = (MODE == kSpecRedo || ACC) ? pick_groups(__popcll(emask), M) : G;
        const int grp       = lane % Gq;
        const int per_round = 32 / Gq;
        const int64_t p     = p0 + q;
        const double T = L.eos[1][p], mu_e = L.eos[7][p];
        const double eta_e = mu_e / T, invT = 1. / T;
        EnergyRec* R       = rec + q * ne;
        __syncwarp();
        load_distr(dsc, q, &W.d, lane);
        if (lane == 28 || lane == 29)
        {
            const int e     = lane - 28;
            const double et = e ? -eta_e : eta_e;
            fdi_orders<0, 5>(et, W.fe[e]);
            W.fd0[e] = fermi_distr(0., 1., et);
        }
        __syncwarp();
        if (lane == 0)
            W.same_cf = same_cf_of(W.d);
        NepsPoint NP;
        NP.T    = T;
        NP.pre  = k::NepsConst * (T * T);
        NP.eta0 = eta_e;
        NP.eta1 = -eta_e;
        NP.fd00 = W.fd0[0];
        NP.fd01 = W.fd0[1];
        NP.fe0  = W.fe[0];
        NP.fe1  = W.fe[1];
        bool m32  = false;
        double sn = 0.;
        if (MIX)
        {
            m32 = fp32_envelope(W.d, eta_e);
            if (m32)
            {
                if (lane < 2)
                {
                    X.Q.eta[lane] = dfm::from_double(lane ? NP.eta1 : NP.eta0);
                    dfm::fdi_raw15(X.Q.eta[lane], X.Q.reta[lane], 1, &S.ftab);
                }
                else if (lane >= 8 && lane < 12)
                    nes_spec_species(W.d, lane - 8, &X.Z);
                else if (lane == 12)
                    nes_spec_masks(W.d, &X.Z);
            }
            sn = (T * T) * NP.pre;
        }
        __syncwarp();
        const bool same_cf = W.same_cf != 0;

        for (int e0 = 0; e0 < ne; e0 += kEChunk)
        {
            const int nec     = (ne - e0) < kEChunk ? (ne - e0) : kEChunk;
            const uint32_t cm = (uint32_t)(emask >> e0) &
                                (nec == 32 ? 0xffffffffu : ((1u << nec) - 1u));
            if (cm == 0u)
                continue;
            __syncwarp();
            for (int c = lane; c < nec; c += 32)
            {
                if (!((cm >> c) & 1u))
                    continue;
                const double nu = L.energies[e0 + c];
                const double y  = nu / T;
                if (!MIX)
                {
                    fdi_orders<0, 5>(eta_e - y, W.fw[c][0]);
                    fdi_orders<0, 5>(NP.eta1 - y, W.fw[c][1]);
                }
                else if (m32 && y >= kSpecNesMinW)
                {
                    X.lnu[c] = dfm::from_double(log(nu));
#pragma unroll 1
                    for (int e = 0; e < 2; ++e)
                    {
                        X.aw[c][e] = dfm::from_double((e ? NP.eta1 : NP.eta0) - y);
                        dfm::fdi_raw15(X.aw[c][e], X.rw[c][e], 1, &S.ftab);
                    }
                }
            }
            __syncwarp();
            const int nt = __popc(cm);
            for (int r0 = 0; r0 < nt; r0 += per_round)
            {
                const int kq    = r0 + lane / Gq;
                const bool act  = kq < nt;
                const int c     = act ? nth_bit(cm, kq) : 0;
                const double nu = act ? L.energies[e0 + c] : 1.;
                const double w  = nu / T;
                const bool run  = act && (!MIX || (m32 && w >= kSpecNesMinW));
                double acc[8];
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                    acc[kk] = 0.;
                float gl[8];
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                    gl[kk] = 0.f;
                float sig[2] = {0.f, 0.f};
                double sne = 0., sna = 0.;
                if (MIX)
                {
                    // scale of this energy: group-wide maximum of the lanes' scans
                    nes_spec_scan(X.Z, (float)w, (float)nu, X.lnu[run ? c : 0].hi, S.x, S.lxd,
                                  n, run ? grp : M, Gq, nbb, sig);
                    for (int o = 1; o < Gq; o <<= 1)
                    {
                        sig[0] = fmaxf(sig[0], __shfl_xor_sync(0xffffffffu, sig[0], o));
                        sig[1] = fmaxf(sig[1], __shfl_xor_sync(0xffffffffu, sig[1], o));
                    }
                    sig[0] = isfinite(sig[0]) ? sig[0] : 0.f;
                    sig[1] = isfinite(sig[1]) ? sig[1] : 0.f;
                    sne    = sn * exp((double)sig[0]);
                    sna    = sn * exp((double)sig[1]);
                }
                const dfm::df Wd = dfm::from_double(w);
                if (run)
                {
                    for (int a = grp; a < M; a += Gq)
                    {
                        const int i      = a < n ? a : a - n;
                        const double wa  = S.B1[a];
                        const double nub =
                            a < n ? nu * S.x[i] : (MIX ? nu * S.xinv[i] : nu / S.x[i]);
                        // mixed passes: nubar/T and log nubar without divisions
                        const double wp  = MIX ? nub * invT : nub / T;
                        const dfm::df NB = dfm::from_double(nub), WPd = dfm::from_double(wp);
                        const dfm::df LB =
                            dfm::add(X.lnu[c], a < n ? S.lxd[i] : dfm::neg(S.lxd[i]));
                        if (ACC)
                        {
                            double te[4], ta[4];
                            float de[4], da[4];
                            nes_spec_node_df(NP, X.Q, X.Z, &S.ftab, w, wp, Wd, WPd, NB, LB, wa,
                                             sig[0], sig[1], nbb, X.rw[c], X.aw[c], te, ta, de,
                                             da);
#pragma unroll
                            for (int s = 0; s < 4; ++s)
                            {
                                acc[s]     = fma(sne, te[s], acc[s]);
                                acc[4 + s] = fma(sna, ta[s], acc[4 + s]);
                                gl[s] += (float)(fabs(te[s]) * (1. / kSpecCancelDf)) + 1e9f * de[s];
                                gl[4 + s] +=
                                    (float)(fabs(ta[s]) * (1. / kSpecCancelDf)) + 1e9f * da[s];
                            }
                        }
                        else if (MIX)
                        {
                            float te[4], ta[4], de[4], da[4];
                            nes_spec_node(NP, X.Q, X.Z, &S.ftab, w, wp, Wd, WPd, NB, LB, (float)wa,
                                          sig[0], sig[1], nbb, X.rw[c], X.aw[c], te, ta, de, da);
#pragma unroll
                            for (int s = 0; s < 4; ++s)
                            {
                                acc[s]     = fma(sne, (double)te[s], acc[s]);
                                acc[4 + s] = fma(sna, (double)ta[s], acc[4 + s]);
                                gl[s] += fabsf(te[s]) * (float)(1. / kSpecCancelNes) + 1e9f * de[s];
                                gl[4 + s] +=
                                    fabsf(ta[s]) * (float)(1. / kSpecCancelNes) + 1e9f * da[s];
                            }
                        }
                        else
                        {
                            double gb[4], em[4], ab[4];
                            total_nu_f4(nub, W.d, same_cf, gb);
                            neps_one(NP, nu, nub, W.fw[c][0], W.fw[c][1], em, ab);
                            const double nb2 = nub * nub;
#pragma unroll
                            for (int s = 0; s < 4; ++s)
                            {
                                const double bf = nbb ? 1. : 1. - gb[s];
                                acc[s] += wa * (nb2 * (em[s] * gb[s]));
                                acc[4 + s] += wa * (nb2 * (ab[s] * bf));
                            }
                        }
                    }
                }
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                {
                    acc[kk] = seg_sum(acc[kk], Gq);
                    if (MIX)
                        gl[kk] = seg_sum(gl[kk], Gq);
                }
                if (act && grp == 0)
                {
                    EnergyRec& E = R[e0 + c];
#pragma unroll
                    for (int kk = 0; kk < 8; ++kk)
                    {
                        E.nes[kk] = acc[kk];
                        if (MIX)
                            E.bnes[kk] = run ? (kk < 4 ? sne : sna) * ((double)gl[kk] + kSpecFloor)
                                             : INFINITY;
                        else if (MODE == kSpecRedo)
                            E.bnes[kk] = 0.;
                    }
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// assemble (m1_opacities.hpp:1571-1660)
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(kWarps * 32)
    spec_assemble_kernel(const __grid_constant__ OpacityLaunch L, int64_t p0, int64_t np,
                         const double* __restrict__ dsc, const EnergyRec* __restrict__ rec,
                         uint64_t* __restrict__ fl_pb, uint64_t* __restrict__ fl_nes)
{
    constexpr bool GUARD = MODE == kSpecMixed || MODE == kSpecRedo;
    __shared__ Distr s_d[kWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    Distr& D       = s_d[wid];
    const int ne   = L.n_energies;
    const bool pb  = L.use_pair || L.use_brem;
    const int64_t nwarp = (int64_t)gridDim.x * kWarps;
    for (int64_t q = (int64_t)blockIdx.x * kWarps + wid; q < np; q += nwarp)
    {
        uint64_t emask = all_energies(ne);
        if (MODE == kSpecRedo || MODE == kSpecFinal)
        {
            emask &= fl_pb[q] | fl_nes[q];
            if (emask == 0ull)
                continue;
        }
        const int64_t p   = p0 + q;
        const double nbar = L.eos[0][p], T = L.eos[1][p];
        const double yp = L.eos[3][p], yn = L.eos[4][p];
        const double mu_p = L.eos[5][p], mu_n = L.eos[6][p], mu_e = L.eos[7][p];
        const double dU = L.eos[9][p], dm_eff = L.eos[10][p];
        __syncwarp();
        load_distr(dsc, q, &D, lane);
        __syncwarp();
        const bool same_cf = same_cf_of(D);
        BetaPoint bp;
        if (L.use_abs_em)
            bp = beta_point(nbar, T, yp, yn, mu_p, mu_n, mu_e, dU, dm_eff, L.use_dU, L.use_dm_eff,
                            L.use_WM_ab, L.use_decay);
        double eta_pp = 0., eta_nn = 0.;
        if (L.use_iso)
        {
            eta_pp = eta_nn_sc(nbar, T, yp);
            eta_nn = eta_nn_sc(nbar, T, yn);
        }
        const double ts = k::TempMultiple * T;
        uint64_t bad_pb = 0ull, bad_nes = 0ull;
        for (int e0 = 0; e0 < ne; e0 += 32)
        {
            const int e    = e0 + lane;
            const bool act = e < ne && ((emask >> e) & 1ull);
            bool fpb = false, fnes = false;
            if (act)
            {
                const double nu    = L.energies[e];
                const EnergyRec& E = rec[q * ne + e];
                double b_ab[4] = {0., 0., 0., 0.}, b_em[4] = {0., 0., 0., 0.};
                if (L.use_abs_em)
                {
                    beta_rates(bp, nu, 0, &b_ab[0], &b_em[0]);
                    beta_rates(bp, nu, 1, &b_ab[1], &b_em[1]);
                }
                const double F = k::FourPiHc3, c = k::Clight;
                double ip[8], in[8];
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                {
                    ip[kk] = pb ? ts * E.pb[kk] : 0.;
                    in[kk] = L.use_inel ? nu * E.nes[kk] : 0.;
                }
                if (GUARD)
                {
                    // FP32 error bounds against each output's total
#pragma unroll
                    for (int kk = 0; kk < 8; ++kk)
                    {
                        const int s      = kk & 3;
                        const double tot = (kk < 4 ? b_em[s] : b_ab[s]) + F * (ip[kk] + in[kk]);
                        const double bb  = pb ? F * ts * E.bpb[kk] : 0.;
                        const double bn  = L.use_inel ? F * nu * E.bnes[kk] : 0.;
                        const double at  = fabs(tot);
                        if (!(bb + bn <= at))
                        {
                            // the parts above half of a finite total (at least
                            // one is); both when neither is (or the total is
                            // not finite).  A bound is ~1e6 x the part's actual
                            // error, so redoing one part hardly moves the total
                            // and the kept part stays below half of it.
                            bool xp = bb > 0., xn = bn > 0.;
                            const bool hp = xp && !(bb <= 0.5 * at);
                            const bool hn = xn && !(bn <= 0.5 * at);
                            if (hp || hn)
                            {
                                xp = hp;
                                xn = hn;
                            }
                            fpb  = fpb || xp;
                            fnes = fnes || xn;
                        }
                    }
                }
                if (!fpb && !fnes)
                {
                    bool nonfinite = false;
                    double ge[4];
                    total_nu_f4(nu, D, same_cf, ge);
                    const double iso =
                        L.use_iso ? iso_scatt_leg0(nu, eta_pp, eta_nn, L.use_WM_sc != 0) : 0.;
                    const int64_t o = p * L.e_stride + L.e_offset + e;
#pragma unroll
                    for (int s = 0; s < 4; ++s)
                    {
                        const double g = ge[s];
                        double j  = b_em[s] + F * (ip[s] + in[s]);
                        double ka = (b_ab[s] + F * (ip[4 + s] + in[4 + s])) / c;
                        double js = 4. * k::Pi * (nu * nu) * g * iso;
                        double ks = 4. * k::Pi * (nu * nu) * (1. - g) * iso / c;
                        if (L.stim)
                        {
                            ka = j / c + ka;
                            ks = js / c + ks;
                        }
                        L.sout[s][o]      = j;
                        L.sout[4 + s][o]  = ka;
                        L.sout[8 + s][o]  = js;
                        L.sout[12 + s][o] = ks;
                        nonfinite = nonfinite || !isfinite(j) || !isfinite(ka) ||
                                    !isfinite(js) || !isfinite(ks);
                    }
                    if (nonfinite)
                        atomicAdd(&g_spec_nonfinite, 1ull);
                }
            }
            if (GUARD)
            {
                bad_pb |= (uint64_t)__ballot_sync(0xffffffffu, fpb) << e0;
                bad_nes |= (uint64_t)__ballot_sync(0xffffffffu, fnes) << e0;
            }
        }
        if (GUARD && lane == 0)
        {
            fl_pb[q]  = bad_pb;
            fl_nes[q] = bad_nes;
            if (MODE == kSpecMixed)
            {
                atomicAdd(&g_spec_counts[0], (unsigned long long)ne);
                atomicAdd(&g_spec_counts[1], (unsigned long long)__popcll(bad_pb | bad_nes));
            }
            atomicAdd(&g_spec_counts[2], (unsigned long long)__popcll(bad_pb));
            atomicAdd(&g_spec_counts[3], (unsigned long long)__popcll(bad_nes));
        }
    }
}

// Dynamic shared memory opt-in (once per kernel) and a persistent grid of two
// waves of resident CTAs, capped by the work.
template <class K>
cudaError_t grid_of(K kernel, size_t smem, bool* attr_set, int num_sms, int64_t warps_needed,
                    int* grid)
{
    cudaError_t err;
    if (!*attr_set)
    {
        if ((err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem)) != cudaSuccess)
            return err;
        *attr_set = true;
    }
    int per_sm = 0;
    if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWarps * 32, smem)) !=
        cudaSuccess)
        return err;
    per_sm             = per_sm < 1 ? 1 : per_sm;
    const int64_t need = (warps_needed + kWarps - 1) / kWarps;
    const int64_t cap  = (int64_t)num_sms * per_sm * 2;
    *grid              = (int)(need < cap ? need : cap);
    return cudaSuccess;
}

template <int MODE>
cudaError_t launch_pb(const OpacityLaunch& L, int64_t p0, int64_t np, const double* dsc,
                      EnergyRec* rec, const uint64_t* flags, int G, cudaStream_t st, int sms)
{
    static bool attr  = false;
    const size_t smem = sizeof(PbShared<MODE>);
    int grid          = 0;
    cudaError_t err   = grid_of(spec_pb_kernel<MODE>, smem, &attr, sms, np, &grid);
    if (err != cudaSuccess || grid == 0)
        return err;
    phase_mark(kPhSpectral, 0, st);
    spec_pb_kernel<MODE><<<grid, kWarps * 32, smem, st>>>(L, p0, np, dsc, rec, flags, G);
    phase_mark(kPhSpectral, 1, st);
    return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_nes(const OpacityLaunch& L, int64_t p0, int64_t np, const double* dsc,
                       EnergyRec* rec, const uint64_t* flags, int G, cudaStream_t st, int sms)
{
    static bool attr  = false;
    const size_t smem = sizeof(NesShared<MODE>);
    int grid          = 0;
    cudaError_t err   = grid_of(spec_nes_kernel<MODE>, smem, &attr, sms, np, &grid);
    if (err != cudaSuccess || grid == 0)
        return err;
    phase_mark(kPhSpectral, 0, st);
    spec_nes_kernel<MODE><<<grid, kWarps * 32, smem, st>>>(L, p0, np, dsc, rec, flags, G);
    phase_mark(kPhSpectral, 1, st);
    return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_assemble(const OpacityLaunch& L, int64_t p0, int64_t np, const double* dsc,
                            const EnergyRec* rec, uint64_t* fl_pb, uint64_t* fl_nes,
                            cudaStream_t st, int sms)
{
    static bool attr = false;
    int grid         = 0;
    cudaError_t err  = grid_of(spec_assemble_kernel<MODE>, 0, &attr, sms, np, &grid);
    if (err != cudaSuccess || grid == 0)
        return err;
    phase_mark(kPhSpectral, 0, st);
    spec_assemble_kernel<MODE><<<grid, kWarps * 32, 0, st>>>(L, p0, np, dsc, rec, fl_pb, fl_nes);
    phase_mark(kPhSpectral, 1, st);
    return cudaGetLastError();
}

} // namespace

int64_t spectral_chunk_points(int n_energies)
{
    const int64_t ne = n_energies < 1 ? 1 : n_energies;
    const int64_t c  = kSpecChunkRecords / ne;
    return c < 32 ? 32 : c;
}

size_t spectral_scratch_bytes(int64_t chunk_points, int n_energies)
{
    return (size_t)chunk_points *
           (28 * sizeof(double) + 2 * sizeof(uint64_t) + (size_t)n_energies * sizeof(EnergyRec));
}

cudaError_t spectral_mixed_counts(unsigned long long* counts, bool reset)
{
    cudaError_t e = cudaMemcpyFromSymbol(counts, g_spec_counts, sizeof(g_spec_counts));
    if (e == cudaSuccess && reset)
    {
        const unsigned long long zero[4] = {0ull, 0ull, 0ull, 0ull};
        e = cudaMemcpyToSymbol(g_spec_counts, zero, sizeof(zero));
    }
    return e;
}

cudaError_t spectral_nonfinite_count(unsigned long long* count, bool reset)
{
    cudaError_t e = cudaMemcpyFromSymbol(count, g_spec_nonfinite, sizeof(*count));
    if (e == cudaSuccess && reset)
    {
        const unsigned long long zero = 0ull;
        e = cudaMemcpyToSymbol(g_spec_nonfinite, &zero, sizeof(zero));
    }
    return e;
}

cudaError_t launch_spectral(const OpacityLaunch& L, cudaStream_t st0, int sms, void* scratch,
                            int64_t chunk_points, cudaStream_t aux, void* scratch1)
{
    if (L.npts <= 0 || L.n_energies <= 0)
        return cudaSuccess;
    const int ne     = L.n_energies;
    const int G      = pick_groups(ne < kEChunk ? ne : kEChunk, 2 * L.n1);
    const bool pb    = L.use_pair || L.use_brem;
    const bool inel  = L.use_inel != 0;
    // With an auxiliary stream and scratch, consecutive chunks alternate
    // between the caller's stream and aux: the redo passes of one chunk (few
    // flagged records, a mostly idle grid) run beside the main passes of the
    // other.  The caller's stream waits for aux at the end.
    const bool two    = aux != nullptr && scratch1 != nullptr && L.npts > chunk_points;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (two)
    {
        cudaError_t e;
        if ((e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventRecord(ev[0], st0)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(aux, ev[0], 0)) != cudaSuccess)
        {
            if (ev[0])
                cudaEventDestroy(ev[0]);
            if (ev[1])
                cudaEventDestroy(ev[1]);
            return e;
        }
    }
    cudaError_t err = cudaSuccess;
    int64_t k       = 0;
    for (int64_t p0 = 0; p0 < L.npts && err == cudaSuccess; p0 += chunk_points, ++k)
    {
        const bool odd        = two && (k & 1);
        const cudaStream_t st = odd ? aux : st0;
        double* dsc           = (double*)(odd ? scratch1 : scratch);
        uint64_t* fl_pb       = (uint64_t*)(dsc + chunk_points * 28);
        uint64_t* fl_nes      = fl_pb + chunk_points;
        EnergyRec* rec        = (EnergyRec*)(fl_nes + chunk_points);
        const int64_t np  = (L.npts - p0) < chunk_points ? (L.npts - p0) : chunk_points;
        const int64_t nth = np * 4;
        phase_mark(kPhSpectral, 0, st);
        spec_prelude_kernel<<<(int)((nth + 127) / 128), 128, 0, st>>>(L, p0, np, dsc);
        phase_mark(kPhSpectral, 1, st);
        if ((err = cudaGetLastError()) != cudaSuccess)
            break;
        if (!L.mixed)
        {
            if (pb && (err = launch_pb<kSpecFp64>(L, p0, np, dsc, rec, nullptr, G, st, sms)))
                break;
            if (inel && (err = launch_nes<kSpecFp64>(L, p0, np, dsc, rec, nullptr, G, st, sms)))
                break;
            err = launch_assemble<kSpecFp64>(L, p0, np, dsc, rec, fl_pb, fl_nes, st, sms);
            continue;
        }
        if (pb && (err = launch_pb<kSpecMixed>(L, p0, np, dsc, rec, nullptr, G, st, sms)))
            break;
        if (inel && (err = launch_nes<kSpecMixed>(L, p0, np, dsc, rec, nullptr, G, st, sms)))
            break;
        if ((err = launch_assemble<kSpecMixed>(L, p0, np, dsc, rec, fl_pb, fl_nes, st, sms)))
            break;
        for (int round = 0; round < 2 && err == cudaSuccess; ++round)
        {
            if (pb && (err = launch_pb<kSpecRedo>(L, p0, np, dsc, rec, fl_pb, G, st, sms)))
                break;
            // NES: double-float products first, FP64 for what still fails
            if (inel && (err = round == 0 ? launch_nes<kSpecAcc>(L, p0, np, dsc, rec, fl_nes, G,
                                                                 st, sms)
                                          : launch_nes<kSpecRedo>(L, p0, np, dsc, rec, fl_nes,
                                                                  G, st, sms)))
                break;
            err = round == 0
                      ? launch_assemble<kSpecRedo>(L, p0, np, dsc, rec, fl_pb, fl_nes, st, sms)
                      : launch_assemble<kSpecFinal>(L, p0, np, dsc, rec, fl_pb, fl_nes, st, sms);
        }
    }
    if (two)
    {
        const cudaError_t e1 = cudaEventRecord(ev[1], aux);
        const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(st0, ev[1], 0) : e1;
        cudaEventDestroy(ev[0]);
        cudaEventDestroy(ev[1]);
        if (err == cudaSuccess)
            err = e2;
    }
    return err;
}

} // namespace bnsn
