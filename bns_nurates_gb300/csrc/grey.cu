// Grey M1 opacity kernels (sm_103a), FP64 and mixed precision.
//
// Restates ComputeM1OpacitiesGenericFormalism (m1_opacities.hpp:1062-1295)
// with the integration rules of integration.hpp:608-844, as six phase
// kernels over a chunk of points.  Each phase has a small hot loop shared by
// all resident warps, so the instruction working set stays in the SM's
// instruction cache (a single fused kernel spent most of its issue slots
// waiting on instruction fetch):
//
//   point   : per (point, task) (one thread): distribution parameters,
//             Fermi integrals at +-eta_e, brem and iso constants, written to
//             the header of the point's scratch record.
//   prelude : per point (one warp): the 2n-energy tables of the double
//             integral (distribution values, F_k(eta +- w/T)) and the 1-D beta
//             and iso-scattering integrals; the per-point record is staged in
//             shared memory and written to the scratch arena.
//   pair    : per point (one warp): the M(M+1)/2 unordered (w, w') cells of
//             the pair kernel, one evaluation filling (w, w') and (w', w),
//             weighted and summed into the number and energy moments.
//   brem    : the same cells for the bremsstrahlung kernel (HR98, BRT06, GP19).
//   neps    : per point (one warp): the 2 n^2 (nu, nubar) pairs of the NES/NPS
//             double integral, both directions from one set of Fermi integrals.
//   final   : per point (one thread): assembly of the 20 outputs.
//
// The reference's 2n x 2n integrand matrices (m1_opacities.hpp:774-1057) are
// never materialised: every cell is multiplied by its quadrature weight and
// summed directly; lane sums are combined with warp shuffles.
//
// MIXED = false: every operation in FP64 (the plain path).
// MIXED = true : the HR98 bremsstrahlung shape of each cell runs in FP32
// (bnsn_fp32.cuh) and the pair kernel takes one expm1 instead of two
// exponentials; Fermi-Dirac integrals, the pair Psi polynomial (catastrophic
// cancellation), distribution reconstruction, detailed balance and the
// distribution-weighted sums stay FP64.

#include <cuda_runtime.h>

#include <cstddef>

#include "bnsn_df.cuh"
#include "bnsn_fp32.cuh"
#include "bnsn_mixed.cuh"
#include "bnsn_fp64.cuh"
#include "bnsn_nes32.cuh"
#include "bnsn_pair32.cuh"
#include "bnsn_internal.h"

namespace bnsn {

using namespace fp64;

// Per-point record in the scratch arena (double words only, no padding).
struct PointTab
{
    Distr d;
    double fe[2][6];  // F_0..F_5 at eta_e and -eta_e
    double fd0[2];    // FermiDistr(0, 1, +-eta_e)
    Hr98Point hr;
    double brt06_pre;
    double eta_pp, eta_nn;
    double same_cf;
    double nu[kMaxM];    // energies of the double-integral grid
    double y[kMaxM];     // nu / T
    double g[kMaxM][4];  // TotalNuF at nu per species
    double fm[kMaxM][5]; // F_1..F_5 at eta_e - nu/T
    double fp[kMaxM][5]; // F_1..F_5 at eta_e + nu/T
    double s2d[16];      // pair + brem: n-moment em/ab, J-moment em/ab
    double snes[16];     // NES/NPS, same layout
    double sbeta[8];     // beta: n_em[2], j_em[2], n_ab[2], j_ab[2]
    double siso[4];      // iso per species
    double sbrem[16];    // brem alone (its part of s2d)
    double bmag[16];     // mixed path: sum of |term| of FP32 brem cells (s2d units), else 0
    double neps_fp64;    // mixed path: 1 if the NES sums of the point must be FP64
    double bredo;        // mixed path: 1 if the brem sums must be recomputed in FP64
};
static_assert(sizeof(PointTab) % sizeof(double) == 0, "PointTab must be double words");
static_assert(sizeof(PointTab) == kGreyRecordBytes, "grey record size");
constexpr int kTabWords = sizeof(PointTab) / sizeof(double);

// Mixed path with the pair kernel on: the pair phase computes no Fermi-integral
// tables (fm, fp), so their words hold its own sums, their magnitudes and the
// final kernel's verdict instead.
struct PairMixed
{
    double spair[16]; // the pair part of s2d
    double pmag[16];  // sum of |term| of the pair cells per moment (s2d units)
    double predo;     // 1 if the point's pair sums must be recomputed in FP64
};
static_assert(sizeof(PairMixed) <= sizeof(((PointTab*)nullptr)->fm), "PairMixed overlay");
// Mixed path: points evaluated, NES handed to the double-float pass, NES in
// FP64, pair sums redone in FP64, brem sums redone in FP64 (read by
// grey_mixed_counts).
__device__ unsigned long long g_grey_mixed[5];

__device__ __forceinline__ PairMixed* pair_mixed(PointTab* P)
{
    return reinterpret_cast<PairMixed*>(&P->fm[0][0]);
}

size_t grey_point_scratch_bytes() { return sizeof(PointTab); }

namespace {

constexpr int kWarps = 4; // warps per CTA in the per-point kernels

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double total_nu_f1(double omega, const Distr& d, int s)
{
    const double ft = fermi_distr(omega, d.temp_t[s], d.temp_t[s] * d.eta_t[s]);
    const double fn = d.beta_f[s] * pow(omega, d.c_f[s]) * exp(-omega / d.temp_f[s]);
    return d.w_t[s] * ft + d.w_f[s] * fn;
}

// Cooperative copy of `words` doubles (lane-strided, coalesced).
__device__ __forceinline__ void warp_copy(double* __restrict__ dst,
                                          const double* __restrict__ src, int words,
                                          int lane)
{
    for (int k = lane; k < words; k += 32)
        dst[k] = src[k];
}

// s_beta of m1_opacities.hpp:1093-1110 from F_4, F_5 at +-eta_e.
__device__ __forceinline__ void beta_scales(double T, double eta_e, const double (&fe)[2][6],
                                            double* sb)
{
    if (eta_e > -30. && eta_e < 30.)
    {
        sb[0] = T * fe[0][5] / fe[0][4];
        sb[1] = T * fe[1][5] / fe[1][4];
    }
    else if (eta_e > 30.)
    {
        sb[0] = T * eta_e * 0.8333333333333333;
        sb[1] = T * 5.;
    }
    else
    {
        sb[0] = T * 5.;
        sb[1] = T * eta_e * 0.8333333333333333;
    }
}

// ---------------------------------------------------------------------------
// point constants: the per-point quantities that do not depend on an energy
// node, as 12 independent tasks, one thread per (point, task) with the task
// in blockIdx.y (every warp runs one code path):
//   0..3  distribution parameters of species 0..3 (or a copy of the given ones)
//   4, 5  F_0..F_5 and FermiDistr(0, 1, .) at +eta_e, -eta_e
//   6..8  HR98 channel constants; 9: HR98 point constants; 10: BRT06 prefactor
//   11    eta_NN of protons and neutrons (iso scattering)
// written straight into the point's scratch record, whose header the prelude
// then loads.  Inside the one-warp-per-point prelude these tasks ran on one to
// four lanes each, one after the other.
// ---------------------------------------------------------------------------
constexpr int kPointTasks = 12;

template <bool MULTI = false>
__global__ void __launch_bounds__(128)
    grey_point_kernel(const __grid_constant__ OpacityLaunch L0, const GroupArgs GA, int64_t p0,
                      int64_t np, double* __restrict__ scratch)
{
    const OpacityLaunch& L = MULTI ? GA.Ls[blockIdx.z] : L0;
    if (MULTI)
    {
        const GroupChunk& gcz = GA.gc[blockIdx.z];
        p0      = gcz.p0;
        np      = gcz.np;
        scratch = gcz.ws;
    }
    const int task = blockIdx.y;
    if ((task >= 6 && task <= 9 && !(L.use_brem && L.brem_impl == 0)) ||
        (task == 10 && !(L.use_brem && L.brem_impl == 1)) || (task == 11 && !L.use_iso))
        return;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < np;
         q += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t p = L.pidx ? L.pidx[p0 + q] : p0 + q;
        PointTab* P     = (PointTab*)(scratch + q * kTabWords);
        const double nb = L.eos[0][p], T = L.eos[1][p];
        if (task < 4)
        {
            const int s = task;
            Distr& d    = P->d;
            if (L.has_distr)
            {
#pragma unroll
                for (int f = 0; f < 7; ++f)
                    (&d.w_t[0])[f * 4 + s] = L.distr[f * 4 + s][p];
            }
            else
                distr_species(L.m1[s][p], L.m1[4 + s][p], L.m1[8 + s][p], L.gamma36, &d.w_t[s],
                              &d.temp_t[s], &d.eta_t[s], &d.w_f[s], &d.temp_f[s], &d.c_f[s],
                              &d.beta_f[s]);
        }
        else if (task < 6)
        {
            const int e     = task - 4;
            const double et = e ? -L.eos[7][p] / T : L.eos[7][p] / T;
            double f[6];
            fdi_orders<0, 5>(et, f);
#pragma unroll
            for (int kk = 0; kk < 6; ++kk)
                P->fe[e][kk] = f[kk];
            P->fd0[e] = fermi_distr(0., 1., et);
        }
        else if (task < 9)
            P->hr.ch[task - 6] = hr98_channel(nb, L.eos[4][p], L.eos[3][p], T, task - 6);
        else if (task == 9)
            hr98_point_common(nb, T, L.use_medium != 0, &P->hr); // leaves hr.ch alone
        else if (task == 10)
            P->brt06_pre = brt06_point(nb, T, L.eos[4][p], L.eos[3][p]);
        else
        {
            P->eta_pp = eta_nn_sc(nb, T, L.eos[3][p]);
            P->eta_nn = eta_nn_sc(nb, T, L.eos[4][p]);
        }
    }
}

// Words of the record header written by grey_point_kernel (everything
// before the energy tables).
constexpr int kHeadWords = (int)(offsetof(PointTab, nu) / sizeof(double));

// TotalNuF of one species in FP32 with its exponent arguments in df form
// (distribution.hpp:298-315): x rt - eta_t and P0 + c_f log x - x rf.  The
// NES items take x = w = omega / T (rt = T / T_t, rf = T / T_f,
// P0 = log beta_f + c_f log T), the prelude's beta and iso items x = omega
// in MeV (rt = 1 / T_t, rf = 1 / T_f, P0 = log beta_f).  Both arguments cancel
// (the product's leading part against eta_t or P0), so they are formed from
// the exact FMA remainders; the occupation and its complement then keep FP32
// relative accuracy (the complement from the two parts' complements,
// w_t + w_f = 1 for the reconstructed distribution).
struct NuSpecies
{
    dfm::df etat, rt, P0, cf, rf;
    float wt, wf;
};

__device__ __forceinline__ void total_nu_one(dfm::df X, dfm::df LX, const NuSpecies& S,
                                             float& g, float& gm)
{
    // a = x rt - eta_t as hi + lo; e^{-|a|} = e^{-|hi|} (1 -+ lo): a float
    // exponent alone would cost |a| 6e-8 of relative accuracy
    const dfm::df pa = dfm::two_prod(X.hi, S.rt.hi);
    const dfm::df sa = dfm::two_sum(pa.hi, -S.etat.hi);
    const dfm::df A  = dfm::fast_two_sum(
        sa.hi, sa.lo + pa.lo + fmaf(X.hi, S.rt.lo, fmaf(X.lo, S.rt.hi, -S.etat.lo)));
    const bool pos  = A.hi > 0.f;
    const float t   = expf(-fabsf(A.hi)) * (pos ? 1.f - A.lo : 1.f + A.lo);
    const float inv = nes32::rcp_nr(t + 1.f);
    const float ft  = pos ? t * inv : inv;
    const float ftm = pos ? inv : t * inv;
    float fn        = 0.f;
    if (S.wf != 0.f)
    {
        const dfm::df p1 = dfm::two_prod(S.cf.hi, LX.hi);
        const dfm::df p2 = dfm::two_prod(-X.hi, S.rf.hi);
        const dfm::df s1 = dfm::two_sum(S.P0.hi, p1.hi);
        const dfm::df s2 = dfm::two_sum(s1.hi, p2.hi);
        const float lo   = (S.P0.lo + p1.lo + p2.lo + s1.lo + s2.lo) +
                         fmaf(S.cf.hi, LX.lo, S.cf.lo * LX.hi) - fmaf(X.hi, S.rf.lo, X.lo * S.rf.hi);
        const dfm::df F = dfm::fast_two_sum(s2.hi, lo);
        fn = expf(F.hi) * (1.f + F.lo);
    }
    g  = S.wt * ft + S.wf * fn;
    gm = S.wt * ftm + S.wf * (1.f - fn);
}

// The constants of species s of distribution d for x = omega * xscale
// (xscale = 1 / T for the NES items, 1 for omega in MeV); lxs = log xscale.
__device__ __forceinline__ void nu_species(const Distr& d, int s, double xscale_inv, double lxs,
                                           NuSpecies* S)
{
    S->wt   = (float)d.w_t[s];
    S->wf   = (float)d.w_f[s];
    S->etat = dfm::from_double(d.eta_t[s]);
    S->rt   = dfm::from_double(xscale_inv / d.temp_t[s]);
    const double lbf = d.beta_f[s] > 0. ? log(d.beta_f[s]) : 0.;
    S->P0   = dfm::from_double(lbf - d.c_f[s] * lxs);
    S->cf   = dfm::from_double(d.c_f[s]);
    S->rf   = dfm::from_double(xscale_inv / d.temp_f[s]);
}

__device__ __forceinline__ void total_nu_q(dfm::df W, dfm::df LW, const NuSpecies* sp, float* g,
                                           float* gm)
{
#pragma unroll
    for (int s = 0; s < 4; ++s)
        total_nu_one(W, LW, sp[s], g[s], gm[s]);
}

// ---------------------------------------------------------------------------
// prelude
// ---------------------------------------------------------------------------
template <bool MULTI = false>
__global__ void __launch_bounds__(kWarps * 32)
    grey_prelude_kernel(const __grid_constant__ OpacityLaunch L0, const GroupArgs GA, int64_t p0,
                        int64_t np, double* __restrict__ scratch)
{
    const OpacityLaunch& L = MULTI ? GA.Ls[blockIdx.z] : L0;
    if (MULTI)
    {
        const GroupChunk& gcz = GA.gc[blockIdx.z];
        p0      = gcz.p0;
        np      = gcz.np;
        scratch = gcz.ws;
    }
    __shared__ double s_B1[kMaxM], s_x1[kMaxQ], s_x2[kMaxQ], s_lx1[kMaxQ];
    __shared__ PointTab s_tab[kWarps];
    // mixed path: the occupation of the beta and iso items in FP32
    // (total_nu_one), omega in MeV; the FP64 path keeps total_nu_f1
    __shared__ NuSpecies s_nu[kWarps][4];
    for (int k = threadIdx.x; k < kMaxM; k += blockDim.x)
        s_B1[k] = L.B1[k];
    for (int k = threadIdx.x; k < kMaxQ; k += blockDim.x)
    {
        s_x1[k]  = L.x1[k];
        s_x2[k]  = L.x2[k];
        s_lx1[k] = L.lx1[k];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    PointTab& W    = s_tab[threadIdx.x >> 5];
    NuSpecies* Snu = s_nu[threadIdx.x >> 5];
    const int n1 = L.n1, n2 = L.n2, M = 2 * n2;
    const int64_t nwarp = (int64_t)gridDim.x * kWarps;

    for (int64_t q = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5); q < np; q += nwarp)
    {
        const int64_t p = L.pidx ? L.pidx[p0 + q] : p0 + q;
        const double nb = L.eos[0][p], T = L.eos[1][p];
        const double yp = L.eos[3][p], yn = L.eos[4][p];
        const double mu_e = L.eos[7][p];
        const double eta_e = mu_e / T;

        // header of the record (distribution, F_k(+-eta_e), brem and iso
        // constants) from grey_point_kernel
        __syncwarp();
        warp_copy((double*)&W, scratch + q * kTabWords, kHeadWords, lane);
        __syncwarp();
        if (lane == 0)
        {
            const double c0 = W.d.c_f[0];
            W.same_cf = ((W.d.c_f[1] == c0) && (W.d.c_f[2] == c0) && (W.d.c_f[3] == c0)) ? 1. : 0.;
        }
        else if (L.mixed && lane >= 8 && lane < 12)
            nu_species(W.d, lane - 8, 1., 0., &Snu[lane - 8]);
        __syncwarp();
        const bool same_cf = W.same_cf != 0.;

        // energy tables of the double integral (m1_opacities.hpp:783-787)
        if (L.use_pair || L.use_brem)
        {
            const double t2d = k::TempMultiple * T;
            for (int a = lane; a < M; a += 32)
            {
                const int i     = a < n2 ? a : a - n2;
                const double nu = a < n2 ? t2d * s_x2[i] : t2d / s_x2[i];
                W.nu[a]         = nu;
                W.y[a]          = nu / T;
                total_nu_f4(nu, W.d, same_cf, W.g[a]);
            }
            if (L.use_pair && !L.mixed) // the mixed pair phase needs no F tables
            {
                for (int qq = lane; qq < 2 * M; qq += 32)
                {
                    const int a     = qq >> 1;
                    const int i     = a < n2 ? a : a - n2;
                    const double nu = a < n2 ? t2d * s_x2[i] : t2d / s_x2[i];
                    const double y  = nu / T;
                    if (qq & 1)
                        fdi_orders<1, 5>(eta_e + y, W.fp[a]);
                    else
                        fdi_orders<1, 5>(eta_e - y, W.fm[a]);
                }
            }
        }

        // beta processes (m1_opacities.hpp:93-237, integration.hpp:805-844)
        if (L.use_abs_em)
        {
            double sb[2];
            beta_scales(T, eta_e, W.fe, sb);
            const BetaPoint bp =
                beta_point(nb, T, yp, yn, L.eos[5][p], L.eos[6][p], mu_e, L.eos[9][p],
                           L.eos[10][p], L.use_dU, L.use_dm_eff, L.use_WM_ab, L.use_decay);
            double acc[8];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                acc[kk] = 0.;
            const int m1n = 2 * n1;
            const double lsb0 = L.mixed ? log(sb[0]) : 0., lsb1 = L.mixed ? log(sb[1]) : 0.;
            for (int it = lane; it < 2 * m1n; it += 32)
            {
                const int s = it >= m1n;
                const int a = it - s * m1n;
                const int i = a < n1 ? a : a - n1;
                const double t  = sb[s];
                const double nu = a < n1 ? t * s_x1[i] : t / s_x1[i];
                double g;
                if (L.mixed)
                {
                    float gf, gmf;
                    const double lnu = (s ? lsb1 : lsb0) + (a < n1 ? s_lx1[i] : -s_lx1[i]);
                    total_nu_one(dfm::from_double(nu), dfm::from_double(lnu), Snu[s], gf, gmf);
                    g = gf;
                }
                else
                    g = total_nu_f1(nu, W.d, s);
                double ab, em;
                beta_rates(bp, nu, s, &ab, &em);
                if (L.stim)
                    ab = ab + em;
                const double nu2 = nu * nu;
                const double ev  = nu2 * em;
                const double av  = nu2 * g * ab;
                const double wn  = s_B1[a];
                const double wj  = wn * nu;
                if (s == 0)
                {
                    acc[0] += wn * ev;
                    acc[2] += wj * ev;
                    acc[4] += wn * av;
                    acc[6] += wj * av;
                }
                else
                {
                    acc[1] += wn * ev;
                    acc[3] += wj * ev;
                    acc[5] += wn * av;
                    acc[7] += wj * av;
                }
            }
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                acc[kk] = warp_sum(acc[kk]);
            if (lane == 0)
            {
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                    W.sbeta[kk] = acc[kk];
            }
        }

        // iso-energetic scattering (m1_opacities.hpp:39-91, integration.hpp:770-802)
        if (L.use_iso)
        {
            double s_iso[4];
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                const double ns = L.m1[s][p];
                s_iso[s] = (ns > k::ThresholdN) ? (L.m1[4 + s][p] / ns) : 1.5 * T;
            }
            double acc[4] = {0., 0., 0., 0.};
            double lsi[4] = {0., 0., 0., 0.};
            if (L.mixed)
            {
#pragma unroll
                for (int s = 0; s < 4; ++s)
                    lsi[s] = log(s_iso[s]);
            }
            const int m1n = 2 * n1;
            for (int it = lane; it < 4 * m1n; it += 32)
            {
                const int s = it / m1n;
                const int a = it - s * m1n;
                const int i = a < n1 ? a : a - n1;
                const double t   = s == 0 ? s_iso[0] : s == 1 ? s_iso[1] : s == 2 ? s_iso[2] : s_iso[3];
                const double nu  = a < n1 ? t * s_x1[i] : t / s_x1[i];
                double g;
                if (L.mixed)
                {
                    float gf, gmf;
                    const double ls  = s == 0 ? lsi[0] : s == 1 ? lsi[1] : s == 2 ? lsi[2] : lsi[3];
                    const double lnu = ls + (a < n1 ? s_lx1[i] : -s_lx1[i]);
                    total_nu_one(dfm::from_double(nu), dfm::from_double(lnu), Snu[s], gf, gmf);
                    g = gf;
                }
                else
                    g = total_nu_f1(nu, W.d, s);
                // mixed: the weak-magnetism factors in FP32 (positive terms; the
                // iso sum enters kappa_s alone, no other reaction cancels it)
                const double iso =
                    (L.mixed && L.use_WM_sc)
                        ? k::IsoConst * (W.eta_pp * (double)fp32::iso_wm_factor((float)nu, 1) +
                                         W.eta_nn * (double)fp32::iso_wm_factor((float)nu, 2))
                        : iso_scatt_total(nu, W.eta_pp, W.eta_nn, L.use_WM_sc != 0);
                const double aux = 4. * k::Pi * (nu * nu) * (nu * nu) * nu * iso;
                const double v   = g * aux * s_B1[a];
                if (s == 0) acc[0] += v;
                else if (s == 1) acc[1] += v;
                else if (s == 2) acc[2] += v;
                else acc[3] += v;
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                acc[kk] = warp_sum(acc[kk]);
            if (lane == 0)
            {
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    W.siso[kk] = acc[kk];
            }
        }
        __syncwarp();
        warp_copy(scratch + q * kTabWords, (const double*)&W, kTabWords, lane);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// weight algebra of m1_opacities.hpp:577-758 for one directed cell (a, b):
// em_s = K_em[s] bf_b[partner(s)], ab_s = K_ab[s] g_b[partner(s)], then
// stimulated absorption and the nu^2 nubar^2 weight, summed with the number
// (W1) and energy (W2) quadrature weights.  The moments are linear in the
// kernel, so pair and brem contributions are summed in separate phases.
// ---------------------------------------------------------------------------
template <bool STIM>
__device__ __forceinline__ void add_cell(double* acc, const double* Kem, const double* Kab,
                                         const double* ga, const double* gb, bool nb_block,
                                         double w4, double W1, double W2)
{
#pragma unroll
    for (int s = 0; s < 4; ++s)
    {
        const int ps    = s ^ 1;
        const double em = Kem[s] * (nb_block ? 1. : 1. - gb[ps]);
        const double am = Kab[s] * gb[ps];
        double EM, AB;
        if (STIM)
        {
            AB = w4 * ga[s] * (em + am);
            EM = em * w4;
        }
        else
        {
            AB = am * (w4 * ga[s]);
            EM = em * (w4 * (1. - ga[s]));
        }
        acc[s] += EM * W1;
        acc[4 + s] += AB * W1;
        acc[8 + s] += EM * W2;
        acc[12 + s] += AB * W2;
    }
}

// Shared-memory copy of the energy tables a cell loop needs.
struct CellTab
{
    double nu[kMaxM];
    double y[kMaxM];
    double g[kMaxM][4];
    double fm[kMaxM][5];
    double fp[kMaxM][5];
    double f3e, f4e;
    double brt06_pre;
    Hr98Point hr;
    fp32::Hr98Mixed hm;
};

__device__ __forceinline__ void load_cell_tab(CellTab& C, const PointTab* __restrict__ P,
                                              int M, bool pair_tables, int lane)
{
    warp_copy(C.nu, P->nu, M, lane);
    warp_copy(C.y, P->y, M, lane);
    warp_copy(&C.g[0][0], &P->g[0][0], 4 * M, lane);
    if (pair_tables)
    {
        warp_copy(&C.fm[0][0], &P->fm[0][0], 5 * M, lane);
        warp_copy(&C.fp[0][0], &P->fp[0][0], 5 * M, lane);
    }
    if (lane == 0)
    {
        C.f3e       = P->fe[0][3];
        C.f4e       = P->fe[0][4];
        C.brt06_pre = P->brt06_pre;
    }
}

// Mixed-path cell tables (FP32): g and 1 - g per species (1 - g formed in
// FP64), and nu/T as a double-float pair for the detailed-balance exponent.
struct CellTab32
{
    float g[kMaxM][4];
    float gm[kMaxM][4];
    float yh[kMaxM], yl[kMaxM];
};

// FP32 cell sums: per-lane partial sums of up to 4 cells are flushed into the
// FP64 accumulators, which bounds the FP32 summation error by a few ulp.
struct Acc32
{
    float v[16];
    float mag[16]; // sum of |term| per moment
    __device__ __forceinline__ void clear()
    {
#pragma unroll
        for (int k = 0; k < 16; ++k)
            v[k] = 0.f;
    }
};

// Largest error amplification over the 16 moments of a point (number and
// energy, emission and absorption, 4 species): the sum of |term| over
// |total|, where the total adds the other reactions' sums of the same output
// (`other`, in the units of scale x acc: the pair, brem or NES sums already
// computed and the beta rates, which cancel the brem or NES sums where the
// reconstructed occupation exceeds 1).  Terms are those of this lane (acc,
// mag, unscaled; moments 8..15 scaled by scale_e); the result is
// warp-reduced and 1 when every contribution has one sign.
// The same from the totals (already summed over the point's lanes).
__device__ __forceinline__ double cancel_factor_tot(const double* acc, const double* mag,
                                                    double scale, double scale_e,
                                                    const double* other)
{
    double amp = 1.;
#pragma unroll
    for (int s = 0; s < 16; ++s)
    {
        const double sc  = s < 8 ? scale : scale_e;
        const double m   = mag[s] * sc;
        const double tot = fabs(acc[s] * sc + other[s]);
        amp = fmax(amp, m > 0. ? m / tot : 1.);
    }
    return amp;
}

// (element by element: the 16 warp sums are not held at once)
__device__ __forceinline__ double cancel_factor(const double* acc, const float* mag, double scale,
                                                double scale_e, const double* other)
{
    double amp = 1.;
#pragma unroll
    for (int s = 0; s < 16; ++s)
    {
        const double sc  = s < 8 ? scale : scale_e;
        const double m   = warp_sum((double)mag[s]) * sc;
        const double tot = fabs(warp_sum(acc[s]) * sc + other[s]);
        amp = fmax(amp, m > 0. ? m / tot : 1.);
    }
    return amp;
}

// v[0..16) summed over the CTA's NW warps in a fixed order; every thread
// receives the totals.  red: NW x 32 doubles of shared memory, columns
// col .. col + 15 used.
template <int NW>
__device__ __forceinline__ void block_sum(double* v, double (*red)[32], int col)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int kk = 0; kk < 16; ++kk)
        v[kk] = warp_sum(v[kk]);
    if (lane == 0)
    {
#pragma unroll
        for (int kk = 0; kk < 16; ++kk)
            red[wid][col + kk] = v[kk];
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk)
    {
        double t = 0.;
        for (int w = 0; w < NW; ++w)
            t += red[w][col + kk];
        v[kk] = t;
    }
    __syncthreads();
}

// The beta rates of a point in the units of the pair/brem sums (s2d, unit
// t2 = (2.182 T)^2 for number and t2d t2 for energy moments) or, with
// to_nes, of the NES sums (unit hn = 8 t2, times T for energy moments), as
// the final assembly combines them (m1_opacities.hpp:1172-1294).
__device__ __forceinline__ void beta_in_sum_units(const PointTab* P, double T, double eta_e,
                                                  bool use_abs_em, bool to_nes, double* b)
{
#pragma unroll
    for (int kk = 0; kk < 16; ++kk)
        b[kk] = 0.;
    if (!use_abs_em)
        return;
    double fe[2][6];
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int kk = 0; kk < 6; ++kk)
            fe[e][kk] = P->fe[e][kk];
    double sb[2];
    beta_scales(T, eta_e, fe, sb);
    const double t2d = k::TempMultiple * T, t2 = t2d * t2d;
    const double un  = k::FourPiHc3 * (to_nes ? 8. * t2 : t2);
    const double ue  = to_nes ? un : un * t2d;
#pragma unroll
    for (int s = 0; s < 2; ++s)
    {
        b[s]      = P->sbeta[s] * sb[s] / un;     // number emission
        b[4 + s]  = P->sbeta[4 + s] * sb[s] / un; // number absorption
        b[8 + s]  = P->sbeta[2 + s] * sb[s] / ue; // energy emission
        b[12 + s] = P->sbeta[6 + s] * sb[s] / ue; // energy absorption
    }
}

// Mixed sums whose terms cancel by more than this are recomputed in FP64: the
// FP32 rounding of each term (a few 1e-7) must stay below 1e-6 in the result.
constexpr double kMaxCancel = 2.0;
// FP32 brem cells carry up to ~6e-7 per term (the HR98 fit in FP32).
constexpr double kMaxCancelBrem = 1.25;
// FP32 pair integrals carry up to ~3e-7 per cell.
constexpr double kMaxCancelPair = 1.5;
// The accurate (all-df) pass keeps ~1e-13 per term.
constexpr double kMaxCancelDf = 1e5;

// add_cell in FP32 for a species-independent kernel (brem): K_em, K_ab are
// dimensionless; P1 = (y_a y_b)^2 W1 and P2 = (y_a y_b)^2 W2 are the cell's
// weights with the energy factor, each one FP32 rounding of a double-float
// product (cell_weight); the caller scales by T^4 and the kernel's prefactor.
template <bool STIM>
__device__ __forceinline__ void add_cell32(Acc32& A, float Kem, float Kab, const float* ga,
                                           const float* gma, const float* gb, const float* gmb,
                                           bool nb_block, float P1, float P2)
{
#pragma unroll
    for (int s = 0; s < 4; ++s)
    {
        const int ps   = s ^ 1;
        const float em = Kem * (nb_block ? 1.f : gmb[ps]);
        const float am = Kab * gb[ps];
        float EM, AB;
        if (STIM)
        {
            AB = ga[s] * (em + am);
            EM = em;
        }
        else
        {
            AB = am * ga[s];
            EM = em * gma[s];
        }
        const float e1 = EM * P1, a1 = AB * P1;
        A.v[s] += e1;
        A.v[4 + s] += a1;
        const float e2 = EM * P2, a2 = AB * P2;
        A.v[8 + s] += e2;
        A.v[12 + s] += a2;
        A.mag[s] += fabsf(e1);
        A.mag[4 + s] += fabsf(a1);
        A.mag[8 + s] += fabsf(e2);
        A.mag[12 + s] += fabsf(a2);
    }
}

// (y_a y_b)^2 w_a w_b rounded once to FP32 from double-float factors (in
// FP32 the fourth power alone magnified the rounding of y to 3e-7).
__device__ __forceinline__ float cell_weight(dfm::df w4, dfm::df wa, dfm::df wb)
{
    const dfm::df p = dfm::mul(w4, dfm::mul(wa, wb));
    return p.hi + p.lo;
}

// FP32 tables of one point from the FP64 ones.
__device__ __forceinline__ void fill_tab32(CellTab32& D, const CellTab& C, int M, int lane)
{
    for (int e = lane; e < 4 * M; e += 32)
    {
        const double gv     = C.g[e >> 2][e & 3];
        D.g[e >> 2][e & 3]  = (float)gv;
        D.gm[e >> 2][e & 3] = (float)(1. - gv);
    }
    for (int a = lane; a < M; a += 32)
    {
        const dfm::df yd = dfm::from_double(C.y[a]);
        D.yh[a]          = yd.hi;
        D.yl[a]          = yd.lo;
    }
}

// Weight algebra of add_cell for the mixed pair cells, with w4 = 1 (the
// caller folds (nu nubar)^2 into the kernel) and the emission terms'
// magnitudes: the pair kernels are non-negative and so are the absorption
// terms (em + am = em (1 + g (e^s - 1)) >= 0), so only the emission terms,
// through 1 - g < 0, can carry the opposite sign.
template <bool STIM>
__device__ __forceinline__ void add_cell_pair(double* acc, double* magem, const double* Kem,
                                              const double* Kab, const double* ga,
                                              const double* gb, bool nb_block, double W1,
                                              double W2)
{
#pragma unroll
    for (int s = 0; s < 4; ++s)
    {
        const int ps    = s ^ 1;
        const double bf = nb_block ? 1. : 1. - gb[ps];
        const double em = Kem[s] * bf;
        const double am = Kab[s] * gb[ps];
        double EM, AB, EMA;
        if (STIM)
        {
            AB  = ga[s] * (em + am);
            EM  = em;
            EMA = Kem[s] * fabs(bf);
        }
        else
        {
            AB  = am * ga[s];
            EM  = em * (1. - ga[s]);
            EMA = Kem[s] * fabs(bf) * fabs(1. - ga[s]);
        }
        acc[s] += EM * W1;
        acc[4 + s] += AB * W1;
        acc[8 + s] += EM * W2;
        acc[12 + s] += AB * W2;
        magem[s] += EMA * W1;
        magem[4 + s] += EMA * W2;
    }
}

// Per-warp node tables of the mixed pair phase: y = nu/T as double-float,
// e^{y - |eta|/2} (e^{Lref} = its product over the two nodes when |eta| >= s)
// and e^{-y} (e^{-s} = the product when s <= 700).
struct PairTab32
{
    float yh[kMaxM], yl[kMaxM];
    double eh[kMaxM], dn[kMaxM];
};

// Pair cell (a, b) of the mixed path from the per-warp node tables
// (pair32::kernel_q).
__device__ __forceinline__ void pair_kernel_q(const PairTab32& X, int a, int b, dfm::df ETA,
                                              double sc, double* em, double* ab)
{
    pair32::kernel_q(dfm::df{X.yh[a], X.yl[a]}, dfm::df{X.yh[b], X.yl[b]}, X.eh[a], X.eh[b],
                     X.dn[a], X.dn[b], ETA, sc, em, ab);
}

// MIXED: pair cells from the FP32 integral; the sums, their magnitudes and
// s2d are written to the record (PairMixed).  !MIXED: the FP64 pair kernel
// (kernel_pair.hpp), with redo_only the mixed path's second pass over the
// points the final kernel marked (predo), whose pair part of s2d it replaces;
// that pass computes its Fermi-integral tables itself.  WIDE (that pass):
// a point per CTA, its cells over all threads (the marked points are few).
template <bool MIXED, bool WIDE = false, bool MULTI = false>
__global__ void __launch_bounds__((WIDE ? 8 : kWarps) * 32)
    grey_pair_kernel(const __grid_constant__ OpacityLaunch L0, const GroupArgs GA, int64_t p0,
                     int64_t np, double* __restrict__ scratch, int redo_only)
{
    const OpacityLaunch& L = MULTI ? GA.Ls[blockIdx.z] : L0;
    if (MULTI)
    {
        const GroupChunk& gcz = GA.gc[blockIdx.z];
        p0      = gcz.p0;
        np      = gcz.np;
        scratch = gcz.ws;
    }
    if (MULTI && !L.use_pair)
        return; // a group without pair (uniform over the CTA)
    constexpr int NW = WIDE ? 8 : kWarps;
    __shared__ double s_A1[kMaxM], s_A2[kMaxM];
    __shared__ uint32_t s_cells[kMaxCells];
    __shared__ CellTab s_ct[WIDE ? 1 : kWarps];
    __shared__ PairTab32 s_pt[MIXED ? kWarps : 1];
    __shared__ double s_red[WIDE ? NW : 1][32];
    for (int k = threadIdx.x; k < kMaxM; k += blockDim.x)
    {
        s_A1[k]  = L.A1[k];
        s_A2[k]  = L.A2[k];
    }
    for (int k = threadIdx.x; k < L.ncell; k += blockDim.x)
        s_cells[k] = L.cells[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wid  = threadIdx.x >> 5;
    CellTab& C     = s_ct[WIDE ? 0 : wid];
    PairTab32& X   = s_pt[MIXED ? wid : 0];
    const int M    = 2 * L.n2;
    const bool nbb = L.neglect_blocking != 0;
    // cells of a point: thread t0, t0 + stride, ...
    const int t0        = WIDE ? (int)threadIdx.x : lane;
    const int stride    = WIDE ? NW * 32 : 32;
    const int64_t q0    = WIDE ? (int64_t)blockIdx.x : (int64_t)blockIdx.x * NW + wid;
    const int64_t qstep = WIDE ? (int64_t)gridDim.x : (int64_t)gridDim.x * NW;

    for (int64_t q = q0; q < np; q += qstep)
    {
        const int64_t p  = L.pidx ? L.pidx[p0 + q] : p0 + q;
        PointTab* P      = (PointTab*)(scratch + q * kTabWords);
        if (!MIXED && redo_only && pair_mixed(P)->predo != 1.)
            continue;
        const double T   = L.eos[1][p];
        const double eta = L.eos[7][p] / T;
        if (WIDE)
            __syncthreads(); // the previous point's readers are done
        else
            __syncwarp();
        if (!WIDE || wid == 0)
            load_cell_tab(C, P, M, !MIXED && !redo_only, lane);
        if (WIDE)
            __syncthreads();
        if (MIXED)
        {
            __syncwarp();
            for (int a = lane; a < M; a += 32)
            {
                const double y = C.y[a];
                const dfm::df yd = dfm::from_double(y);
                X.yh[a] = yd.hi;
                X.yl[a] = yd.lo;
                X.eh[a] = exp(y - 0.5 * fabs(eta));
                X.dn[a] = exp(-y);
            }
        }
        if (!MIXED && redo_only)
        {
            // the F_1..F_5 tables the mixed prelude left out
            for (int qq = t0; qq < 2 * M; qq += stride)
            {
                const int a = qq >> 1;
                if (qq & 1)
                    fdi_orders<1, 5>(eta + C.y[a], C.fp[a]);
                else
                    fdi_orders<1, 5>(eta - C.y[a], C.fm[a]);
            }
        }
        if (WIDE)
            __syncthreads();
        else
            __syncwarp();
        double acc[16], magem[MIXED ? 8 : 1];
#pragma unroll
        for (int kk = 0; kk < 16; ++kk)
            acc[kk] = 0.;
#pragma unroll
        for (int kk = 0; kk < (MIXED ? 8 : 1); ++kk)
            magem[kk] = 0.;
        const dfm::df ETA = dfm::from_double(eta);
        const double T2 = T * T;
        const double scq = 0.5 * k::PairPhi * T2 * (T2 * T2) / 15.;
        for (int c = t0; c < L.ncell; c += stride)
        {
            const uint32_t ab = s_cells[c];
            const int a = ab & 0xffffu, b = ab >> 16;
            const double nua = C.nu[a], nub = C.nu[b];
            double pe[4], pa[4];
            if (MIXED)
                pair_kernel_q(X, a, b, ETA, scq, pe, pa);
            else
                pair_kernel(T, eta, nua, nub, C.y[a], C.y[b], C.fm[a], C.fp[a], C.fm[b],
                            C.fp[b], C.f3e, C.f4e, pe, pa);
            const double w4 = (nua * nua) * (nub * nub);
            const double W1 = s_A1[a] * s_A1[b];
            // (b, a): the inverse kernel swaps partner species (kernel_pair.hpp:200-216)
            const double qe[4] = {pe[1], pe[0], pe[3], pe[2]};
            const double qa[4] = {pa[1], pa[0], pa[3], pa[2]};
            if (MIXED)
            {
                if (L.stim)
                    add_cell_pair<true>(acc, magem, pe, pa, C.g[a], C.g[b], nbb, W1,
                                        s_A2[a] * s_A1[b]);
                else
                    add_cell_pair<false>(acc, magem, pe, pa, C.g[a], C.g[b], nbb, W1,
                                         s_A2[a] * s_A1[b]);
                if (a != b)
                {
                    if (L.stim)
                        add_cell_pair<true>(acc, magem, qe, qa, C.g[b], C.g[a], nbb, W1,
                                            s_A2[b] * s_A1[a]);
                    else
                        add_cell_pair<false>(acc, magem, qe, qa, C.g[b], C.g[a], nbb, W1,
                                             s_A2[b] * s_A1[a]);
                }
            }
            else
            {
                if (L.stim)
                    add_cell<true>(acc, pe, pa, C.g[a], C.g[b], nbb, w4, W1, s_A2[a] * s_A1[b]);
                else
                    add_cell<false>(acc, pe, pa, C.g[a], C.g[b], nbb, w4, W1, s_A2[a] * s_A1[b]);
                if (a != b)
                {
                    if (L.stim)
                        add_cell<true>(acc, qe, qa, C.g[b], C.g[a], nbb, w4, W1,
                                       s_A2[b] * s_A1[a]);
                    else
                        add_cell<false>(acc, qe, qa, C.g[b], C.g[a], nbb, w4, W1,
                                        s_A2[b] * s_A1[a]);
                }
            }
        }
        double magd[16];
        if (WIDE)
            block_sum<NW>(acc, s_red, 0);
        else
        {
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                acc[kk] = warp_sum(acc[kk]);
        }
        if (MIXED)
        {
            // emission moments: sum of |term|; absorption terms are non-negative
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                magd[s]      = warp_sum(magem[s]);
                magd[8 + s]  = warp_sum(magem[4 + s]);
                magd[4 + s]  = fabs(acc[4 + s]);
                magd[12 + s] = fabs(acc[12 + s]);
            }
        }
        if (WIDE ? threadIdx.x == 0 : lane == 0)
        {
            PairMixed* X = pair_mixed(P);
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
            {
                if (MIXED)
                {
                    P->s2d[kk]   = acc[kk];
                    X->spair[kk] = acc[kk];
                    X->pmag[kk]  = magd[kk];
                }
                else if (redo_only)
                    P->s2d[kk] = P->s2d[kk] - X->spair[kk] + acc[kk];
                else
                    P->s2d[kk] = acc[kk];
            }
            if (MIXED)
                X->predo = 0.;
        }
    }
}

// Per-warp GP19 state of the brem kernel.
struct Gp19Warp
{
    Gp19Point pt;
    Gp19Corners cor[2];
    double p[2][kGp19MaxW];
    float pf[2][kGp19MaxW];
};

// IMPL: 0 HR98, 1 BRT06, 2 GP19.  ADD: accumulate onto the pair sums.
// WIDE (the mixed path's FP64 pass over the few marked points): a point per
// CTA, its cells over all threads.
template <bool MIXED, int IMPL, bool WIDE = false, bool MULTI = false>
__global__ void __launch_bounds__((WIDE ? 8 : kWarps) * 32)
    grey_brem_kernel(const __grid_constant__ OpacityLaunch L0, const GroupArgs GA, int64_t p0,
                     int64_t np, double* __restrict__ scratch, int add, int redo_only)
{
    const OpacityLaunch& L = MULTI ? GA.Ls[blockIdx.z] : L0;
    if (MULTI)
    {
        const GroupChunk& gcz = GA.gc[blockIdx.z];
        p0      = gcz.p0;
        np      = gcz.np;
        scratch = gcz.ws;
    }
    if (MULTI)
    {
        if (!L.use_brem || L.brem_impl != IMPL)
            return; // another brem variant's launch serves this group
        add = L.use_pair;
    }
    constexpr int NW = WIDE ? 8 : kWarps;
    constexpr int NT = WIDE ? 1 : kWarps; // point tables in flight per CTA
    __shared__ double s_A1[kMaxM], s_A2[kMaxM];
    __shared__ dfm::df s_A1d[MIXED ? kMaxM : 1], s_A2d[MIXED ? kMaxM : 1];
    __shared__ uint32_t s_cells[kMaxCells];
    __shared__ CellTab s_ct[NT];
    __shared__ CellTab32 s_c32[MIXED ? kWarps : 1];
    __shared__ Gp19Warp s_gw[IMPL == 2 ? NT : 1];
    __shared__ double s_red[WIDE ? NW : 1][32];
    __shared__ double s_lw[IMPL == 2 ? kGp19MaxW : 1];
    __shared__ float s_lwf[IMPL == 2 ? kGp19MaxW : 1];
    constexpr int kWF = (IMPL == 2 && MIXED) ? kGp19MaxW : 1;
    __shared__ double s_wax[kWF], s_iw[kWF];
    __shared__ float s_idl[kWF];
    const Gp19Table G19 = {L.gp19.d0, L.gp19.d1, L.gp19.d2,    L.gp19.d3,   L.gp19.nb,  L.gp19.ye,
                           L.gp19.t,  L.gp19.w,  L.gp19.lognb, L.gp19.logw, L.gp19.data};
    const bool prof = IMPL == 2 && G19.d3 <= kGp19MaxW;
    for (int k = threadIdx.x; k < kMaxM; k += blockDim.x)
    {
        s_A1[k] = L.A1[k];
        s_A2[k] = L.A2[k];
        if (MIXED)
        {
            s_A1d[k] = dfm::from_double(L.A1[k]);
            s_A2d[k] = dfm::from_double(L.A2[k]);
        }
    }
    for (int k = threadIdx.x; k < L.ncell; k += blockDim.x)
        s_cells[k] = L.cells[k];
    if (IMPL == 2 && prof)
        for (int k = threadIdx.x; k < G19.d3; k += blockDim.x)
        {
            s_lw[k]  = G19.logw[k];
            s_lwf[k] = (float)G19.logw[k];
            if (MIXED)
            {
                s_wax[k] = G19.w[k];
                s_iw[k]  = 1. / G19.w[k];
                s_idl[k] = k + 1 < G19.d3 ? (float)(1. / (G19.logw[k + 1] - G19.logw[k])) : 0.f;
            }
        }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wid  = threadIdx.x >> 5;
    CellTab& C     = s_ct[WIDE ? 0 : wid];
    const int M    = 2 * L.n2;
    const bool nbb = L.neglect_blocking != 0;
    // cells of a point: thread t0, t0 + stride, ...
    const int t0        = WIDE ? (int)threadIdx.x : lane;
    const int stride    = WIDE ? NW * 32 : 32;
    const int64_t q0    = WIDE ? (int64_t)blockIdx.x : (int64_t)blockIdx.x * NW + wid;
    const int64_t qstep = WIDE ? (int64_t)gridDim.x : (int64_t)gridDim.x * NW;
    const double wmin = IMPL == 2 ? G19.w[0] : 0., wmax = IMPL == 2 ? G19.w[G19.d3 - 1] : 0.;

    for (int64_t q = q0; q < np; q += qstep)
    {
        const int64_t p = L.pidx ? L.pidx[p0 + q] : p0 + q;
        PointTab* P     = (PointTab*)(scratch + q * kTabWords);
        if (redo_only && P->bredo != 1.)
            continue; // uniform: one point per warp (per CTA when WIDE)
        const double T  = L.eos[1][p];
        if (WIDE)
            __syncthreads(); // the previous point's readers are done
        else
            __syncwarp();
        if (!WIDE || wid == 0)
        {
            load_cell_tab(C, P, M, false, lane);
            if (IMPL == 0)
                warp_copy((double*)&C.hr, (const double*)&P->hr,
                          sizeof(Hr98Point) / sizeof(double), lane);
        }
        if (WIDE)
            __syncthreads();
        else
            __syncwarp();
        if (IMPL == 0 && MIXED && lane == 0)
            fp32::hr98_mixed_from(C.hr, &C.hm);
        const double nbp = L.eos[0][p], yep = L.eos[2][p];
        Gp19Warp& GW     = s_gw[IMPL == 2 && !WIDE ? wid : 0];
        if (IMPL == 2 && prof)
        {
            if (WIDE ? threadIdx.x == 0 : lane == 0)
                gp19_point(G19, nbp, yep, T, &GW.pt);
            if (WIDE)
                __syncthreads();
            else
                __syncwarp();
            const int np19 = (GW.pt.regime >= 2) ? 2 : 1;
            if (t0 < np19)
                gp19_profile_corners(G19, GW.pt.nbp, GW.pt.yep, GW.pt.pT[t0], &GW.cor[t0]);
            if (WIDE)
                __syncthreads();
            else
                __syncwarp();
            for (int e = t0; e < np19 * G19.d3; e += stride)
            {
                const int pr = e / G19.d3, l = e - pr * G19.d3;
                const double v = gp19_profile_eval(G19, GW.cor[pr], l);
                GW.p[pr][l]  = v;
                GW.pf[pr][l] = (float)v;
            }
            if (WIDE)
                __syncthreads();
            else
                __syncwarp();
        }
        // Mixed cells in FP32 except the GP19 high-T extrapolation (which
        // differences two table values); points whose cells the other
        // reactions cancel go to FP64 below (the guard).
        const bool fp32_cells =
            MIXED && (IMPL == 0 || IMPL == 1 ||
                      (IMPL == 2 && prof && GW.pt.regime != 3 && GW.pt.regime != 5));
        double acc[16], bm[16];
#pragma unroll
        for (int kk = 0; kk < 16; ++kk)
            acc[kk] = bm[kk] = 0.;
        bool redo = false;
        if (fp32_cells)
        {
            CellTab32& D = s_c32[MIXED ? wid : 0];
            fill_tab32(D, C, M, lane);
            __syncwarp();
            double scale = (T * T) * (T * T);
            float thr = 0.f, lt2 = 0.f;
            if (IMPL == 0)
                scale *= C.hm.outer;
            else if (IMPL == 1)
                scale *= C.brt06_pre;
            else
            {
                scale *= 3. * GW.pt.C;
                thr = (float)(1e-30 / GW.pt.C);
                lt2 = (float)log2(T * 0.5);
            }
            Acc32 A;
            A.clear();
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                A.mag[kk] = 0.f;
            int pending = 0;
            for (int c = lane; c < L.ncell; c += 32)
            {
                const uint32_t ab = s_cells[c];
                const int a = ab & 0xffffu, b = ab >> 16;
                // x = (nu_a + nu_b) / T as hi + lo (accurate exponent)
                const dfm::df xs = dfm::add(dfm::df{D.yh[a], D.yl[a]}, dfm::df{D.yh[b], D.yl[b]});
                const float ex = expf(-xs.hi) * (1.f - xs.lo);
                float Kab;
                bool slow = false;
                if (IMPL == 0)
                    Kab = fp32::hr98_shape(C.hm, xs.hi, xs.lo);
                else if (IMPL == 1)
                {
                    // BRT06 (kernel_brem_BRT06.hpp:24-69): ab = pre K_1(x) e^{x} / x,
                    // x = (nu_a + nu_b) / 2T; em = ab e^{-2x}
                    const float xh = 0.5f * (xs.hi + xs.lo);
                    Kab            = fp32::bessk1e(xh) / xh;
                }
                else
                {
                    double wv = C.nu[a] + C.nu[b];
                    wv        = wv > wmax ? wmax : (wv < wmin ? wmin : wv);
                    float tw;
                    const int l = gp19_bracket32(wv, s_lwf, s_wax, s_iw, s_idl, G19.d3, &tw);
                    const float v0 = GW.pf[0][l] + tw * (GW.pf[0][l + 1] - GW.pf[0][l]);
                    if (GW.pt.regime <= 1)
                        Kab = v0;
                    else
                    {
                        const float v1 = GW.pf[1][l] + tw * (GW.pf[1][l + 1] - GW.pf[1][l]);
                        Kab = v0 * exp2f(log2f(v1 / v0) * lt2);
                        // regime 2 clips k2, k4 and s at 1e-30 (rare: exact FP64 cell)
                        slow = GW.pt.regime == 2 && (v0 < thr || v1 < thr || Kab < thr);
                    }
                    Kab = fabsf(Kab);
                }
                float Kem = Kab * ex;
                if (IMPL == 2 && slow)
                {
                    const double nua = C.nu[a], nub = C.nu[b];
                    double w = nua + nub;
                    w        = w > wmax ? wmax : (w < wmin ? wmin : w);
                    double tw;
                    const int l = bracket_sorted<double>(log(w), s_lw, G19.d3, &tw);
                    const double v0 = GW.p[0][l] * (1. - tw) + GW.p[0][l + 1] * tw;
                    const double v1 = GW.p[1][l] * (1. - tw) + GW.p[1][l + 1] * tw;
                    double em, abv;
                    gp19_cell(GW.pt, v0, v1, w, nua + nub, &em, &abv);
                    Kab = (float)(abv / (3. * GW.pt.C));
                    Kem = (float)(em / (3. * GW.pt.C));
                }
                const dfm::df yab = dfm::mul(dfm::df{D.yh[a], D.yl[a]}, dfm::df{D.yh[b], D.yl[b]});
                const dfm::df w4  = dfm::mul(yab, yab); // (y_a y_b)^2
                const float P1    = cell_weight(w4, s_A1d[a], s_A1d[b]);
                const float P2    = cell_weight(w4, s_A2d[a], s_A1d[b]);
                if (L.stim)
                    add_cell32<true>(A, Kem, Kab, D.g[a], D.gm[a], D.g[b], D.gm[b], nbb, P1, P2);
                else
                    add_cell32<false>(A, Kem, Kab, D.g[a], D.gm[a], D.g[b], D.gm[b], nbb, P1, P2);
                if (a != b)
                {
                    const float P2r = cell_weight(w4, s_A2d[b], s_A1d[a]);
                    if (L.stim)
                        add_cell32<true>(A, Kem, Kab, D.g[b], D.gm[b], D.g[a], D.gm[a], nbb, P1,
                                         P2r);
                    else
                        add_cell32<false>(A, Kem, Kab, D.g[b], D.gm[b], D.g[a], D.gm[a], nbb, P1,
                                          P2r);
                }
                if (++pending == 4)
                {
#pragma unroll
                    for (int kk = 0; kk < 16; ++kk)
                        acc[kk] += (double)A.v[kk];
                    A.clear();
                    pending = 0;
                }
            }
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                acc[kk] = acc[kk] + (double)A.v[kk];
            // cells of both signs (occupation above 1 makes 1 - g negative), or
            // a brem sum cancelling the pair sum or the beta rates: recompute
            // this point in FP64
            double other[16];
            beta_in_sum_units(P, T, L.eos[7][p] / T, L.use_abs_em, false, other);
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                other[kk] += add ? P->s2d[kk] : 0.;
            redo = cancel_factor(acc, A.mag, scale, scale, other) > kMaxCancelBrem;
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
            {
                acc[kk] = redo ? 0. : acc[kk] * scale;
                bm[kk]  = redo ? 0. : warp_sum((double)A.mag[kk]) * scale;
            }
        }
        if (!fp32_cells || redo)
        {
            for (int c = t0; c < L.ncell; c += stride)
            {
                const uint32_t ab = s_cells[c];
                const int a = ab & 0xffffu, b = ab >> 16;
                const double nua = C.nu[a], nub = C.nu[b];
                double be, ba;
                if (IMPL == 0)
                    hr98_kernel(C.hr, nua, nub, &be, &ba);
                else if (IMPL == 1)
                    brt06_kernel(C.brt06_pre, T, nua, nub, &be, &ba);
                else if (prof)
                {
                    double w = nua + nub;
                    w        = w > wmax ? wmax : (w < wmin ? wmin : w);
                    double tw;
                    const int l = bracket_sorted<double>(log(w), s_lw, G19.d3, &tw);
                    const double v0 = GW.p[0][l] * (1. - tw) + GW.p[0][l + 1] * tw;
                    const double v1 =
                        GW.pt.regime >= 2 ? GW.p[1][l] * (1. - tw) + GW.p[1][l + 1] * tw : 0.;
                    gp19_cell(GW.pt, v0, v1, w, nua + nub, &be, &ba);
                }
                else
                    gp19_kernel(G19, nbp, yep, T, nua, nub, &be, &ba);
                const double Kem[4] = {be, be, be, be};
                const double Kab[4] = {ba, ba, ba, ba};
                const double w4 = (nua * nua) * (nub * nub);
                const double W1 = s_A1[a] * s_A1[b];
                if (L.stim)
                    add_cell<true>(acc, Kem, Kab, C.g[a], C.g[b], nbb, w4, W1, s_A2[a] * s_A1[b]);
                else
                    add_cell<false>(acc, Kem, Kab, C.g[a], C.g[b], nbb, w4, W1, s_A2[a] * s_A1[b]);
                if (a != b)
                {
                    if (L.stim)
                        add_cell<true>(acc, Kem, Kab, C.g[b], C.g[a], nbb, w4, W1,
                                       s_A2[b] * s_A1[a]);
                    else
                        add_cell<false>(acc, Kem, Kab, C.g[b], C.g[a], nbb, w4, W1,
                                        s_A2[b] * s_A1[a]);
                }
            }
        }
        if (WIDE)
            block_sum<NW>(acc, s_red, 0);
        else
        {
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                acc[kk] = warp_sum(acc[kk]);
        }
        if (WIDE ? threadIdx.x == 0 : lane == 0)
        {
            // a redo replaces the FP32 brem part of s2d by the FP64 one
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
            {
                const double base = add ? (redo_only ? P->s2d[kk] - P->sbrem[kk] : P->s2d[kk]) : 0.;
                P->s2d[kk]   = base + acc[kk];
                P->sbrem[kk] = acc[kk];
                P->bmag[kk]  = bm[kk];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// NES / NPS (m1_opacities.hpp:864-1057, integration.hpp:687-768)
// ---------------------------------------------------------------------------
struct NepsTab
{
    Distr d;
    double fe[2][6];
    double fd0[2];
    double same_cf;
};

// Energies of NES item (r, i, j) (m1_opacities.hpp:880-905).
__device__ __forceinline__ void neps_energies(int r, double xi, double xj, double tn, double* nu,
                                              double* nub)
{
    if (!r)
    {
        *nu  = 0.5 * tn * xi * (1. - xj);
        *nub = 0.5 * tn * xi * (1. + xj);
    }
    else
    {
        *nu  = 0.5 * tn * (1. - xj) / xi;
        *nub = 0.5 * tn * (1. + xj) / xi;
    }
}

// The FP64 item sums of one point (the plain path, and the mixed path's
// fallback for points outside the FP32 range envelope).
__device__ __forceinline__ void neps_items_fp64(const NepsPoint& NP, const Distr& d, bool same_cf,
                                                int n2, double tn, bool stim, bool nbb,
                                                const double* s_x2, const double* s_w2,
                                                const double* s_wx, const double* s_wx3,
                                                int t0, int stride, double* acc)
{
    const int nn2 = n2 * n2;
    for (int it = t0; it < 2 * nn2; it += stride)
    {
        const int r   = it >= nn2;
        const int rem = it - r * nn2;
        const int i = rem / n2, j = rem - (rem / n2) * n2;
        double nu, nub;
        neps_energies(r, s_x2[i], s_x2[j], tn, &nu, &nub);
        const double w4 = (nu * nu) * (nub * nub);
        double g[4], gb[4];
        total_nu_f4(nu, d, same_cf, g);
        total_nu_f4(nub, d, same_cf, gb);
        double em1[4], ab1[4], em2[4], ab2[4];
        neps_pair(NP, nu, nub, em1, ab1, em2, ab2);
        const double Wr = (r ? s_wx3[i] : s_wx[i]) * s_w2[j];
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            const double e1 = em1[s] * gb[s];
            const double a1 = ab1[s] * (nbb ? 1. : 1. - gb[s]);
            const double e2 = em2[s] * g[s];
            const double a2 = ab2[s] * (nbb ? 1. : 1. - g[s]);
            double EM1, AB1, EM2, AB2;
            if (stim)
            {
                AB1 = w4 * g[s] * (e1 + a1);
                EM1 = w4 * e1;
                AB2 = w4 * gb[s] * (e2 + a2);
                EM2 = w4 * e2;
            }
            else
            {
                AB1 = w4 * g[s] * a1;
                EM1 = w4 * (1. - g[s]) * e1;
                AB2 = w4 * gb[s] * a2;
                EM2 = w4 * (1. - gb[s]) * e2;
            }
            acc[s] += Wr * (EM1 + EM2);
            acc[4 + s] += Wr * (AB1 + AB2);
            acc[8 + s] += Wr * (nu * EM1 + nub * EM2);
            acc[12 + s] += Wr * (nu * AB1 + nub * AB2);
        }
    }
}

// TotalNuF and 1 - TotalNuF in df (the accurate pass of the mixed path).
__device__ __forceinline__ void total_nu_df(double omega, double lw, const NepsMixed& Q,
                                            const double* wt, const double* wf, dfm::df* g,
                                            dfm::df* gm)
{
    using namespace dfm;
#pragma unroll 1
    for (int s = 0; s < 4; ++s)
    {
        const double arg = fma(omega, Q.invTt[s], -Q.etat[s]);
        const df t       = exp_df(from_double(-fabs(arg)));
        const df inv     = div(mk(1.f), add(t, 1.f));
        const df ti      = mul(t, inv);
        const df ft = arg > 0. ? ti : inv, ftm = arg > 0. ? inv : ti;
        const df fn = exp_df(from_double(fma(Q.cf[s], lw, fma(-omega, Q.invTf[s], Q.lbf[s]))));
        const df Wt = from_double(wt[s]), Wf = from_double(wf[s]);
        g[s]  = add(mul(Wt, ft), mul(Wf, fn));
        gm[s] = add(mul(Wt, ftm), mul(Wf, add(neg(fn), 1.f)));
    }
}

// NEPSExpFunc in df.
__device__ __forceinline__ dfm::df neps_exp_df(double d, bool negd)
{
    using namespace dfm;
    const df e  = exp_df(from_double(-fabs(d)));
    const df dn = add(add(neg(e), 1.f), d == 0. ? 1.f : 0.f);
    return div(negd ? mk(1.f) : neg(e), dn);
}

// neps_item_mixed with every product after the Fermi integrals in df.
__device__ __forceinline__ void neps_item_df(const NepsPoint& P, const NepsMixed& Q,
                                             const dfm::FdiTab* ftab, double w, double wp,
                                             dfm::df* em1, dfm::df* ab1, dfm::df* em2,
                                             dfm::df* ab2)
{
    using namespace dfm;
    const double x = (w > wp) ? w : wp;
    const double y = (w < wp) ? w : wp;
    const double d1 = wp - w, d2 = w - wp;
    const bool n1 = signbit(d1) != 0, n2 = signbit(d2) != 0;
    const df efa = neps_exp_df(d1, n1);
    const df efb = neps_exp_df(d2, n2);
    const float sign1 = n1 ? 1.f : -1.f;
    const float sign2 = n2 ? 1.f : -1.f;
#pragma unroll
    for (int s = 0; s < 4; ++s)
        em1[s] = ab1[s] = em2[s] = ab2[s] = {0.f, 0.f};
    const df W  = from_double(w), WP = from_double(wp);
    const df S  = add(W, WP);
    const df Pp = mul(W, WP);
    const df Dn = mul(Pp, Pp);
    const df iDn = div(mk(1.f), Dn); // the four brackets per lepton share 1 / Dn
    const df X  = from_double(x), Y = from_double(y);
    // e+ terms scale as e^{-eta_e}: below 1e-13 of the e- terms for eta_e > 30
    const int nlep = P.eta0 > 30. ? 1 : 2;
#pragma unroll 1
    for (int e = 0; e < nlep; ++e)
    {
        const double eta = e ? P.eta1 : P.eta0;
        df r1[4], r2[4];
        if (y > eta * 1e-3)
        {
            const df aw = from_double(eta - w), awp = from_double(eta - wp);
            const double adw = fabs(w - wp);
            const df aab = from_double(eta - adw);
            df rw[5], rwp[5], rab[5];
            fdi_raw15(aw, rw, 1, ftab);
            fdi_raw15(awp, rwp, 1, ftab);
            fdi_raw15(aab, rab, 3, ftab); // only F_3..F_5 enter through |w - w'|
            rab[0] = rab[1] = Q.reta[e][0]; // unused orders: keep the arrays defined
            df dw[5], d5[5];
            fdi_diff15(rw, rwp, aw, awp, from_double(w - wp), dw);
            fdi_diff15(rab, Q.reta[e], aab, Q.eta[e], from_double(adw), d5);
            const df dabs[3] = {d5[2], d5[3], d5[4]};
            const df T1 = add(dw[3], mul(add(mul(S, dw[2]), mul(mul(Pp, 3.f), dw[1])), 2.f));
            const df U  = add(mul(X, dabs[1]), mul(mul(mul(X, X), 2.f), dabs[0]));
            const df V  = add(neg(mul(Y, dabs[1])), mul(mul(mul(Y, Y), 2.f), dabs[0]));
            const df ST = mul(S, T1);
            constexpr dfc kFifth(0.2);
            const df dd2 = mul(dabs[2], mk(kFifth)), dw4 = mul(dw[4], mk(kFifth));
            const df c1 = sub(mul(dd2, sign1), dw4);
            const df c2 = add(mul(dd2, sign2), dw4);
            const df s6 = mul(dw[0], 6.f);
            const df A1 = sub(mul(add(sub(c1, ST), mul(U, sign1)), iDn), s6);
            const df B1 = mul(add(c1, mul(V, sign1)), iDn);
            const df A2 = add(mul(add(add(c2, ST), mul(U, sign2)), iDn), s6);
            const df B2 = mul(add(c2, mul(V, sign2)), iDn);
            constexpr dfc kBp(k::NepsBPlus), kBm(k::NepsBMinus), kBz(k::NepsBZero);
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                const df bo      = (s < 2) ? mk(kBp) : mk(kBm);
                const bool first = ((s & 1) == 0) != (e == 1);
                r1[s] = first ? add(mul(A1, bo), mul(B1, mk(kBz))) : add(mul(A1, mk(kBz)), mul(B1, bo));
                r2[s] = first ? add(mul(A2, bo), mul(B2, mk(kBz))) : add(mul(A2, mk(kBz)), mul(B2, bo));
            }
        }
        else
        {
            double t1[4], t2[4];
            neps_taylor(P, e, w, wp, x, y, (int)sign1, (int)sign2, t1, t2);
#pragma unroll
            for (int s = 0; s < 4; ++s)
            {
                r1[s] = from_double(t1[s]);
                r2[s] = from_double(t2[s]);
            }
        }
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            em1[s] = sub(em1[s], mul(r1[s], efb));
            ab1[s] = add(ab1[s], mul(r1[s], efa));
            em2[s] = sub(em2[s], mul(r2[s], efa));
            ab2[s] = add(ab2[s], mul(r2[s], efb));
        }
    }
}

// NES launch modes.  The plain path runs kNesFp64All.  The mixed path runs
// three launches per chunk, each over all points but working only on its own:
//   grey_nes_fast_kernel  FP32 kernel integrals (bnsn_nes32.cuh); flags a
//                 point 1 when its sums cancel (terms of both signs, or
//                 negative pair + brem sums) and 2 when it leaves the FP32
//                 range envelope;
//   kNesAccurate  flag 1: every product in df (cancellation up to ~1e5);
//                 beyond that the point is flagged 2;
//   kNesFp64Flag  flag 2: FP64 items.
enum NesMode
{
    kNesFp64All = 0,
    kNesAccurate = 2,
    kNesFp64Flag
};

// Warps per CTA of the NES kernels: the plain path runs a point per warp; the
// mixed path's passes over the few points flagged by the fast pass run a
// point per CTA, its items over all the CTA's threads (one warp alone would
// leave the pass as long as a point's whole item loop).
template <int MODE>
__host__ __device__ constexpr int nes_warps()
{
    return MODE == kNesFp64All ? kWarps : 8;
}

template <int MODE, bool MULTI = false>
__global__ void __launch_bounds__(nes_warps<MODE>() * 32, MODE == kNesAccurate ? 2 : 1)
    grey_neps_kernel(const __grid_constant__ OpacityLaunch L0, const GroupArgs GA, int64_t p0,
                     int64_t np, double* __restrict__ scratch)
{
    const OpacityLaunch& L = MULTI ? GA.Ls[blockIdx.z] : L0;
    if (MULTI)
    {
        const GroupChunk& gcz = GA.gc[blockIdx.z];
        p0      = gcz.p0;
        np      = gcz.np;
        scratch = gcz.ws;
    }
    if (MULTI && !L.use_inel)
        return;
    constexpr bool MIX  = MODE == kNesAccurate;
    constexpr bool WIDE = MODE != kNesFp64All;  // a point per CTA
    constexpr int NW    = nes_warps<MODE>();
    constexpr int NT    = WIDE ? 1 : NW;        // point tables in flight per CTA
    __shared__ double s_x2[kMaxQ], s_w2[kMaxQ], s_wx[kMaxQ], s_wx3[kMaxQ];
    __shared__ NepsTab s_nt[NT];
    __shared__ NepsMixed s_nm[MIX ? NT : 1];
    __shared__ dfm::FdiTab s_ftab;
    __shared__ double s_red[WIDE ? NW : 1][32];
    for (int k = threadIdx.x; k < kMaxQ; k += blockDim.x)
    {
        s_x2[k]  = L.x2[k];
        s_w2[k]  = L.w2[k];
        s_wx[k]  = L.wx[k];
        s_wx3[k] = L.wx3[k];
    }
    if (MIX)
        for (int k = threadIdx.x; k < (int)(sizeof(dfm::FdiTab) / sizeof(float)); k += blockDim.x)
            ((float*)&s_ftab)[k] = ((const float*)&dfm::kFdiTab)[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wid  = threadIdx.x >> 5;
    NepsTab& N     = s_nt[WIDE ? 0 : wid];
    const int n2   = L.n2;
    const bool nbb = L.neglect_blocking != 0;
    // items of a point: thread t0, t0 + stride, ...
    const int t0     = WIDE ? (int)threadIdx.x : lane;
    const int stride = WIDE ? NW * 32 : 32;
    const int64_t q0    = WIDE ? (int64_t)blockIdx.x : (int64_t)blockIdx.x * NW + wid;
    const int64_t qstep = WIDE ? (int64_t)gridDim.x : (int64_t)gridDim.x * NW;

    for (int64_t q = q0; q < np; q += qstep)
    {
        const int64_t p = L.pidx ? L.pidx[p0 + q] : p0 + q;
        PointTab* P     = (PointTab*)(scratch + q * kTabWords);
        if (MODE == kNesAccurate && P->neps_fp64 != 1.)
            continue;
        if (MODE == kNesFp64Flag && P->neps_fp64 != 2.)
            continue;
        const double T = L.eos[1][p], mu_e = L.eos[7][p];
        if (WIDE)
            __syncthreads(); // the previous point's readers are done
        else
            __syncwarp();
        if (!WIDE || wid == 0)
        {
            warp_copy((double*)&N.d, (const double*)&P->d, 28 + 12 + 2, lane);
            if (lane == 0)
                N.same_cf = P->same_cf;
        }
        if (WIDE)
            __syncthreads();
        else
            __syncwarp();
        const bool same_cf = N.same_cf != 0.;
        NepsPoint NP;
        NP.T    = T;
        NP.pre  = k::NepsConst * (T * T);
        NP.eta0 = mu_e / T;
        NP.eta1 = -mu_e / T;
        NP.fd00 = N.fd0[0];
        NP.fd01 = N.fd0[1];
        NP.fe0  = N.fe[0];
        NP.fe1  = N.fe[1];
        const double tn = 4. * (k::TempMultiple * T);
        double acc[16];
#pragma unroll
        for (int kk = 0; kk < 16; ++kk)
            acc[kk] = 0.;
        if (!MIX)
        {
            neps_items_fp64(NP, N.d, same_cf, n2, tn, L.stim != 0, nbb, s_x2, s_w2, s_wx, s_wx3,
                            t0, stride, acc);
        }
        else
        {
            int flag = 0;
            {
                NepsMixed& Q = s_nm[WIDE ? 0 : wid];
                if ((!WIDE || wid == 0) && lane < 2)
                {
                    Q.eta[lane] = dfm::from_double(lane ? NP.eta1 : NP.eta0);
                    dfm::fdi_raw15(Q.eta[lane], Q.reta[lane], 1, &s_ftab);
                }
                else if ((!WIDE || wid == 0) && lane >= 8 && lane < 12)
                {
                    const int s    = lane - 8;
                    const Distr& d = N.d;
                    Q.invTt[s] = 1. / d.temp_t[s];
                    Q.etat[s]  = d.eta_t[s];
                    Q.lbf[s]   = d.beta_f[s] > 0. ? log(d.beta_f[s]) : -INFINITY;
                    Q.invTf[s] = 1. / d.temp_f[s];
                    Q.cf[s]    = d.c_f[s];
                }
                if (WIDE)
                    __syncthreads();
                else
                    __syncwarp();
                const double invT = 1. / T;
                const double lhtn = log(0.5 * tn);
                dfm::df dacc[16];
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    dacc[kk] = {0.f, 0.f};
                float mag[16];
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    mag[kk] = 0.f;
                const int nn2 = n2 * n2;
                for (int it = t0; it < 2 * nn2; it += stride)
                {
                    const int r   = it >= nn2;
                    const int rem = it - r * nn2;
                    const int i = rem / n2, j = rem - (rem / n2) * n2;
                    double nu, nub;
                    neps_energies(r, s_x2[i], s_x2[j], tn, &nu, &nub);
                    const double w = nu * invT, wp = nub * invT;
                    // log nu, log nubar from the node logarithms
                    const double lx = L.lx2[i], lm = L.l1m[j], lp = L.l1p[j];
                    const double lnu  = lhtn + (r ? lm - lx : lx + lm);
                    const double lnub = lhtn + (r ? lp - lx : lx + lp);
                    const double Wr   = (r ? s_wx3[i] : s_wx[i]) * s_w2[j];
                    {
                        using namespace dfm;
                        df em1[4], ab1[4], em2[4], ab2[4];
                        neps_item_df(NP, Q, &s_ftab, w, wp, em1, ab1, em2, ab2);
                        double wt[4], wfd[4];
#pragma unroll
                        for (int s = 0; s < 4; ++s)
                        {
                            wt[s]  = N.d.w_t[s];
                            wfd[s] = N.d.w_f[s];
                        }
                        df g[4], gm[4], gb[4], gbm[4];
                        total_nu_df(nu, lnu, Q, wt, wfd, g, gm);
                        total_nu_df(nub, lnub, Q, wt, wfd, gb, gbm);
                        const df W = from_double(w), WP = from_double(wp);
                        const df ww = mul(W, WP), w4 = mul(ww, ww), Wd = from_double(Wr);
#pragma unroll
                        for (int s = 0; s < 4; ++s)
                        {
                            const df e1 = mul(em1[s], gb[s]);
                            const df a1 = nbb ? ab1[s] : mul(ab1[s], gbm[s]);
                            const df e2 = mul(em2[s], g[s]);
                            const df a2 = nbb ? ab2[s] : mul(ab2[s], gm[s]);
                            df EM1, AB1, EM2, AB2;
                            if (L.stim)
                            {
                                AB1 = mul(mul(w4, g[s]), add(e1, a1));
                                EM1 = mul(w4, e1);
                                AB2 = mul(mul(w4, gb[s]), add(e2, a2));
                                EM2 = mul(w4, e2);
                            }
                            else
                            {
                                AB1 = mul(mul(w4, g[s]), a1);
                                EM1 = mul(mul(w4, gm[s]), e1);
                                AB2 = mul(mul(w4, gb[s]), a2);
                                EM2 = mul(mul(w4, gbm[s]), e2);
                            }
                            const df tem = mul(Wd, add(EM1, EM2)), tab = mul(Wd, add(AB1, AB2));
                            const df tee = mul(Wd, add(mul(W, EM1), mul(WP, EM2)));
                            const df tae = mul(Wd, add(mul(W, AB1), mul(WP, AB2)));
                            dacc[s]      = add(dacc[s], tem);
                            dacc[4 + s]  = add(dacc[4 + s], tab);
                            dacc[8 + s]  = add(dacc[8 + s], tee);
                            dacc[12 + s] = add(dacc[12 + s], tae);
                            mag[s] += fabsf(tem.hi);
                            mag[4 + s] += fabsf(tab.hi);
                            mag[8 + s] += fabsf(tee.hi);
                            mag[12 + s] += fabsf(tae.hi);
                        }
                    }
                }
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    acc[kk] = dfm::to_double(dacc[kk]);
                // terms of both signs (occupation above 1), or NES sums
                // cancelling the pair + brem sums of the same output (those enter
                // the assembly with t2d^2 = hn / 8, times t2d for energy moments)
                // or the beta rates: the fast pass hands the point to the
                // accurate pass, the accurate pass to FP64
                const double T4 = (T * T) * (T * T);
                double other[16];
                beta_in_sum_units(P, T, NP.eta0, L.use_abs_em, true, other);
                const double t2d = k::TempMultiple * T;
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    other[kk] += (L.use_pair || L.use_brem)
                                     ? 0.125 * P->s2d[kk] * (kk >= 8 ? t2d : 1.)
                                     : 0.;
                double macc[16];
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    macc[kk] = (double)mag[kk];
                if (WIDE)
                {
                    block_sum<NW>(acc, s_red, 0);
                    block_sum<NW>(macc, s_red, 16);
                }
                else
                {
#pragma unroll
                    for (int kk = 0; kk < 16; ++kk)
                    {
                        acc[kk]  = warp_sum(acc[kk]);
                        macc[kk] = warp_sum(macc[kk]);
                    }
                }
                const double amp =
                    cancel_factor_tot(acc, macc, NP.pre * T4, NP.pre * T4 * T, other);
                if (amp > kMaxCancelDf)
                    flag = 2;
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    acc[kk] *= NP.pre * T4 * (kk >= 8 ? T : 1.);
            }
            if (flag != 0)
            {
                if (WIDE ? threadIdx.x == 0 : lane == 0)
                {
                    P->neps_fp64 = (double)flag;
                    atomicAdd(&g_grey_mixed[2], 1ull);
                }
                continue; // a later launch writes this point's sums
            }
        }
        if (!MIX) // (the mixed pass has summed over the point's threads already)
        {
            if (WIDE)
                block_sum<NW>(acc, s_red, 0);
            else
            {
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    acc[kk] = warp_sum(acc[kk]);
            }
        }
        if (WIDE ? threadIdx.x == 0 : lane == 0)
        {
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                P->snes[kk] = acc[kk];
        }
    }
}

// ---------------------------------------------------------------------------
// NES/NPS fast pass of the mixed path (InelasticScattKernels and the grey
// item sums of m1_opacities.hpp:880-905): one warp per point, one item per
// lane, the kernel integrals of bnsn_nes32.cuh in FP32.
// ---------------------------------------------------------------------------

constexpr int kNesWarps = 8;
constexpr int kNesItems = 2 * kMaxQ * kMaxQ;

// One (w, w') item.  w = nu/T and w' = nubar/T depend only on the quadrature
// nodes, so one table per CTA serves every point; the table follows the
// host's item order (ascending max(w, w')), which keeps a warp's lanes on
// items of similar quadrature cost.
struct NesItem
{
    float wh, wl, wph, wpl;     // w, w' as df
    float lwh, lwl, lwph, lwpl; // log w, log w' as df
    float sefa, sefb;           // sign x NEPSExpFunc(w' - w), sign x NEPSExpFunc(w - w')
    float wf;                   // quadrature weight
    float pad;
};

// Per-warp data of the point in work.
struct NesWarp
{
    NepsTab N; // distribution and F_k(eta) for the FP64 Taylor branches
    nes32::Lepton lep[2];
    NuSpecies sp[4];
};

struct NesSmem
{
    NesItem items[kNesItems];
    NesWarp w[kNesWarps];
    uint16_t q[kNesWarps][kNesItems]; // items (| lepton mask << 14) for the Taylor branches
    float2 dacc[16][kNesWarps * 32];  // per-lane df sums of the 16 moments
    float4 mag[4][kNesWarps * 32];    // per-lane sums of |term|
};

// Adds one item's terms to the lane's sums: em1..ab2 are R(nu, nubar) and
// R(nubar, nu) with NEPSExpFunc applied, times (w w')^2 (m1_opacities.hpp:880-905).
__device__ __forceinline__ void nes_accumulate(NesSmem& S, int t, bool stim, bool nbb, float Wf,
                                               float fw, float fwp, const float* g,
                                               const float* gm, const float* gb,
                                               const float* gbm, const float* em1,
                                               const float* ab1, const float* em2,
                                               const float* ab2)
{
    float tm[16];
#pragma unroll
    for (int s = 0; s < 4; ++s)
    {
        const float e1 = em1[s] * gb[s];
        const float a1 = ab1[s] * (nbb ? 1.f : gbm[s]);
        const float e2 = em2[s] * g[s];
        const float a2 = ab2[s] * (nbb ? 1.f : gm[s]);
        float EM1, AB1, EM2, AB2;
        if (stim)
        {
            AB1 = g[s] * (e1 + a1);
            EM1 = e1;
            AB2 = gb[s] * (e2 + a2);
            EM2 = e2;
        }
        else
        {
            AB1 = g[s] * a1;
            EM1 = gm[s] * e1;
            AB2 = gb[s] * a2;
            EM2 = gbm[s] * e2;
        }
        tm[s]      = Wf * (EM1 + EM2);
        tm[4 + s]  = Wf * (AB1 + AB2);
        tm[8 + s]  = Wf * (fw * EM1 + fwp * EM2);
        tm[12 + s] = Wf * (fw * AB1 + fwp * AB2);
    }
#pragma unroll
    for (int kk = 0; kk < 16; ++kk)
    {
        const float2 a   = S.dacc[kk][t];
        const dfm::df r  = dfm::add(dfm::df{a.x, a.y}, tm[kk]);
        S.dacc[kk][t]    = make_float2(r.hi, r.lo);
    }
#pragma unroll
    for (int k4 = 0; k4 < 4; ++k4)
    {
        float4 m = S.mag[k4][t];
        m.x += fabsf(tm[4 * k4]);
        m.y += fabsf(tm[4 * k4 + 1]);
        m.z += fabsf(tm[4 * k4 + 2]);
        m.w += fabsf(tm[4 * k4 + 3]);
        S.mag[k4][t] = m;
    }
}

template <bool MULTI = false>
__global__ void __launch_bounds__(kNesWarps * 32, 2)
    grey_nes_fast_kernel(const __grid_constant__ OpacityLaunch L0, const GroupArgs GA,
                         int64_t p0, int64_t np, double* __restrict__ scratch)
{
    const OpacityLaunch& L = MULTI ? GA.Ls[blockIdx.z] : L0;
    if (MULTI)
    {
        const GroupChunk& gcz = GA.gc[blockIdx.z];
        p0      = gcz.p0;
        np      = gcz.np;
        scratch = gcz.ws;
    }
    if (MULTI && !L.use_inel)
        return;
    extern __shared__ __align__(16) unsigned char nes_smem_raw[];
    NesSmem& S   = *reinterpret_cast<NesSmem*>(nes_smem_raw);
    const int n2 = L.n2, nn2 = n2 * n2, nit = 2 * nn2;
    {
        // w = c x_i (1 -+ x_j) for r = 0 and c (1 -+ x_j) / x_i for r = 1, c = 2 x 2.182
        constexpr double c = 2. * k::TempMultiple;
        const double lc    = log(c);
        for (int k = threadIdx.x; k < nit; k += blockDim.x)
        {
            const int it    = L.nes_order[k];
            const int r     = it >= nn2;
            const int rem   = it - r * nn2;
            const int i     = rem / n2, j = rem - (rem / n2) * n2;
            const double xi = L.x2[i], xj = L.x2[j];
            const double w  = r ? c * (1. - xj) / xi : c * xi * (1. - xj);
            const double wp = r ? c * (1. + xj) / xi : c * xi * (1. + xj);
            const double lw  = lc + (r ? L.l1m[j] - L.lx2[i] : L.lx2[i] + L.l1m[j]);
            const double lwp = lc + (r ? L.l1p[j] - L.lx2[i] : L.lx2[i] + L.l1p[j]);
            const double d1 = wp - w, d2 = w - wp;
            const bool n1 = signbit(d1) != 0, n2b = signbit(d2) != 0;
            const float sg = n1 ? 1.f : -1.f; // the reference's sign of R(w, w')
            NesItem I;
            dfm::df t = dfm::from_double(w);
            I.wh = t.hi, I.wl = t.lo;
            t = dfm::from_double(wp);
            I.wph = t.hi, I.wpl = t.lo;
            t = dfm::from_double(lw);
            I.lwh = t.hi, I.lwl = t.lo;
            t = dfm::from_double(lwp);
            I.lwph = t.hi, I.lwpl = t.lo;
            I.sefa = sg * neps_exp_f32(d1, n1);
            I.sefb = sg * neps_exp_f32(d2, n2b);
            I.wf   = (float)((r ? L.wx3[i] : L.wx[i]) * L.w2[j]);
            I.pad  = 0.f;
            S.items[k] = I;
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wid  = threadIdx.x >> 5;
    const int t    = threadIdx.x;
    NesWarp& Wd    = S.w[wid];
    uint16_t* qw   = S.q[wid];
    const bool nbb  = L.neglect_blocking != 0;
    const bool stim = L.stim != 0;
    const int64_t nwarp = (int64_t)gridDim.x * kNesWarps;
    constexpr float kBp = (float)k::NepsBPlus, kBm = (float)k::NepsBMinus,
                    kBz = (float)k::NepsBZero;

    for (int64_t qp = (int64_t)blockIdx.x * kNesWarps + wid; qp < np; qp += nwarp)
    {
        const int64_t p = L.pidx ? L.pidx[p0 + qp] : p0 + qp;
        PointTab* P     = (PointTab*)(scratch + qp * kTabWords);
        const double T = L.eos[1][p], mu_e = L.eos[7][p];
        __syncwarp();
        warp_copy((double*)&Wd.N.d, (const double*)&P->d, 28 + 12 + 2, lane);
        if (lane == 0)
            Wd.N.same_cf = P->same_cf;
        __syncwarp();
        NepsPoint NP;
        NP.T    = T;
        NP.pre  = k::NepsConst * (T * T);
        NP.eta0 = mu_e / T;
        NP.eta1 = -mu_e / T;
        NP.fd00 = Wd.N.fd0[0];
        NP.fd01 = Wd.N.fd0[1];
        NP.fe0  = Wd.N.fe[0];
        NP.fe1  = Wd.N.fe[1];
        // range envelope: the occupation of every species far above the FP32
        // normal range at its peak; e^{-Lref} of the e+ integrals finite
        bool ok = isfinite(NP.eta0) && NP.eta0 > -80.;
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            const Distr& d = Wd.N.d;
            ok = ok && (d.w_t[s] == 0. || d.eta_t[s] > -60.) &&
                 (d.w_f[s] == 0. || d.beta_f[s] > 1e-30) && (d.temp_t[s] > 0.) &&
                 (d.temp_f[s] > 0.) && isfinite(d.eta_t[s]) && isfinite(d.beta_f[s]);
        }
        int flag = ok ? 0 : 2;
        double acc[16];
        if (flag == 0)
        {
            if (lane < 2)
                Wd.lep[lane] = nes32::make_lepton(lane ? NP.eta1 : NP.eta0);
            else if (lane >= 8 && lane < 12)
            {
                // x = w = omega / T
                nu_species(Wd.N.d, lane - 8, T, -log(T), &Wd.sp[lane - 8]);
            }
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                S.dacc[kk][t] = make_float2(0.f, 0.f);
#pragma unroll
            for (int k4 = 0; k4 < 4; ++k4)
                S.mag[k4][t] = make_float4(0.f, 0.f, 0.f, 0.f);
            __syncwarp();
            // e+ terms scale as e^{-eta_e}: below 1e-13 of the e- terms for eta_e > 30
            const int nlep = NP.eta0 > 30. ? 1 : 2;
            int nq = 0;
            for (int base = 0; base < nit; base += 32)
            {
                const int k  = base + lane;
                unsigned tmk = 0;
                if (k < nit)
                {
                    const NesItem I    = S.items[k];
                    const dfm::df W    = {I.wh, I.wl}, WP = {I.wph, I.wpl};
                    const nes32::Geo G = nes32::make_geo(W, WP);
                    // A e^{-Lref}-scaled kernel sum b1 I_1 + b2 I_2 per species
                    // over the leptons: R(nu, nubar) (w w')^2 = sign x c
                    float c[4] = {0.f, 0.f, 0.f, 0.f};
                    bool any   = false;
#pragma unroll 1
                    for (int e = 0; e < nlep; ++e)
                    {
                        const nes32::Lepton& Lp = Wd.lep[e];
                        if (!nes32::above_taylor(G, Lp))
                        {
                            tmk |= 1u << e;
                            continue;
                        }
                        float I1, I2;
                        nes32::lepton_integrals(G, Lp, I1, I2);
                        const float A = Lp.A * I1, B = Lp.A * I2;
#pragma unroll
                        for (int s = 0; s < 4; ++s)
                        {
                            const float bo   = (s < 2) ? kBp : kBm;
                            const bool first = ((s & 1) == 0) != (e == 1); // b1 = bo, b2 = B0
                            c[s] += first ? fmaf(A, bo, B * kBz) : fmaf(A, kBz, B * bo);
                        }
                        any = true;
                    }
                    if (any)
                    {
                        // R(nubar, nu) = -R(nu, nubar)
                        float em1[4], ab1[4], em2[4], ab2[4];
#pragma unroll
                        for (int s = 0; s < 4; ++s)
                        {
                            em1[s] = ab2[s] = -c[s] * I.sefb;
                            ab1[s] = em2[s] = c[s] * I.sefa;
                        }
                        float g[4], gm[4], gb[4], gbm[4];
                        total_nu_q(W, dfm::df{I.lwh, I.lwl}, Wd.sp, g, gm);
                        total_nu_q(WP, dfm::df{I.lwph, I.lwpl}, Wd.sp, gb, gbm);
                        nes_accumulate(S, t, stim, nbb, I.wf, I.wh, I.wph, g, gm, gb, gbm, em1,
                                       ab1, em2, ab2);
                    }
                }
                const unsigned tb = __ballot_sync(0xffffffffu, tmk != 0);
                if (tmk)
                    qw[nq + __popc(tb & ((1u << lane) - 1u))] = (uint16_t)(k | (tmk << 14));
                nq += __popc(tb);
            }
            __syncwarp();
            // items in the reference's Taylor branches (w or w' below 1e-3 eta,
            // kernel_nes.hpp:82-132), FP64, all lanes busy
            for (int base = 0; base < nq; base += 32)
            {
                const int qi = base + lane;
                if (qi >= nq)
                    continue;
                const unsigned ent = qw[qi];
                const int k        = (int)(ent & 0x3fffu);
                const unsigned tmq = ent >> 14;
                const NesItem I    = S.items[k];
                const double w  = (double)I.wh + (double)I.wl;
                const double wp = (double)I.wph + (double)I.wpl;
                const double x = w > wp ? w : wp, y = w > wp ? wp : w;
                const bool n1 = signbit(wp - w) != 0, n2b = signbit(w - wp) != 0;
                const int sign1 = n1 ? 1 : -1, sign2 = n2b ? 1 : -1;
                const float efa = (float)sign1 * I.sefa, efb = (float)sign1 * I.sefb;
                const float w4  = (float)((w * wp) * (w * wp));
                float em1[4], ab1[4], em2[4], ab2[4];
#pragma unroll
                for (int s = 0; s < 4; ++s)
                    em1[s] = ab1[s] = em2[s] = ab2[s] = 0.f;
#pragma unroll 1
                for (int e = 0; e < 2; ++e)
                {
                    if (!((tmq >> e) & 1u))
                        continue;
                    double t1[4], t2[4];
                    neps_taylor(NP, e, w, wp, x, y, sign1, sign2, t1, t2);
#pragma unroll
                    for (int s = 0; s < 4; ++s)
                    {
                        const float r1 = (float)t1[s] * w4, r2 = (float)t2[s] * w4;
                        em1[s] += -r1 * efb;
                        ab1[s] += r1 * efa;
                        em2[s] += -r2 * efa;
                        ab2[s] += r2 * efb;
                    }
                }
                float g[4], gm[4], gb[4], gbm[4];
                total_nu_q(dfm::df{I.wh, I.wl}, dfm::df{I.lwh, I.lwl}, Wd.sp, g, gm);
                total_nu_q(dfm::df{I.wph, I.wpl}, dfm::df{I.lwph, I.lwpl}, Wd.sp, gb, gbm);
                nes_accumulate(S, t, stim, nbb, I.wf, I.wh, I.wph, g, gm, gb, gbm, em1, ab1, em2,
                               ab2);
            }
            float mag[16];
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
            {
                const float2 a = S.dacc[kk][t];
                acc[kk]        = (double)a.x + (double)a.y;
            }
#pragma unroll
            for (int k4 = 0; k4 < 4; ++k4)
            {
                const float4 m = S.mag[k4][t];
                mag[4 * k4]     = m.x;
                mag[4 * k4 + 1] = m.y;
                mag[4 * k4 + 2] = m.z;
                mag[4 * k4 + 3] = m.w;
            }
            // terms of both signs (occupation above 1), or NES sums cancelling
            // the pair + brem sums of the same output (those enter the assembly
            // with t2d^2 = hn / 8, times t2d for energy moments) or the beta
            // rates: the point goes to the accurate pass
            const double T4 = (T * T) * (T * T);
            double other[16];
            beta_in_sum_units(P, T, NP.eta0, L.use_abs_em, true, other);
            const double t2d = k::TempMultiple * T;
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                other[kk] += (L.use_pair || L.use_brem)
                                 ? 0.125 * P->s2d[kk] * (kk >= 8 ? t2d : 1.)
                                 : 0.;
            const double amp = cancel_factor(acc, mag, NP.pre * T4, NP.pre * T4 * T, other);
            if (amp > kMaxCancel)
                flag = 1;
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                acc[kk] *= NP.pre * T4 * (kk >= 8 ? T : 1.);
        }
        if (lane == 0)
        {
            P->neps_fp64 = (double)flag;
            if (flag != 0)
                atomicAdd(&g_grey_mixed[flag], 1ull);
        }
        if (flag != 0)
            continue; // a later launch writes this point's sums
#pragma unroll
        for (int kk = 0; kk < 16; ++kk)
            acc[kk] = warp_sum(acc[kk]);
        if (lane == 0)
        {
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                P->snes[kk] = acc[kk];
        }
    }
}

// ---------------------------------------------------------------------------
// assembly (m1_opacities.hpp:1172-1294), one thread per point
// ---------------------------------------------------------------------------

// Points whose outputs hold a NaN or Inf (the reference propagates them from
// bad inputs, e.g. GP19 outside its table); read by grey_nonfinite_count.
__device__ unsigned long long g_grey_nonfinite;

template <bool MULTI = false>
__global__ void __launch_bounds__(128)
    grey_final_kernel(const __grid_constant__ OpacityLaunch L0, const GroupArgs GA, int64_t p0,
                      int64_t np, double* __restrict__ scratch, int redo_only)
{
    const OpacityLaunch& L = MULTI ? GA.Ls[blockIdx.z] : L0;
    if (MULTI)
    {
        const GroupChunk& gcz = GA.gc[blockIdx.z];
        p0      = gcz.p0;
        np      = gcz.np;
        scratch = gcz.ws;
    }
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < np;
         q += (int64_t)gridDim.x * blockDim.x)
    {
        bool nonfinite      = false;
        const int64_t p     = L.pidx ? L.pidx[p0 + q] : p0 + q;
        PointTab* P         = (PointTab*)(scratch + q * kTabWords);
        const bool pcheck   = L.mixed && L.use_pair;
        if (redo_only && P->bredo != 1. && !(pcheck && pair_mixed(P)->predo == 1.))
            continue;
        // mixed path: FP32 brem terms whose sum the other reactions cancel
        // (the NES sums of the opposite sign where the occupation exceeds 1)
        // by more than kMaxCancelBrem are recomputed in FP64 (bredo = 1); the
        // same for the FP32 pair integrals beyond kMaxCancelPair (predo = 1)
        const bool check = !redo_only && L.mixed && L.use_brem;
        const bool check_pair = !redo_only && pcheck;
        bool bredo       = false;
        bool predo       = false;
        const double T      = L.eos[1][p];
        const double eta_e  = L.eos[7][p] / T;
        const double t2d    = k::TempMultiple * T;
        const double t2     = t2d * t2d;
        const double tn     = 4. * (k::TempMultiple * T);
        const double hn     = 0.5 * (tn * tn);
        const bool has2d    = L.use_pair || L.use_brem;
        double sb[2];
        double fe[2][6];
#pragma unroll
        for (int e = 0; e < 2; ++e)
#pragma unroll
            for (int kk = 0; kk < 6; ++kk)
                fe[e][kk] = P->fe[e][kk];
        beta_scales(T, eta_e, fe, sb);
        const double F = k::FourPiHc3, F2 = k::FourPiHc3Sqr, c = k::Clight;
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            const double n = L.m1[s][p], J = L.m1[4 + s][p];
            const double s_iso = (n > k::ThresholdN) ? (J / n) : 1.5 * T;
            const double n2d_em = has2d ? P->s2d[s] * t2 : 0.;
            const double n2d_ab = has2d ? P->s2d[4 + s] * t2 : 0.;
            const double e2d_em = has2d ? P->s2d[8 + s] * t2d * t2 : 0.;
            const double e2d_ab = has2d ? P->s2d[12 + s] * t2d * t2 : 0.;
            const double nne_em = L.use_inel ? P->snes[s] * hn : 0.;
            const double nne_ab = L.use_inel ? P->snes[4 + s] * hn : 0.;
            const double ene_em = L.use_inel ? P->snes[8 + s] * hn : 0.;
            const double ene_ab = L.use_inel ? P->snes[12 + s] * hn : 0.;
            const double iso    = L.use_iso ? P->siso[s] * s_iso : 0.;
            double o[5];
            double bne = 0., bje = 0., bna = 0., bja = 0.;
            if (s < 2)
            {
                if (L.use_abs_em)
                {
                    bne = P->sbeta[s] * sb[s];
                    bje = P->sbeta[2 + s] * sb[s];
                    bna = P->sbeta[4 + s] * sb[s];
                    bja = P->sbeta[6 + s] * sb[s];
                }
                o[0] = F * (F * (n2d_em + nne_em) + bne);
                o[2] = F * (F * (e2d_em + ene_em) + bje);
                o[1] = (n > k::ThresholdN) ? F / (c * n) * (F * (n2d_ab + nne_ab) + bna) : 0.;
                o[3] = (J > k::ThresholdJ) ?
                           ((s == 0 && n == 0.) ? 0. : F / (c * J) * (F * (e2d_ab + ene_ab) + bja)) :
                           0.;
            }
            else
            {
                o[0] = F2 * (n2d_em + nne_em);
                o[2] = F2 * (e2d_em + ene_em);
                o[1] = (n > k::ThresholdN) ?
                           ((s == 3 && n == 0.) ? 0. : F2 / (c * n) * (n2d_ab + nne_ab)) :
                           0.;
                o[3] = (J > k::ThresholdJ) ? F2 / (c * J) * (e2d_ab + ene_ab) : 0.;
            }
            o[4] = (J > k::ThresholdJ) ? F / (c * J) * iso : 0.;
            if (check || check_pair)
            {
                // totals of the four moments before the output factors, and the
                // brem (pair) terms' magnitude in the same units
                const double tot[4] = {F * (n2d_em + nne_em) + bne, F * (n2d_ab + nne_ab) + bna,
                                       F * (e2d_em + ene_em) + bje, F * (e2d_ab + ene_ab) + bja};
#pragma unroll
                for (int m = 0; m < 4; ++m)
                {
                    const double u = F * (m < 2 ? t2 : t2d * t2);
                    if (check)
                        bredo = bredo || u * P->bmag[4 * m + s] > kMaxCancelBrem * fabs(tot[m]);
                    if (check_pair)
                        predo = predo ||
                                u * pair_mixed(P)->pmag[4 * m + s] > kMaxCancelPair * fabs(tot[m]);
                }
            }
#pragma unroll
            for (int qq = 0; qq < 5; ++qq)
            {
                L.out[qq * 4 + s][p] = o[qq];
                nonfinite = nonfinite || !isfinite(o[qq]);
            }
        }
        if (!redo_only)
            P->bredo = bredo ? 1. : 0.; // also where brem is off: scratch is reused
        if (check_pair)
            pair_mixed(P)->predo = predo ? 1. : 0.;
        if (!redo_only && L.mixed)
        {
            atomicAdd(&g_grey_mixed[0], 1ull);
            if (predo)
                atomicAdd(&g_grey_mixed[3], 1ull);
            if (bredo)
                atomicAdd(&g_grey_mixed[4], 1ull);
        }
        if (nonfinite && !redo_only)
            atomicAdd(&g_grey_nonfinite, 1ull);
    }
}

// Persistent grid: resident CTAs (occupancy) x num_sms x the launch's
// grid_scale (a tuning knob; 2 by default), capped by the work.
thread_local double g_grid_scale = 1.;

template <class K>
int grid_for(K kernel, int threads, int64_t work, int num_sms)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) !=
            cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    int64_t cap = (int64_t)((double)num_sms * per_sm * g_grid_scale);
    cap = cap < 1 ? 1 : cap;
    return (int)(work < cap ? (work > 0 ? work : 1) : cap);
}

// One step of the phase pipeline.  Single launch (MULTI false): L is the
// launch, points p0 .. p0 + np of it with scratch ws.  Multi-group launch: G
// groups in grid z, their descriptors and chunk shares in GA (device memory);
// L is a host copy whose flags are the union of the groups' (which phases
// run), brem_set the brem variants present (bit i: variant i), np the largest
// share (grid x), p0 and ws unused.
struct Step
{
    OpacityLaunch const* L;
    GroupArgs GA;
    unsigned G;
    unsigned brem_set;
    int64_t p0, np;
    double* ws;
};

// The fast NES pass: 8-warp CTAs with the item table and the per-lane sums in
// dynamic shared memory (two CTAs per SM).
template <bool MULTI>
cudaError_t launch_nes_fast(const Step& S, cudaStream_t st, int sms)
{
    const int smem    = (int)sizeof(NesSmem);
    cudaError_t e     = cudaFuncSetAttribute(grey_nes_fast_kernel<MULTI>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grey_nes_fast_kernel<MULTI>,
                                                      kNesWarps * 32, smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    const int64_t work = (S.np + kNesWarps - 1) / kNesWarps;
    int64_t cap        = (int64_t)((double)sms * per_sm * g_grid_scale);
    cap                = cap < 1 ? 1 : cap;
    const int grid     = (int)(work < cap ? (work > 0 ? work : 1) : cap);
    grey_nes_fast_kernel<MULTI><<<dim3(grid, 1, MULTI ? S.G : 1), kNesWarps * 32, smem, st>>>(
        *S.L, S.GA, S.p0, S.np, S.ws);
    return cudaGetLastError();
}

template <bool MIXED, int IMPL, bool WIDE, bool MULTI>
void launch_brem_impl(const Step& S, cudaStream_t st, int sms, int add, int redo_only)
{
    constexpr int threads = (WIDE ? 8 : kWarps) * 32;
    const int64_t work    = WIDE ? S.np : (S.np + kWarps - 1) / kWarps;
    const int gx          = grid_for(grey_brem_kernel<MIXED, IMPL, WIDE, MULTI>, threads, work, sms);
    phase_mark(kPhBrem, 0, st);
    grey_brem_kernel<MIXED, IMPL, WIDE, MULTI><<<dim3(gx, 1, MULTI ? S.G : 1), threads, 0, st>>>(
        *S.L, S.GA, S.p0, S.np, S.ws, add, redo_only);
    phase_mark(kPhBrem, 1, st);
}

template <bool MIXED, bool WIDE, bool MULTI>
void launch_brem_set(const Step& S, cudaStream_t st, int sms, int add, int redo_only)
{
    // single launch: the launch's variant; multi-group: one launch per variant
    // present (each returns at once for the other variants' groups)
    const unsigned set = MULTI ? S.brem_set : 1u << S.L->brem_impl;
    if (set & 1u)
        launch_brem_impl<MIXED, 0, WIDE, MULTI>(S, st, sms, add, redo_only);
    if (set & 2u)
        launch_brem_impl<MIXED, 1, WIDE, MULTI>(S, st, sms, add, redo_only);
    if (set & 4u)
        launch_brem_impl<MIXED, 2, WIDE, MULTI>(S, st, sms, add, redo_only);
}

// redo_only (the FP64 pass over the points the final kernel marked) runs a
// point per CTA.
template <bool MIXED, bool MULTI>
cudaError_t launch_brem(const Step& S, cudaStream_t st, int sms, int add, int redo_only = 0)
{
    if constexpr (!MIXED)
    {
        if (redo_only)
            launch_brem_set<false, true, MULTI>(S, st, sms, add, redo_only);
        else
            launch_brem_set<false, false, MULTI>(S, st, sms, add, redo_only);
    }
    else
        launch_brem_set<true, false, MULTI>(S, st, sms, add, redo_only);
    return cudaGetLastError();
}

// The phase kernels of one step on stream st: point constants, prelude, pair,
// brem, NES, final, and on the mixed path the FP64 passes over the points the
// final kernel marked, with a second final pass.
template <bool MULTI>
cudaError_t launch_step(const Step& S, cudaStream_t st, int sms)
{
    const OpacityLaunch& L = *S.L;
    const int64_t np       = S.np;
    const int64_t wb       = (np + kWarps - 1) / kWarps;
    const unsigned gz      = MULTI ? S.G : 1;
    cudaError_t err        = cudaSuccess;
    phase_mark(kPhPrelude, 0, st);
    {
        const int64_t bx = (np + 127) / 128;
        const dim3 pgrid((unsigned)(bx < (int64_t)sms * 4 ? bx : (int64_t)sms * 4), kPointTasks,
                         gz);
        grey_point_kernel<MULTI><<<pgrid, 128, 0, st>>>(L, S.GA, S.p0, np, S.ws);
    }
    phase_mark(kPhPrelude, 1, st);
    phase_mark(kPhPrelude, 0, st);
    grey_prelude_kernel<MULTI>
        <<<dim3(grid_for(grey_prelude_kernel<MULTI>, kWarps * 32, wb, sms), 1, gz), kWarps * 32,
           0, st>>>(L, S.GA, S.p0, np, S.ws);
    phase_mark(kPhPrelude, 1, st);
    if (L.use_pair)
    {
        phase_mark(kPhPair, 0, st);
        if (L.mixed)
            grey_pair_kernel<true, false, MULTI>
                <<<dim3(grid_for(grey_pair_kernel<true, false, MULTI>, kWarps * 32, wb, sms), 1,
                        gz),
                   kWarps * 32, 0, st>>>(L, S.GA, S.p0, np, S.ws, 0);
        else
            grey_pair_kernel<false, false, MULTI>
                <<<dim3(grid_for(grey_pair_kernel<false, false, MULTI>, kWarps * 32, wb, sms), 1,
                        gz),
                   kWarps * 32, 0, st>>>(L, S.GA, S.p0, np, S.ws, 0);
        phase_mark(kPhPair, 1, st);
    }
    if (L.use_brem)
    {
        err = L.mixed ? launch_brem<true, MULTI>(S, st, sms, L.use_pair) :
                        launch_brem<false, MULTI>(S, st, sms, L.use_pair);
        if (err != cudaSuccess)
            return err;
    }
    if (L.use_inel)
    {
        if (L.mixed)
        {
            phase_mark(kPhNeps, 0, st);
            if ((err = launch_nes_fast<MULTI>(S, st, sms)) != cudaSuccess)
                return err;
            phase_mark(kPhNeps, 1, st);
            phase_mark(kPhNepsAccurate, 0, st);
            constexpr int wa = nes_warps<kNesAccurate>() * 32;
            grey_neps_kernel<kNesAccurate, MULTI>
                <<<dim3(grid_for(grey_neps_kernel<kNesAccurate, MULTI>, wa, np, sms), 1, gz), wa,
                   0, st>>>(L, S.GA, S.p0, np, S.ws);
            phase_mark(kPhNepsAccurate, 1, st);
            phase_mark(kPhNepsFp64, 0, st);
            constexpr int wf = nes_warps<kNesFp64Flag>() * 32;
            grey_neps_kernel<kNesFp64Flag, MULTI>
                <<<dim3(grid_for(grey_neps_kernel<kNesFp64Flag, MULTI>, wf, np, sms), 1, gz), wf,
                   0, st>>>(L, S.GA, S.p0, np, S.ws);
            phase_mark(kPhNepsFp64, 1, st);
        }
        else
        {
            phase_mark(kPhNeps, 0, st);
            grey_neps_kernel<kNesFp64All, MULTI>
                <<<dim3(grid_for(grey_neps_kernel<kNesFp64All, MULTI>, kWarps * 32, wb, sms), 1,
                        gz),
                   kWarps * 32, 0, st>>>(L, S.GA, S.p0, np, S.ws);
            phase_mark(kPhNeps, 1, st);
        }
    }
    const dim3 fgrid(grid_for(grey_final_kernel<MULTI>, 128, (np + 127) / 128, sms), 1, gz);
    phase_mark(kPhFinal, 0, st);
    grey_final_kernel<MULTI><<<fgrid, 128, 0, st>>>(L, S.GA, S.p0, np, S.ws, 0);
    phase_mark(kPhFinal, 1, st);
    if (L.mixed && (L.use_brem || L.use_pair))
    {
        // points whose FP32 brem or pair sums the other reactions cancel:
        // those parts in FP64, outputs again
        if (L.use_pair)
        {
            phase_mark(kPhPair, 0, st);
            grey_pair_kernel<false, true, MULTI>
                <<<dim3(grid_for(grey_pair_kernel<false, true, MULTI>, 8 * 32, np, sms), 1, gz),
                   8 * 32, 0, st>>>(L, S.GA, S.p0, np, S.ws, 1);
            phase_mark(kPhPair, 1, st);
        }
        if (L.use_brem && (err = launch_brem<false, MULTI>(S, st, sms, L.use_pair, 1)) !=
                              cudaSuccess)
            return err;
        phase_mark(kPhFinal, 0, st);
        grey_final_kernel<MULTI><<<fgrid, 128, 0, st>>>(L, S.GA, S.p0, np, S.ws, 1);
        phase_mark(kPhFinal, 1, st);
    }
    return cudaGetLastError();
}

} // namespace

namespace {

// The mixed path's pair integrals at given (y, z, eta): J_l = e^{ls} j_l with
// J_0 = Psi_0(y, z) / (1 - e^{y+z}), J_1 = Psi_0(z, y) / (1 - e^{y+z})
// (kernel_pair.hpp:16-120), ls = Lref - (y + z).  Zero where the reference
// zeroes Psi (eta - y - z > 200).
__global__ void __launch_bounds__(128)
    pair_j_kernel(const double* __restrict__ y, const double* __restrict__ z,
                  const double* __restrict__ eta, double* __restrict__ j0,
                  double* __restrict__ j1, double* __restrict__ ls, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        pair32::Cell c;
        double lref;
        if (!pair32::make_cell(y[i], z[i], eta[i], c, lref))
        {
            j0[i] = j1[i] = 0.;
            ls[i] = 0.;
            continue;
        }
        double Q0, Q1;
        pair32::cell_integrals(c, Q0, Q1);
        const double yz = y[i] * z[i];
        j0[i] = Q0 / (15. * (yz * yz));
        j1[i] = Q1 / (15. * (yz * yz));
        ls[i] = lref - (y[i] + z[i]);
    }
}

// The mixed path's NES/NPS out-kernel integrals at given (w, w', eta):
// MezzacappaIntOut(w, w', b1, b2) of kernel_nes.hpp:50-78 (the general
// branch, without the Taylor expansions) = e^{ls} (b1 m1 + b2 m2).
__global__ void __launch_bounds__(128)
    nes_m_kernel(const double* __restrict__ w, const double* __restrict__ wp,
                 const double* __restrict__ eta, double* __restrict__ m1,
                 double* __restrict__ m2, double* __restrict__ ls, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        float I1, I2;
        double lref;
        nes32::lepton_integrals(w[i], wp[i], eta[i], I1, I2, lref);
        const double xy  = w[i] * wp[i];
        const double sgn = w[i] > wp[i] ? 1. : -1.;
        m1[i] = sgn * (double)I1 / (xy * xy);
        m2[i] = sgn * (double)I2 / (xy * xy);
        ls[i] = lref;
    }
}

} // namespace

cudaError_t launch_nes_m(const double* w, const double* wp, const double* eta, double* m1,
                         double* m2, double* ls, int64_t n, cudaStream_t st, int sms)
{
    if (n <= 0)
        return cudaSuccess;
    const int64_t blocks = (n + 127) / 128;
    const int grid       = (int)(blocks < (int64_t)sms * 8 ? blocks : (int64_t)sms * 8);
    phase_mark(kPhAux, 0, st);
    nes_m_kernel<<<grid, 128, 0, st>>>(w, wp, eta, m1, m2, ls, n);
    phase_mark(kPhAux, 1, st);
    return cudaGetLastError();
}

cudaError_t launch_pair_j(const double* y, const double* z, const double* eta, double* j0,
                          double* j1, double* ls, int64_t n, cudaStream_t st, int sms)
{
    if (n <= 0)
        return cudaSuccess;
    const int64_t blocks = (n + 127) / 128;
    const int grid       = (int)(blocks < (int64_t)sms * 8 ? blocks : (int64_t)sms * 8);
    phase_mark(kPhAux, 0, st);
    pair_j_kernel<<<grid, 128, 0, st>>>(y, z, eta, j0, j1, ls, n);
    phase_mark(kPhAux, 1, st);
    return cudaGetLastError();
}

cudaError_t grey_mixed_counts(unsigned long long* counts, bool reset)
{
    cudaError_t e = cudaMemcpyFromSymbol(counts, g_grey_mixed, 5 * sizeof(*counts));
    if (e == cudaSuccess && reset)
    {
        const unsigned long long zero[5] = {0ull, 0ull, 0ull, 0ull, 0ull};
        e = cudaMemcpyToSymbol(g_grey_mixed, zero, sizeof(zero));
    }
    return e;
}

cudaError_t grey_nonfinite_count(unsigned long long* count, bool reset)
{
    cudaError_t e = cudaMemcpyFromSymbol(count, g_grey_nonfinite, sizeof(*count));
    if (e == cudaSuccess && reset)
    {
        const unsigned long long zero = 0ull;
        e = cudaMemcpyToSymbol(g_grey_nonfinite, &zero, sizeof(zero));
    }
    return e;
}

cudaError_t launch_grey_chunks(const OpacityLaunch& L, cudaStream_t st0, cudaStream_t aux, int sms,
                               double* ws0, double* ws1, int64_t chunk, int64_t* k)
{
    if (L.npts <= 0)
        return cudaSuccess;
    if (!ws0 || (aux && !ws1) || chunk < 1 || !k)
        return cudaErrorInvalidValue;
    // default grid: four waves of resident CTAs per phase kernel (per-point
    // work is uneven; later waves fill the tails of earlier ones, and the
    // other stream's kernel the tail of both).  Measured on the 256^3
    // all-reactions slab: 2, 3, 4 waves gave 411k, 417k, 423k points/s mixed
    // (FP64 172k, 174k, 177k); half a wave per stream, so that both streams'
    // kernels stay resident side by side, was 15% slower than 2 waves.
    g_grid_scale = L.grid_scale > 0. ? L.grid_scale : 4.;
    cudaError_t err = cudaSuccess;
    for (int64_t p0 = 0; p0 < L.npts && err == cudaSuccess; p0 += chunk, ++*k)
    {
        const bool odd        = aux != nullptr && (*k & 1);
        const cudaStream_t st = odd ? aux : st0;
        double* const wsk     = odd ? ws1 : ws0;
        const int64_t np      = (L.npts - p0) < chunk ? (L.npts - p0) : chunk;
        const Step S          = {&L, GroupArgs{nullptr, nullptr}, 0u, 0u, p0, np, wsk};
        err                   = launch_step<false>(S, st, sms);
    }
    return err;
}

cudaError_t launch_grey_multi(const OpacityLaunch& U, unsigned brem_set, const GroupArgs& GA,
                              unsigned groups, int64_t np_max, cudaStream_t st, int sms)
{
    if (groups == 0 || np_max <= 0)
        return cudaSuccess;
    if (!GA.Ls || !GA.gc || groups > 65535u)
        return cudaErrorInvalidValue;
    g_grid_scale = U.grid_scale > 0. ? U.grid_scale : 4.;
    const Step S = {&U, GA, groups, brem_set, 0, np_max, nullptr};
    return launch_step<true>(S, st, sms);
}

cudaError_t launch_grey(const OpacityLaunch& L, cudaStream_t st0, int sms, double* ws,
                        int64_t ws_points, cudaStream_t aux)
{
    if (L.npts <= 0)
        return cudaSuccess;
    if (!ws || ws_points < 1)
        return cudaErrorInvalidValue;
    // With an auxiliary stream, consecutive chunks alternate between the
    // caller's stream and aux, each with half of the scratch, so that the
    // FP64-pipe phases (prelude, pair) of one chunk run beside the FP32-pipe
    // NES phase of the other.  The caller's stream waits for aux at the end.
    const bool two      = aux != nullptr && ws_points >= 2 && L.npts > ws_points / 2;
    const int64_t chunk = two ? ws_points / 2 : ws_points;
    cudaEvent_t ev[2]   = {nullptr, nullptr};
    if (two)
    {
        cudaError_t e;
        if ((e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventRecord(ev[0], st0)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(aux, ev[0], 0)) != cudaSuccess)
            return e;
    }
    int64_t k       = 0;
    cudaError_t err = launch_grey_chunks(L, st0, two ? aux : nullptr, sms, ws,
                                         two ? ws + chunk * kTabWords : nullptr, chunk, &k);
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
