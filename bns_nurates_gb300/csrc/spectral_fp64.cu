// FP64 spectral opacity kernel (sm_103a).
//
// One warp computes all requested energies of one point.  Per point, the
// antineutrino grid of the pair/brem integral (t x_i, t / x_i with
// t = 2.182 T) is the same for every energy, so its distribution values and
// Fermi integrals F_k(eta +- nubar/T) are staged once in shared memory; per
// energy the Fermi integrals at eta +- nu/T (pair) and eta_e/eta_p - nu/T
// (NES/NPS) are staged too.  Lanes then take (energy, node group) tasks with
// groups of G consecutive lanes per energy (G a power of two) and combine the
// group sums with an xor-shuffle inside each segment.  Each integrand is
// evaluated once per node; the reference evaluates the full integrand once
// per (output, node) (integration.hpp:524-543), which only repeats identical
// values.
//
// Restates ComputeSpectralOpacities{NotStimulatedAbs,StimulatedAbs} and
// SpectralIntegrand (m1_opacities.hpp:1317-1660).

#include <cuda_runtime.h>

#include "bnsn_fp64.cuh"
#include "bnsn_internal.h"

namespace bnsn {
namespace {

using namespace fp64;

constexpr int kWarps  = 4;
constexpr int kEChunk = 32; // energies staged per pass

struct SpecScratch
{
    Distr d;
    double fe[2][6];
    double fd0[2];
    Hr98Point hr;
    double brt06_pre;
    double eta_pp, eta_nn;
    int same_cf;
    // antineutrino grid of the pair/brem integral
    double nb[kMaxM];
    double gb[kMaxM][4];
    double fmz[kMaxM][5], fpz[kMaxM][5];
    // per energy of the current chunk
    double ge[kEChunk][4];
    double fmy[kEChunk][5], fpy[kEChunk][5];
    double fw[kEChunk][2][6];
};

__device__ __forceinline__ double seg_sum(double v, int G)
{
    for (int o = 1; o < G; o <<= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kWarps * 32)
    spectral_fp64_kernel(const __grid_constant__ OpacityLaunch L, int G)
{
    __shared__ double s_x[kMaxQ], s_B1[kMaxM];
    __shared__ SpecScratch s_ws[kWarps];
    for (int k = threadIdx.x; k < kMaxQ; k += blockDim.x)
        s_x[k] = L.x1[k];
    for (int k = threadIdx.x; k < kMaxM; k += blockDim.x)
        s_B1[k] = L.B1[k];
    __syncthreads();

    const int lane      = threadIdx.x & 31;
    SpecScratch& W      = s_ws[threadIdx.x >> 5];
    const int64_t nwarp = (int64_t)gridDim.x * kWarps;
    const int n = L.n1, M = 2 * n, ne = L.n_energies;
    const bool nb_block = L.neglect_blocking != 0;

    for (int64_t p = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5); p < L.npts; p += nwarp)
    {
        const double nbar = L.eos[0][p], T = L.eos[1][p], ye = L.eos[2][p];
        const double yp = L.eos[3][p], yn = L.eos[4][p];
        const double mu_p = L.eos[5][p], mu_n = L.eos[6][p], mu_e = L.eos[7][p];
        const double dU = L.eos[9][p], dm_eff = L.eos[10][p];
        const double eta_e = mu_e / T;

        if (L.has_distr)
        {
            if (lane < 28)
                (&W.d.w_t[0])[lane] = L.distr[lane][p];
        }
        else if (lane < 4)
        {
            const int s = lane;
            distr_species(L.m1[s][p], L.m1[4 + s][p], L.m1[8 + s][p], L.gamma36, &W.d.w_t[s],
                          &W.d.temp_t[s], &W.d.eta_t[s], &W.d.w_f[s], &W.d.temp_f[s],
                          &W.d.c_f[s], &W.d.beta_f[s]);
        }
        if (lane == 4 || lane == 5)
        {
            const int e     = lane - 4;
            const double et = e ? -mu_e / T : eta_e;
            fdi_orders<0, 5>(et, W.fe[e]);
            W.fd0[e] = fermi_distr(0., 1., et);
        }
        if (L.use_brem && L.brem_impl == 0)
        {
            if (lane >= 6 && lane < 9)
                W.hr.ch[lane - 6] = hr98_channel(nbar, yn, yp, T, lane - 6);
            if (lane == 9)
                hr98_point_common(nbar, T, L.use_medium != 0, &W.hr);
        }
        if (lane == 10 && L.use_brem && L.brem_impl == 1)
            W.brt06_pre = brt06_point(nbar, T, yn, yp);
        if (lane == 11 && L.use_iso)
        {
            W.eta_pp = eta_nn_sc(nbar, T, yp);
            W.eta_nn = eta_nn_sc(nbar, T, yn);
        }
        __syncwarp();
        if (lane == 0)
        {
            const double c0 = W.d.c_f[0];
            W.same_cf = (W.d.c_f[1] == c0) && (W.d.c_f[2] == c0) && (W.d.c_f[3] == c0);
        }
        __syncwarp();
        const bool same_cf = W.same_cf != 0;
        const bool pb      = L.use_pair || L.use_brem;

        // antineutrino grid of the pair/brem integral (m1_opacities.hpp:1542)
        const double ts = k::TempMultiple * T;
        if (pb)
        {
            for (int a = lane; a < M; a += 32)
            {
                const int i     = a < n ? a : a - n;
                const double nu = a < n ? ts * s_x[i] : ts / s_x[i];
                W.nb[a]         = nu;
                total_nu_f4(nu, W.d, same_cf, W.gb[a]);
            }
            if (L.use_pair)
                for (int q = lane; q < 2 * M; q += 32)
                {
                    const int a     = q >> 1;
                    const int i     = a < n ? a : a - n;
                    const double z  = (a < n ? ts * s_x[i] : ts / s_x[i]) / T;
                    if (q & 1)
                        fdi_orders<1, 5>(eta_e + z, W.fpz[a]);
                    else
                        fdi_orders<1, 5>(eta_e - z, W.fmz[a]);
                }
        }
        NepsPoint NP;
        NP.T    = T;
        NP.pre  = k::NepsConst * (T * T);
        NP.eta0 = eta_e;
        NP.eta1 = -mu_e / T;
        NP.fd00 = W.fd0[0];
        NP.fd01 = W.fd0[1];
        NP.fe0  = W.fe[0];
        NP.fe1  = W.fe[1];
        BetaPoint bp;
        if (L.use_abs_em)
            bp = beta_point(nbar, T, yp, yn, mu_p, mu_n, mu_e, dU, dm_eff, L.use_dU,
                            L.use_dm_eff, L.use_WM_ab, L.use_decay);
        const Gp19Table G19 = {L.gp19.d0, L.gp19.d1, L.gp19.d2, L.gp19.d3, L.gp19.nb,
                               L.gp19.ye, L.gp19.t,  L.gp19.w,  L.gp19.lognb,
                               L.gp19.logw, L.gp19.data};

        for (int e0 = 0; e0 < ne; e0 += kEChunk)
        {
            const int nec = (ne - e0) < kEChunk ? (ne - e0) : kEChunk;
            __syncwarp();
            // per-energy staging
            for (int q = lane; q < nec; q += 32)
            {
                const double nu = L.energies[e0 + q];
                total_nu_f4(nu, W.d, same_cf, W.ge[q]);
                const double y = nu / T;
                if (L.use_pair)
                {
                    fdi_orders<1, 5>(eta_e - y, W.fmy[q]);
                    fdi_orders<1, 5>(eta_e + y, W.fpy[q]);
                }
                if (L.use_inel)
                {
                    fdi_orders<0, 5>(eta_e - y, W.fw[q][0]);
                    fdi_orders<0, 5>(NP.eta1 - y, W.fw[q][1]);
                }
            }
            __syncwarp();
            const int per_round = 32 / G;
            for (int r0 = 0; r0 < nec; r0 += per_round)
            {
                const int q    = r0 + lane / G;
                const int grp  = lane % G;
                const bool act = q < nec;
                double acc[16];
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    acc[kk] = 0.;
                const double nu = act ? L.energies[e0 + q] : 1.;
                if (act)
                {
                    for (int a = grp; a < M; a += G)
                    {
                        const int i     = a < n ? a : a - n;
                        const double wa = s_B1[a];
                        if (pb)
                        {
                            const double nub = W.nb[a];
                            const double* gb = W.gb[a];
                            double pe[4] = {0., 0., 0., 0.}, pa[4] = {0., 0., 0., 0.};
                            double be = 0., ba = 0.;
                            if (L.use_pair)
                                pair_kernel(T, eta_e, nu, nub, nu / T, nub / T, W.fmy[q],
                                            W.fpy[q], W.fmz[a], W.fpz[a], W.fe[0][3],
                                            W.fe[0][4], pe, pa);
                            if (L.use_brem)
                            {
                                if (L.brem_impl == 0)
                                    hr98_kernel(W.hr, nu, nub, &be, &ba);
                                else if (L.brem_impl == 1)
                                    brt06_kernel(W.brt06_pre, T, nu, nub, &be, &ba);
                                else
                                    gp19_kernel(G19, nbar, ye, T, nu, nub, &be, &ba);
                            }
                            const double nb2 = nub * nub;
#pragma unroll
                            for (int s = 0; s < 4; ++s)
                            {
                                const int ps   = s ^ 1;
                                const double bf = nb_block ? 1. : 1. - gb[ps];
                                const double pro = (pe[s] + be) * bf;
                                const double ann = (pa[s] + ba) * gb[ps];
                                acc[s] += wa * (nb2 * pro);
                                acc[4 + s] += wa * (nb2 * ann);
                            }
                        }
                        if (L.use_inel)
                        {
                            const double nub = a < n ? nu * s_x[i] : nu / s_x[i];
                            double gb[4], em[4], ab[4];
                            total_nu_f4(nub, W.d, same_cf, gb);
                            neps_one(NP, nu, nub, W.fw[q][0], W.fw[q][1], em, ab);
                            const double nb2 = nub * nub;
#pragma unroll
                            for (int s = 0; s < 4; ++s)
                            {
                                const double bf = nb_block ? 1. : 1. - gb[s];
                                acc[8 + s] += wa * (nb2 * (em[s] * gb[s]));
                                acc[12 + s] += wa * (nb2 * (ab[s] * bf));
                            }
                        }
                    }
                }
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    acc[kk] = seg_sum(acc[kk], G);
                if (act && grp == 0)
                {
                    // assemble (m1_opacities.hpp:1571-1660)
                    double b_ab[4] = {0., 0., 0., 0.}, b_em[4] = {0., 0., 0., 0.};
                    if (L.use_abs_em)
                    {
                        beta_rates(bp, nu, 0, &b_ab[0], &b_em[0]);
                        beta_rates(bp, nu, 1, &b_ab[1], &b_em[1]);
                    }
                    const double iso =
                        L.use_iso ? iso_scatt_leg0(nu, W.eta_pp, W.eta_nn, L.use_WM_sc != 0) : 0.;
                    const double F = k::FourPiHc3, c = k::Clight;
                    const int64_t o = p * L.e_stride + L.e_offset + e0 + q;
#pragma unroll
                    for (int s = 0; s < 4; ++s)
                    {
                        const double ip_e = pb ? ts * acc[s] : 0.;
                        const double ip_a = pb ? ts * acc[4 + s] : 0.;
                        const double in_e = L.use_inel ? nu * acc[8 + s] : 0.;
                        const double in_a = L.use_inel ? nu * acc[12 + s] : 0.;
                        const double g    = W.ge[q][s];
                        double j  = b_em[s] + F * (ip_e + in_e);
                        double ka = (b_ab[s] + F * (ip_a + in_a)) / c;
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
                    }
                }
            }
        }
        __syncwarp();
    }
}

int pick_groups(int ne, int M)
{
    // G in {1,2,...,32} (power of two, <= M) minimising rounds x nodes per task
    int best = 1;
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

} // namespace

cudaError_t launch_spectral_fp64(const OpacityLaunch& L, cudaStream_t stream, int num_sms)
{
    if (L.npts <= 0 || L.n_energies <= 0)
        return cudaSuccess;
    const int G = pick_groups(L.n_energies < kEChunk ? L.n_energies : kEChunk, 2 * L.n1);
    int blocks_per_sm = 0;
    cudaError_t err   = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &blocks_per_sm, spectral_fp64_kernel, kWarps * 32, 0);
    if (err != cudaSuccess)
        return err;
    if (blocks_per_sm < 1)
        blocks_per_sm = 1;
    const int64_t need = (L.npts + kWarps - 1) / kWarps;
    const int64_t cap  = (int64_t)num_sms * blocks_per_sm;
    phase_mark(kPhSpectral, 0, stream);
    spectral_fp64_kernel<<<(int)(need < cap ? need : cap), kWarps * 32, 0, stream>>>(L, G);
    phase_mark(kPhSpectral, 1, stream);
    return cudaGetLastError();
}

} // namespace bnsn
